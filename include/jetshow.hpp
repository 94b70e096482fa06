/* jetshow.hpp -- C++ facade of the GB300 renderer with the reference's class
 * names and constructor signatures (header-only, forwards to the C ABI of
 * jetshow_capi.h; link with -ljetshow_gb300).
 *
 * Reference classes and where their signatures come from:
 *   Cone, Cylinder, Parabaloid, ParabaloidCone   include/Cone.h:14-15,
 *       include/Cylinder.h:14-15, include/Parabaloid.h:18-19,
 *       include/ParabaloidCone.h:19-20
 *   B fields   include/BField.h:36-208   (ScalarBField / VectorBField)
 *   N fields   include/NField.h:10-69
 *   V fields   include/VField.h:11-185
 *   Jet        include/Jet.h:16 (plus the commented VectorBField overload, :14)
 *   ImagePlane include/ImagePlane.h:22-23
 *   Observation include/Observation.h:14-23 (run, getImage, getImageSize)
 *
 * Differences a caller sees: the classes are descriptors (no virtual
 * bf/nf/vf evaluation on the host); Simulation*Field take the id of a grid
 * uploaded with SimulationGrid instead of a CGAL triangulation; Observation
 * takes one or several frequencies and `output_type` "full" integrates IQUV;
 * every failing call throws std::runtime_error with jsh_last_error().
 */
#ifndef JETSHOW_HPP
#define JETSHOW_HPP

#include <array>
#include <cstring>
#include <memory>
#include <mutex>
#include <ostream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "jetshow_capi.h"

namespace jetshow {

struct Vector3d {
  double x = 0, y = 0, z = 0;
  Vector3d() = default;
  Vector3d(double x_, double y_, double z_) : x(x_), y(y_), z(z_) {}
};

namespace consts {  // include/utils.h:17-36
constexpr double pc = 3.0856775814671913e+18;
constexpr double mas_to_rad = 4.84813681109536e-09;
constexpr double c = 29979245800.0;
}  // namespace consts

inline void check(int status) {
  if (status != JSH_OK) throw std::runtime_error(jsh_last_error());
}

// Process-wide context on device 0, created on first use.
inline jsh_ctx* default_context() {
  static std::once_flag once;
  static std::shared_ptr<jsh_ctx> ctx;
  std::call_once(once, [] {
    jsh_ctx* c = nullptr;
    check(jsh_ctx_create(0, 0, &c));
    ctx.reset(c, jsh_ctx_destroy);
  });
  return ctx.get();
}

// ------------------------------------------------------------- geometry
class BaseGeometry {
 public:
  virtual ~BaseGeometry() = default;
  const jsh_geometry_desc& desc() const { return d_; }

 protected:
  BaseGeometry(int kind, const Vector3d& o, const Vector3d& dir) {
    std::memset(&d_, 0, sizeof(d_));
    d_.kind = kind;
    d_.origin[0] = o.x, d_.origin[1] = o.y, d_.origin[2] = o.z;
    d_.direction[0] = dir.x, d_.direction[1] = dir.y, d_.direction[2] = dir.z;
  }
  jsh_geometry_desc d_;
};
using Geometry = BaseGeometry;

class Cone : public BaseGeometry {
 public:
  Cone(const Vector3d& origin, const Vector3d& direction, const double& angle, const double& scale)
      : BaseGeometry(JSH_GEO_CONE, origin, direction) {
    d_.angle = angle;
    d_.big_scale = scale;
  }
};

class Cylinder : public BaseGeometry {
 public:
  Cylinder(const Vector3d& origin, const Vector3d& direction, const double& r)
      : BaseGeometry(JSH_GEO_CYLINDER, origin, direction) {
    d_.r = r;
    d_.big_scale = 100. * r;  // src/Cylinder.cpp:97-99
  }
};

class Parabaloid : public BaseGeometry {
 public:
  Parabaloid(const Vector3d& origin, const Vector3d& direction, const double& r0, const double& big_scale)
      : BaseGeometry(JSH_GEO_PARABALOID, origin, direction) {
    d_.r0 = r0;
    d_.big_scale = big_scale;
  }
};

class ParabaloidCone : public BaseGeometry {
 public:
  ParabaloidCone(const Vector3d& origin, const Vector3d& direction, const double& r0, const double& z0,
                 const double& scale)
      : BaseGeometry(JSH_GEO_PARABALOID_CONE, origin, direction) {
    d_.r0 = r0;
    d_.z0 = z0;
    d_.big_scale = scale;
  }
};

// SimulationGeometry(tree) (include/Geometry.h:58-65, src/Geometry.cpp:92-132):
// the reference passes an AABB tree over CGAL::convex_hull_3 of the grid
// points revolved at 36 azimuths (src/main.cpp:880-897); here the hull is
// built from the (z, r) points [pc] and uploaded by this constructor.
class SimulationGeometry : public BaseGeometry {
 public:
  SimulationGeometry(const std::vector<double>& zr, int n_circle = 36, jsh_ctx* ctx = default_context())
      : BaseGeometry(JSH_GEO_SIMULATION, Vector3d(), Vector3d(0, 0, 1)) {
    int32_t id = 0;
    check(jsh_hull_upload(ctx, zr.data(), (int64_t)(zr.size() / 2), n_circle, &id));
    d_.hull_id = id;
  }
};

// --------------------------------------------------------------- fields
class Field {
 public:
  virtual ~Field() = default;
  const jsh_field_desc& desc() const { return d_; }

 protected:
  Field(int kind, std::initializer_list<double> p, bool in_plasma_frame = true) {
    std::memset(&d_, 0, sizeof(d_));
    d_.kind = kind;
    d_.in_plasma_frame = in_plasma_frame ? 1 : 0;
    int i = 0;
    for (double v : p) d_.p[i++] = v;
  }
  jsh_field_desc d_;
};

class ScalarBField : public Field {
 protected:
  using Field::Field;
};
class VectorBField : public Field {
 protected:
  using Field::Field;
};
// Random directions added to a vector field: RandomVectorBField and its
// kinds (src/BField.cpp:149-193).  The wrapper's field is taken in the
// plasma frame, as the reference's VectorBField(true) base makes it.
class RandomVectorBField : public VectorBField {
 public:
  const jsh_random_desc& random() const { return r_; }

 protected:
  RandomVectorBField(VectorBField* bfield, double rnd_fraction, int kind) : VectorBField(*bfield) {
    std::memset(&r_, 0, sizeof(r_));
    r_.kind = kind;
    r_.fraction = rnd_fraction;
  }
  jsh_random_desc r_;
};

// RandomCellsInSphere(N, n_exponent, seed) (src/Cells.cpp:24-47): N cells
// drawn on the host by the counter-based generator (jsh_cells_generate),
// uploaded by create().
class RandomCellsInSphere {
 public:
  RandomCellsInSphere(int N, double n_exponent, unsigned int seed = 0) : n_(N), exponent_(n_exponent), seed_(seed) {}
  void setGeometry(double coord1_max, double coord2_max, double coord1_min = 0., double coord2_min = 0.) {
    r_max_ = coord1_max, theta_max_ = coord2_max, r_min_ = coord1_min, theta_min_ = coord2_min;
  }
  void create(jsh_ctx* ctx = default_context()) {
    points_.assign(3 * (size_t)n_, 0.0);
    directions_.assign(3 * (size_t)n_, 0.0);
    check(jsh_cells_generate(n_, r_min_, r_max_, theta_max_, exponent_, seed_, points_.data(), directions_.data()));
    check(jsh_cells_upload(ctx, points_.data(), directions_.data(), n_, &id_));
  }
  const std::vector<double>& getCells() const { return points_; }
  int32_t id() const { return id_; }

 private:
  int n_;
  double exponent_;
  unsigned int seed_;
  double r_max_ = 0, theta_max_ = 0, r_min_ = 0, theta_min_ = 0;
  std::vector<double> points_, directions_;
  int32_t id_ = -1;
};

// CellsRandomVectorBField(cells, bfield, rnd_fraction) (src/BField.cpp:164-172).
class CellsRandomVectorBField : public RandomVectorBField {
 public:
  CellsRandomVectorBField(RandomCellsInSphere* cells, VectorBField* bfield, double rnd_fraction)
      : RandomVectorBField(bfield, rnd_fraction, JSH_RND_CELLS) {
    if (!cells || cells->id() < 0) throw std::runtime_error("CellsRandomVectorBField: create() the cells first");
    r_.cells_id = cells->id();
  }
};

// PointsRandomVectorBField(bfield, rnd_fraction, seed) (src/BField.cpp:175-193):
// a fresh direction at every evaluation, keyed by (seed, pixel, frequency,
// evaluation index) instead of per-thread generators.
class PointsRandomVectorBField : public RandomVectorBField {
 public:
  PointsRandomVectorBField(VectorBField* bfield, double rnd_fraction, unsigned int seed)
      : RandomVectorBField(bfield, rnd_fraction, JSH_RND_POINTS) {
    r_.seed = seed;
  }
};

class NField : public Field {
 protected:
  using Field::Field;
};
class VField : public Field {
 protected:
  using Field::Field;
};

#define JETSHOW_FIELD2(Base, Name, KIND, A1, A2) \
  class Name : public Base {                      \
   public:                                        \
    Name(double A1, double A2) : Base(KIND, {A1, A2}) {} \
  };
#define JETSHOW_FIELD2P(Base, Name, KIND, A1, A2)                                            \
  class Name : public Base {                                                                  \
   public:                                                                                    \
    Name(double A1, double A2, bool in_plasma_frame) : Base(KIND, {A1, A2}, in_plasma_frame) {} \
  };

JETSHOW_FIELD2(ScalarBField, RandomScalarBField, JSH_B_RANDOM_SCALAR, b_0, m_b)
JETSHOW_FIELD2(ScalarBField, RandomScalarBFieldZ, JSH_B_RANDOM_SCALAR_Z, b_0, m_b)
class CompositeRandomScalarBFieldZ : public ScalarBField {
 public:
  CompositeRandomScalarBFieldZ(double b_0, double m_b_inner, double m_b_outer, double z0)
      : ScalarBField(JSH_B_COMPOSITE_RANDOM_SCALAR_Z, {b_0, m_b_inner, m_b_outer, z0}) {}
};
JETSHOW_FIELD2P(VectorBField, ConstCylinderBField, JSH_B_CONST_CYLINDER, b_0, n_b)
JETSHOW_FIELD2P(VectorBField, ConstCylinderBFieldZ, JSH_B_CONST_CYLINDER_Z, b_0, n_b)
JETSHOW_FIELD2P(VectorBField, RadialConicalBField, JSH_B_RADIAL_CONICAL, b_0, n_b)
JETSHOW_FIELD2P(VectorBField, ToroidalBField, JSH_B_TOROIDAL, b_0, n_b)
JETSHOW_FIELD2P(VectorBField, HelicalCylinderBField, JSH_B_HELICAL_CYLINDER, b_0, pitch_angle)
JETSHOW_FIELD2P(VectorBField, SpiralConicalBField, JSH_B_SPIRAL_CONICAL, b_0, pitch_angle)
JETSHOW_FIELD2P(VectorBField, ForceFreeCylindricalBField, JSH_B_FORCE_FREE_CYLINDRICAL, b_0, mu)
// Builder-defined: b_0 (|x|/pc)^-n_b (sin(pitch) phi_hat + cos(pitch) z_hat).
class HelicalConicalBField : public VectorBField {
 public:
  HelicalConicalBField(double b_0, double n_b, double pitch_angle, bool in_plasma_frame = true,
                       bool atan_quirk = false)
      : VectorBField(JSH_B_HELICAL_CONICAL, {b_0, n_b, pitch_angle, atan_quirk ? 1.0 : 0.0}, in_plasma_frame) {}
};
// Fields of an uploaded grid: B_p = field_p, B_phi = field_phi.
class SimulationBField : public VectorBField {
 public:
  SimulationBField(int grid_id, int field_p, int field_phi, bool in_plasma_frame)
      : VectorBField(JSH_B_SIMULATION, {(double)grid_id, (double)field_p, (double)field_phi}, in_plasma_frame) {}
};

class ConstNField : public NField {
 public:
  ConstNField(double n, bool in_plasma_frame) : NField(JSH_N_CONST, {n}, in_plasma_frame) {}
};
JETSHOW_FIELD2P(NField, BKNField, JSH_N_BK, n_0, n_n)
JETSHOW_FIELD2P(NField, BKNFieldZ, JSH_N_BKZ, n_0, n_n)
class CompositeBKNField : public NField {
 public:
  CompositeBKNField(double n_0, double n_n_inner, double n_n_outer, double z0, bool in_plasma_frame)
      : NField(JSH_N_COMPOSITE_BK, {n_0, n_n_inner, n_n_outer, z0}, in_plasma_frame) {}
};
class SimulationNField : public NField {
 public:
  SimulationNField(int grid_id, int field, bool in_plasma_frame)
      : NField(JSH_N_SIMULATION, {(double)grid_id, (double)field}, in_plasma_frame) {}
};

class ConstFlatVField : public VField {
 public:
  explicit ConstFlatVField(double gamma) : VField(JSH_V_CONST_FLAT, {gamma}) {}
};
class ShearedFlatVField : public VField {
 public:
  ShearedFlatVField(double gamma_axis, double gamma_border, double r)
      : VField(JSH_V_SHEARED_FLAT, {gamma_axis, gamma_border, r}) {}
};
class SheathFlatVField : public VField {
 public:
  SheathFlatVField(double gamma_spine, double gamma_sheath, double r_sheath)
      : VField(JSH_V_SHEATH_FLAT, {gamma_spine, gamma_sheath, r_sheath}) {}
};
class ConstCentralVField : public VField {
 public:
  explicit ConstCentralVField(double gamma, Vector3d origin = {0, 0, 0})
      : VField(JSH_V_CONST_CENTRAL, {gamma, origin.x, origin.y, origin.z}) {}
};
class ShearedCentralVField : public VField {
 public:
  ShearedCentralVField(double gamma_axis, double gamma_border, double theta, Vector3d origin = {0, 0, 0})
      : VField(JSH_V_SHEARED_CENTRAL, {gamma_axis, gamma_border, theta, origin.x, origin.y, origin.z}) {}
};
class SheathCentralVField : public VField {
 public:
  SheathCentralVField(double gamma_spine, double gamma_sheath, double theta_sheath, Vector3d origin = {0, 0, 0})
      : VField(JSH_V_SHEATH_CENTRAL, {gamma_spine, gamma_sheath, theta_sheath, origin.x, origin.y, origin.z}) {}
};
class ConstParabolicVField : public VField {
 public:
  ConstParabolicVField(double gamma, double Rz0) : VField(JSH_V_CONST_PARABOLIC, {gamma, Rz0}) {}
};
class AccParabolicVField : public VField {
 public:
  AccParabolicVField(double gamma0, double R0, double Rz0) : VField(JSH_V_ACC_PARABOLIC, {gamma0, R0, Rz0}) {}
};
class ShearedAccParabolicVField : public VField {
 public:
  ShearedAccParabolicVField(double gamma_axis0, double gamma_border0, double R0, double Rz0)
      : VField(JSH_V_SHEARED_ACC_PARABOLIC, {gamma_axis0, gamma_border0, R0, Rz0}) {}
};
class AccParabolicConstConeVField : public VField {
 public:
  AccParabolicConstConeVField(double gamma0, double Rz0, double z0)
      : VField(JSH_V_ACC_PARABOLIC_CONST_CONE, {gamma0, Rz0, z0}) {}
};
class ShearedAccParabolicConstConeVField : public VField {
 public:
  ShearedAccParabolicConstConeVField(double gamma_axis0, double gamma_border0, double Rz0, double z0)
      : VField(JSH_V_SHEARED_ACC_PARABOLIC_CONST_CONE, {gamma_axis0, gamma_border0, Rz0, z0}) {}
};
class SimulationVField : public VField {
 public:
  SimulationVField(int grid_id, int field) : VField(JSH_V_SIMULATION, {(double)grid_id, (double)field}) {}
};

#undef JETSHOW_FIELD2
#undef JETSHOW_FIELD2P

// A (z, r) simulation grid [pc] triangulated on the host and uploaded once
// (create_triangulation + SimulationInterpolater, src/SimulationInterpolater.cpp:30-117).
class SimulationGrid {
 public:
  // zr: n points (z, r); values: n x n_fields, row-major FP32
  SimulationGrid(const std::vector<double>& zr, const std::vector<float>& values, int n_fields,
                 jsh_ctx* ctx = default_context()) {
    const int64_t n = (int64_t)(zr.size() / 2);
    if (n_fields < 1 || values.size() != (size_t)n * (size_t)n_fields)
      throw std::runtime_error("SimulationGrid: values must be n_points x n_fields");
    std::vector<int32_t> tri((size_t)(6 * n));
    int64_t n_tri = 0;
    check(jsh_grid_triangulate(zr.data(), n, tri.data(), &n_tri));
    check(jsh_grid_upload(ctx, zr.data(), n, values.data(), n_fields, tri.data(), n_tri, &id_));
    ctx_ = ctx;
    n_tri_ = n_tri;
  }
  int id() const { return id_; }
  int64_t n_triangles() const { return n_tri_; }
  // interpolated_value (src/SimulationInterpolater.cpp:43-102) at (z, r) [pc]
  std::vector<double> interpolated_values(int field, const std::vector<double>& zr, double nan_value) const {
    std::vector<double> out(zr.size() / 2);
    check(jsh_grid_interpolate(ctx_, id_, field, zr.data(), (int64_t)out.size(), nan_value, out.data()));
    return out;
  }

 private:
  jsh_ctx* ctx_ = nullptr;
  int32_t id_ = -1;
  int64_t n_tri_ = 0;
};

// ------------------------------------------------------------------ Jet
class Jet {
 public:
  // s: power-law index (the reference hard-codes 3.42, src/Jet.cpp:32);
  // gamma_min enters k_F_r, k_C_r; thermal_fraction adds cold-plasma
  // Faraday terms of n_th = fraction * n.
  Jet(BaseGeometry* geo, VField* vfield, ScalarBField* bField, NField* nField, double s = 3.42,
      double gamma_min = 100.0, double thermal_fraction = 0.0) {
    init(geo, vfield, bField, nField, s, gamma_min, thermal_fraction);
  }
  Jet(BaseGeometry* geo, VField* vfield, VectorBField* bField, NField* nField, double s = 3.42,
      double gamma_min = 100.0, double thermal_fraction = 0.0) {
    init(geo, vfield, bField, nField, s, gamma_min, thermal_fraction);
  }
  const jsh_model_desc& desc() const { return d_; }

 private:
  void init(BaseGeometry* geo, VField* v, Field* b, NField* n, double s, double gmin, double fth) {
    if (!geo || !v || !b || !n) throw std::runtime_error("Jet: null geometry or field");
    std::memset(&d_, 0, sizeof(d_));
    d_.geometry = geo->desc();
    d_.vfield = v->desc();
    d_.bfield = b->desc();
    if (auto* rb = dynamic_cast<RandomVectorBField*>(b)) d_.random = rb->random();
    d_.nfield = n->desc();
    d_.s = s;
    d_.gamma_min = gmin;
    d_.thermal_fraction = fth;
  }
  jsh_model_desc d_;
};

// ------------------------------------------------------------ ImagePlane
class ImagePlane {
 public:
  ImagePlane(std::pair<unsigned long int, unsigned long int> image_size, double lg_pixel_size_start,
             double lg_pixel_size_stop, double los_angle) {
    d_.n_across = image_size.first;
    d_.n_along = image_size.second;
    d_.lg_pixel_size_start_cm = lg_pixel_size_start;
    d_.lg_pixel_size_stop_cm = lg_pixel_size_stop;
    d_.los_angle = los_angle;
  }
  const jsh_plane_desc& desc() const { return d_; }
  std::pair<unsigned long int, unsigned long int> image_size() const {
    return {(unsigned long)d_.n_across, (unsigned long)d_.n_along};
  }

 private:
  jsh_plane_desc d_{};
};

// ----------------------------------------------------------- Observation
class Observation {
 public:
  Observation(Jet* newjet, ImagePlane* imagePlane, double nu) : Observation(newjet, imagePlane, std::vector<double>{nu}) {}
  Observation(Jet* newjet, ImagePlane* imagePlane, std::vector<double> nu_list)
      : nu(nu_list.empty() ? 0.0 : nu_list[0]), jet_(newjet), plane_(imagePlane), nus_(std::move(nu_list)) {
    if (!jet_ || !plane_ || nus_.empty()) throw std::runtime_error("Observation: null jet/plane or no frequency");
    jsh_params_default(&params_);
  }

  // src/Observation.cpp:20-41; dt_max in pc as there.  integration_type,
  // n_max, tau_n_min and tau_n_max are accepted and unused, as in the
  // reference's adaptive path.
  void run(int n, double tau_max, double dt_max, double tau_min, std::string integration_type,
           std::string output_type, int n_max = 0, double tau_n_min = 0.1, double tau_n_max = 100.0) {
    (void)integration_type, (void)n_max, (void)tau_n_min, (void)tau_n_max;
    if (output_type != "I" && output_type != "full") throw std::runtime_error("output_type must be \"I\" or \"full\"");
    params_.n = n;
    params_.tau_max = tau_max;
    params_.dt_max = dt_max * consts::pc;
    params_.tau_min = tau_min;
    params_.output = output_type == "full" ? JSH_OUT_FULL : JSH_OUT_I;
    render();
  }

  // The GB300 choices: precision (JSH_PREC_FP64 / JSH_PREC_MIXED), schedule
  // and tolerances; taking effect at the next run().
  jsh_params& params() { return params_; }

  std::vector<std::vector<double>> getImage(std::string value, size_t freq_index = 0) const {
    const std::vector<double>* src = nullptr;
    if (value == "tau") src = &tau_;
    else if (value == "l") src = &l_;
    else if (value == "I") src = &I_;
    else if (value == "Q") src = &Q_;
    else if (value == "U") src = &U_;
    else if (value == "V") src = &V_;
    else throw std::runtime_error("getImage: unknown value " + value);
    if (src->empty()) throw std::runtime_error("getImage: run() first");
    if (freq_index >= nus_.size()) throw std::runtime_error("getImage: frequency index out of range");
    const auto sz = plane_->image_size();
    std::vector<std::vector<double>> img(sz.first, std::vector<double>(sz.second));
    const size_t off = freq_index * sz.first * sz.second;
    for (size_t i = 0; i < sz.first; ++i)
      for (size_t j = 0; j < sz.second; ++j) img[i][j] = (*src)[off + i * sz.second + j];
    return img;
  }
  // Observation::run_stripe (src/Observation.cpp:310-347): tau only, along
  // half of the central row, n constant RK4 steps per intersection, stop at
  // tau_max; tau_min is accepted and unused, as in the reference.
  void run_stripe(int n, double tau_max, double tau_min, size_t freq_index = 0) {
    (void)tau_min;
    if (freq_index >= nus_.size()) throw std::runtime_error("run_stripe: frequency index out of range");
    const auto sz = plane_->image_size();
    stripe_.assign(sz.second - sz.second / 2, 0.0);
    check(jsh_observation_run_stripe(default_context(), &jet_->desc(), &plane_->desc(), nus_[freq_index], n,
                                     tau_max, stripe_.data()));
  }
  // Image::getStripe (src/Image.cpp:31-41); stripe mode computes tau only.
  std::vector<double> getStripe(std::string value) const {
    if (value != "tau") throw std::runtime_error("getStripe: stripe mode computes tau only");
    if (stripe_.empty()) throw std::runtime_error("getStripe: run_stripe() first");
    return stripe_;
  }
  std::pair<unsigned long int, unsigned long int> getImageSize() const { return plane_->image_size(); }
  const jsh_stats& stats() const { return stats_; }
  const std::vector<uint32_t>& status() const { return status_; }

  const double nu;

 private:
  void render() {
    const auto sz = plane_->image_size();
    const size_t m = sz.first * sz.second * nus_.size();
    for (auto* v : {&tau_, &l_, &I_, &Q_, &U_, &V_}) v->assign(m, 0.0);
    status_.assign(m, 0u);
    jsh_image img{tau_.data(), l_.data(), I_.data(), Q_.data(), U_.data(), V_.data(), status_.data()};
    check(jsh_observation_run(default_context(), &jet_->desc(), &plane_->desc(), nus_.data(), (int32_t)nus_.size(),
                              &params_, &img, &stats_));
  }
  Jet* jet_;
  ImagePlane* plane_;
  std::vector<double> nus_;
  jsh_params params_{};
  jsh_stats stats_{};
  std::vector<double> tau_, l_, I_, Q_, U_, V_, stripe_;
  std::vector<uint32_t> status_;
};

// Text writers of the legacy drivers (src/utils.cpp:211-236): every value
// divided by `scale`, separated by a space, one image row per line
// (write_2dvector) or one value per line (write_vector), default ostream
// formatting.
inline std::ostream& write_2dvector(std::ostream& os, const std::vector<std::vector<double>>& v,
                                    double scale = 1.0) {
  for (const auto& row : v) {
    for (double x : row) os << x / scale << " ";
    os << "\n";
  }
  return os;
}

inline std::ostream& write_vector(std::ostream& os, const std::vector<double>& v, double scale = 1.0) {
  for (double x : v) os << x / scale << " " << "\n";
  return os;
}

}  // namespace jetshow

#endif  // JETSHOW_HPP
