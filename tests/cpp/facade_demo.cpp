// A reference-style caller of the C++ facade: builds the conical jet of the
// parity tests with the reference's class names, renders "I" and "full" on
// the GPU, writes the planes to a binary file (argv[1]) for comparison with
// the Python binding, renders the jet inside a SimulationGeometry hull, and
// checks the error paths throw.
#include <cmath>
#include <cstdio>
#include <stdexcept>

#include "jetshow.hpp"

using namespace jetshow;

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s out.bin\n", argv[0]);
    return 2;
  }
  const double pc = consts::pc;
  Vector3d origin = {0., 0., 0.};
  Vector3d direction = {0., 0., 1.};
  Cone geometry(origin, direction, 0.05, 100. * pc);
  HelicalConicalBField bfield(0.1, 1.0, M_PI / 4, true);
  BKNField nfield(500., 2., true);
  ConstFlatVField vfield(10.);
  Jet bkjet(&geometry, &vfield, &bfield, &nfield, 2.5, 10.0);
  const double lg = std::log10(0.4 * 1.8443 * pc);  // 0.4 mas pixels at z = 0.1
  ImagePlane imagePlane({32, 32}, lg, lg, 0.1);
  Observation observation(&bkjet, &imagePlane, 15.4e9 * 1.1);

  std::FILE* f = std::fopen(argv[1], "wb");
  if (!f) return 3;
  for (const char* out : {"I", "full"}) {
    observation.run(100, 1e4, 0.0, 1e-10, "adaptive", out);
    for (const char* v : {"tau", "I", "Q", "U", "V"}) {
      auto img = observation.getImage(v);
      for (auto& row : img) std::fwrite(row.data(), sizeof(double), row.size(), f);
    }
  }
  std::fclose(f);
  auto sz = observation.getImageSize();
  std::printf("image %lu x %lu, hit pixels %llu\n", sz.first, sz.second,
              (unsigned long long)observation.stats().n_hit_pixels);

  int thrown = 0;
  try {
    observation.run(100, 1e4, 0.0, 1e-10, "adaptive", "XYZ");
  } catch (const std::runtime_error&) {
    ++thrown;
  }
  try {
    ImagePlane odd({31, 32}, lg, lg, 0.1);  // n_across must be even
    Observation bad(&bkjet, &odd, 15.4e9);
    bad.run(100, 1e4, 0.0, 1e-10, "adaptive", "I");
  } catch (const std::runtime_error& e) {
    std::printf("error path: %s\n", e.what());
    ++thrown;
  }
  try {
    observation.getImage("W");
  } catch (const std::runtime_error&) {
    ++thrown;
  }
  try {
    SimulationGeometry flat({1.0, 0.1, 1.0, 0.2});  // one z: a flat hull
  } catch (const std::runtime_error&) {
    ++thrown;
  }
  // the conical jet bounded by the revolved hull of a (z, r) rectangle
  SimulationGeometry hull({0.0, 0.0, 0.0, 2.0, 40.0, 0.0, 40.0, 2.0});
  Jet hulljet(&hull, &vfield, &bfield, &nfield, 2.5, 10.0);
  Observation in_hull(&hulljet, &imagePlane, 15.4e9 * 1.1);
  in_hull.run(100, 1e4, 0.0, 1e-10, "adaptive", "I");
  std::printf("hull: hit pixels %llu\n", (unsigned long long)in_hull.stats().n_hit_pixels);
  std::printf("thrown %d\n", thrown);
  return thrown == 4 ? 0 : 1;
}
