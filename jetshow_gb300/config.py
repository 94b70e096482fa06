"""Driver of jetshow's legacy config.json pipeline: the config-driven
observation of src/main.cpp:69-225 (commented out in the reference, which
reads the file with boost::property_tree), restated over the GPU renderer.

Keys read (the reference file's layout):
  observation.{redshift, frequency_ghz, los_angle}
  jet.geometry: type "cone" with parameters {angle, scale_pc}
  jet.bfield: type "radial_conical" {b_1, n_b} or "spiral_conical"
              {b_1, pitch_angle}, plus random_fraction (> 0 wraps the field
              in PointsRandomVectorBField(bfield, random_fraction, 123) as
              the driver does, src/main.cpp:119-126; its per-evaluation
              directions come from the counter-based stream)
  jet.vfield: type "const_central" {gamma};  jet.nfield: type "bk" {n_1, n_n}
  image.{pixel_size_mas, number_of_pixels}
  integration.parameters.{n, tau_max, dl_max_pc, log10_tau_min, tau_n_min,
              n_tau_max, log10_abs_error_tau, log10_rel_error_tau,
              log10_abs_error_I, log10_rel_error_I}
  output.{file_tau, file_i, file_length, file_q, file_u, file_v}
  calculate: "I" or "full"

As in the driver: the pixel is pixel_size_mas * 0.25 * (pc per mas) pc on
a side, the frequency is redshifted to the source frame, maps are appended
to their files by write_2dvector, Stokes maps in Jy (divided by 1e-23 /
(pixel_size_mas * mas_to_rad)^2, src/utils.cpp:239-245) and lengths in pc.
Builder choices where the reference API has moved on since the driver: the
field classes' in_plasma_frame flag (absent in the driver's constructors) is
True, the config's tolerances are passed to the integrator (the driver
left the hard-coded ones), and the tau-pass step limit is dl_max_pc * pc cm:
the driver handed dt_max = pc * dl_max_pc to Observation::run, which
multiplies by pc once more (src/Observation.cpp:23), so its limit was
pc^2 * dl_max_pc cm -- in effect none.  Map files of configs whose
dl_max_pc binds can therefore differ from the legacy driver's.
"""
from __future__ import annotations

import json
import math
import os

from . import jet as J
from .runtime import default_context, mas_to_pc
from .textio import write_2dvector


def load(cfg) -> dict:
    """A config dict, from a dict, a JSON string or a path."""
    if isinstance(cfg, dict):
        return cfg
    if isinstance(cfg, str) and cfg.lstrip().startswith("{"):
        return json.loads(cfg)
    with open(cfg) as fh:
        return json.load(fh)


def build(cfg) -> dict:
    """Model, plane, frequency, run arguments and output files of a config
    (no device work)."""
    c = load(cfg)
    ob, jt, im, it = c["observation"], c["jet"], c["image"], c["integration"]["parameters"]
    z, los = float(ob["redshift"]), float(ob["los_angle"])
    geo = jt["geometry"]
    if geo["type"] != "cone":
        raise ValueError(f"geometry type {geo['type']!r} is not one the config driver knows (cone)")
    g = geo["parameters"]
    geometry = J.Cone((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), float(g["angle"]), float(g["scale_pc"]) * J.pc)
    b = jt["bfield"]
    bp = b["parameters"]
    if b["type"] == "radial_conical":
        bfield = J.RadialConicalBField(float(bp["b_1"]), float(bp["n_b"]), True)
    elif b["type"] == "spiral_conical":
        bfield = J.SpiralConicalBField(float(bp["b_1"]), float(bp["pitch_angle"]), True)
    else:
        raise ValueError(f"bfield type {b['type']!r} is not one the config driver knows")
    rnd = float(bp.get("random_fraction", 0.0))
    if rnd > 0.0:
        # as the driver: PointsRandomVectorBField(bfield, rnd_fraction, 123)
        bfield = J.PointsRandomVectorBField(bfield, rnd, seed=123)
    v = jt["vfield"]
    if v["type"] != "const_central":
        raise ValueError(f"vfield type {v['type']!r} is not one the config driver knows (const_central)")
    vfield = J.ConstCentralVField(float(v["parameters"]["gamma"]))
    n = jt["nfield"]
    if n["type"] != "bk":
        raise ValueError(f"nfield type {n['type']!r} is not one the config driver knows (bk)")
    nfield = J.BKNField(float(n["parameters"]["n_1"]), float(n["parameters"]["n_n"]), True)
    jet = J.Jet(geometry, vfield, bfield, nfield)
    npix = int(im["number_of_pixels"])
    size_mas = float(im["pixel_size_mas"])
    pixel_size_cm = size_mas * 0.25 * mas_to_pc(z) * J.pc
    lg = math.log10(pixel_size_cm)
    plane = J.ImagePlane((npix, npix), lg, lg, los)
    nu = float(ob["frequency_ghz"]) * 1e9 * (1.0 + z)
    output = c.get("calculate", "I")
    if output not in ("I", "full"):
        raise ValueError("calculate must be \"I\" or \"full\"")
    run = dict(n=int(it["n"]), tau_max=float(it["tau_max"]), dt_max=float(it["dl_max_pc"]),
               tau_min=10.0 ** float(it["log10_tau_min"]), integration_type=c["integration"].get("step_type",
                                                                                                "adaptive"),
               output_type=output, n_max=int(it.get("n_tau_max", 0)), tau_n_min=float(it.get("tau_n_min", 0.1)),
               tau_atol=10.0 ** float(it["log10_abs_error_tau"]), tau_rtol=10.0 ** float(it["log10_rel_error_tau"]),
               atol=10.0 ** float(it["log10_abs_error_I"]), rtol=10.0 ** float(it["log10_rel_error_I"]))
    jy = 1e-23 / (size_mas * size_mas * J.mas_to_rad * J.mas_to_rad)
    files = c.get("output", {})
    maps = [("tau", files.get("file_tau"), 1.0), ("I", files.get("file_i"), jy), ("l", files.get("file_length"), J.pc)]
    if output == "full":
        maps += [("Q", files.get("file_q"), jy), ("U", files.get("file_u"), jy), ("V", files.get("file_v"), jy)]
    return {"jet": jet, "plane": plane, "nu": nu, "run": run, "maps": [m for m in maps if m[1]]}


def run_config(cfg, out_dir: str = ".", ctx=None) -> dict:
    """Render a config on the GPU and append its maps to the output files
    (relative to out_dir); returns the rendered planes by name."""
    b = build(cfg)
    obs = J.Observation(b["jet"], b["plane"], b["nu"]).run(ctx=ctx or default_context(), **b["run"])
    images = {}
    for value, fname, scale in b["maps"]:
        img = obs.getImage(value)
        images[value] = img
        with open(os.path.join(out_dir, fname), "a") as fh:
            write_2dvector(fh, img, scale)
    return images
