"""Writes render_fixtures.npz: oracle renders (FP64 restatement of the
reference's Observation::run) of small planes of the benchmark jets, kept as
regression fixtures so that the oracle itself and the GPU's FP64 path are
checked against fixed numbers, not only against each other.

  * c0_full:  the conical jet (helical B, BK n, Gamma 10) on 16x16 pixels of
              0.8 mas at 15.4 GHz (1+z), full Stokes, the reference's default
              tolerances (tau 1e-7/1e-14, IQUV 1e-9/1e-9)
  * c2_full:  the ParabaloidCone jet with thermal electrons (Faraday
              rotation) on 8x8 pixels, 5 and 15.4 GHz, full Stokes
  * tangled_I: the model pyjetshow.get_i_image builds (s = 3.42, tangled B
              1/z, BK n in z, ConstCentral Gamma 8) on a 6x10 log plane, I only

Run from the repository root: python tests/golden/make_render_fixtures.py
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from jetshow_gb300 import jet as J  # noqa: E402
from jetshow_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402


def cases():
    jet, plane, nu, _ = W.conical_c0(scale=8)
    yield "c0_full", jet, plane, nu, J.make_params(output="full")
    jet, plane, nu, _ = W.parabolic_c2(scale=128)
    yield "c2_full", jet, plane, nu, J.make_params(output="full")
    jet = J.Jet(J.Cone((0., 0., 0.), (0., 0., 1.), 0.0165, 100), J.ConstCentralVField(8.0),
                J.RandomScalarBFieldZ(0.1, 1.0), J.BKNFieldZ(500, 2, True), s=3.42)
    lg0, lg1 = math.log10(1e-2 * 1.86 * J.pc), math.log10(1e-1 * 1.86 * J.pc)
    plane = J.ImagePlane((6, 10), lg0, lg1, 0.05)
    yield "tangled_I", jet, plane, np.array([15.4e9 * 1.1]), J.make_params(output="I", dt_max=J.pc * 0.001 * J.pc)


def main():
    O.build()
    out = {}
    for name, jet, plane, nu, params in cases():
        r = O.render(jet.desc(), plane.desc(), nu, params)
        for k in ("tau", "l", "I", "Q", "U", "V", "status"):
            out[f"{name}/{k}"] = r[k]
    np.savez_compressed(os.path.join(HERE, "render_fixtures.npz"), **out)
    print({k: v.shape for k, v in out.items() if k.endswith("/I")})


if __name__ == "__main__":
    main()
