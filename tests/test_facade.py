"""C++ facade (include/jetshow.hpp): a reference-style caller compiles and
links against the library on the CPU; on the GPU its images are bitwise
those of the Python binding with the same descriptors and parameters, and
its error paths throw."""
import math
import os
import subprocess

import numpy as np
import pytest

from jetshow_gb300 import jet as J

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "cpp", "facade_demo.cpp")


def build_demo(out_dir):
    from jetshow_gb300 import build
    exe = os.path.join(out_dir, "facade_demo")
    libdir = os.path.dirname(build.LIB)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(REPO, "include"),
                    SRC, "-L", libdir, "-ljetshow_gb300", "-Wl,-rpath," + libdir, "-o", exe], check=True)
    return exe


def test_facade_compiles_and_links(lib, tmp_path):
    exe = build_demo(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_facade_matches_python_binding(lib, ctx, tmp_path):
    exe = build_demo(str(tmp_path))
    out = tmp_path / "planes.bin"
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "thrown 4" in r.stdout
    assert "hull: hit pixels 0" not in r.stdout
    got = np.fromfile(out, dtype=np.float64).reshape(2, 5, 32, 32)
    jet = J.Jet(J.Cone((0., 0., 0.), (0., 0., 1.), 0.05, 100. * J.pc), J.ConstFlatVField(10.),
                J.HelicalConicalBField(0.1, 1.0, math.pi / 4, True), J.BKNField(500., 2., True), s=2.5,
                gamma_min=10.0)
    lg = math.log10(0.4 * 1.8443 * J.pc)
    plane = J.ImagePlane((32, 32), lg, lg, 0.1)
    for k, output in enumerate(("I", "full")):
        img, st = ctx.render(jet.desc(), plane.desc(), [15.4e9 * 1.1], J.make_params(output=output))
        assert st["n_hit_pixels"] > 0
        for j, v in enumerate(("tau", "I", "Q", "U", "V")):
            assert np.array_equal(got[k, j], img[v][0]), (output, v)
