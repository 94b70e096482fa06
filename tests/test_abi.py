"""The C-ABI library builds, loads without a GPU and exports every entry
point declared in include/jetshow_capi.h; host-only entry points work."""
import ctypes as C
import os
import re

import numpy as np

from jetshow_gb300 import _capi as A

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(REPO, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(REPO, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(jsh_[a-z0-9_]+)\s*\(", txt))
    return names


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert {s[0] for s in A.SIGNATURES} >= names


def test_struct_sizes_match_header(lib):
    # the header's structs as laid out by ctypes (x86-64 / aarch64 LP64)
    assert C.sizeof(A.GeometryDesc) == 8 + 8 * 11
    assert C.sizeof(A.FieldDesc) == 8 + 64
    assert C.sizeof(A.Params) == 16 + 8 * 8 + 8 + 16


def test_params_default(lib):
    p = A.Params()
    lib.jsh_params_default(C.byref(p))
    assert p.n == 100 and p.tau_max == 1e4 and p.tau_min == 1e-10
    assert p.tau_atol == 1e-7 and p.tau_rtol == 1e-14 and p.atol == 1e-9 and p.rtol == 1e-9


def test_mas_to_pc_matches_oracle(lib, oracle):
    flat = A.Cosmology(H0=70.0, omega_M=0.3, omega_V=0.7, gamma_nu=0.0)
    for z in (0.01, 0.1, 0.5, 2.0):
        a = lib.jsh_mas_to_pc(z, C.byref(flat))
        b = oracle.mas_to_pc(z, flat)
        assert abs(a - b) <= 1e-12 * b, (z, a, b)
        assert abs(lib.jsh_mas_to_pc(z, None) - oracle.mas_to_pc(z)) <= 1e-12 * b


def test_ctx_create_without_gpu_fails_cleanly(lib):
    import ctypes
    h = ctypes.c_void_p()
    st = lib.jsh_ctx_create(0, 0, ctypes.byref(h))
    if st == 0:  # running on a GPU machine
        lib.jsh_ctx_destroy(h)
    else:
        assert st in (A.JSH_ERR_NO_DEVICE, A.JSH_ERR_CUDA)
        assert lib.jsh_last_error()


def test_request_h2d_bytes(lib):
    # the request record plus 8 bytes per frequency, plus the FP32
    # constants (56 bytes per frequency) for mixed precision
    b1 = lib.jsh_request_h2d_bytes(1, A.PREC_FP64)
    assert lib.jsh_request_h2d_bytes(4, A.PREC_FP64) == b1 + 3 * 8
    assert lib.jsh_request_h2d_bytes(4, A.PREC_MIXED) == b1 + 3 * 8 + 4 * 56
    assert 1024 < b1 < 4096


def test_tau_panel_rule_is_gauss_kronrod(lib):
    """The tau pass's panel rule: the 15-point Kronrod rule integrates
    monomials of degree <= 22 exactly on [-1, 1], its embedded 7-point Gauss
    rule those of degree <= 13 and equals the Gauss-Legendre rule."""
    import ctypes as C
    x, wk, wg = (np.zeros(15) for _ in range(3))
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    lib.jsh_tau_panel_rule(p(x), p(wk), p(wg))
    assert np.all(np.diff(x) > 0) and np.allclose(x, -x[::-1], rtol=0, atol=1e-16)
    for k in range(23):
        exact = (1 - (-1) ** (k + 1)) / (k + 1)
        assert abs((wk * x ** k).sum() - exact) < 1e-14, k
        if k < 14:
            assert abs((wg * x ** k).sum() - exact) < 1e-14, k
    assert abs((wk * x ** 24).sum() - 2 / 25) > 1e-10  # not exact beyond degree 22
    gx, gw = np.polynomial.legendre.leggauss(7)
    assert np.allclose(x[1::2], gx, rtol=0, atol=1e-15) and np.allclose(wg[1::2], gw, rtol=0, atol=1e-15)
    assert np.all(wg[0::2] == 0)


def test_faraday_thick_build_is_linked_and_uncontracted(lib):
    """The Faraday-thick mode's kernels are jsh_persistent.cu compiled a
    second time (jsh_persistent_ft.cu): that unit is built, like its twin,
    without compiler-fused multiply-adds (every form of the mixed path gives
    the same bits only then), rebuilt when its twin changes, and its launch
    sequence is linked beside the default one."""
    from jetshow_gb300 import build as B
    assert "jsh_persistent_ft.cu" in B.CU_SOURCES
    assert {"jsh_persistent.cu", "jsh_persistent_ft.cu"} <= B.NO_CONTRACT
    assert B.INCLUDED["jsh_persistent_ft.cu"] == ["jsh_persistent.cu"]
    src = open(os.path.join(REPO, "jetshow_gb300", "csrc", "jsh_persistent_ft.cu")).read()
    assert "#define JSH_FARADAY_THICK_BUILD 1" in src and '#include "jsh_persistent.cu"' in src
    import subprocess
    syms = subprocess.run(["nm", "-D", A.LIB_PATH], capture_output=True, text=True).stdout
    assert "28jsh_launch_transfer_mixed_ftP" in syms  # the mode's launch sequence (mangled name)
    assert "25jsh_launch_transfer_mixedP" in syms  # the default one
    assert A.FLAG_FARADAY_THICK == 0x100
