"""The allocation-free entry point (jsh_observation_run_noalloc) against the
stream-ordered entry point that allocates (jsh_observation_run_device).

Callers whose framework owns the device memory pool, or whose loops cannot
take cudaMalloc's implicit synchronisation, cannot allocate; this entry point
keeps its scratch in a file-scope device array.  Both entry points run the
same kernels with the same launch shape, so two calls in a row must each
reproduce the allocating entry point's images bit for bit (the array keeps
the previous call's contents, so the second call checks that everything that
must start at zero is cleared).  Runs alone in a fresh process or after the
suite.
"""
import ctypes as C

import numpy as np
import pytest

from jetshow_gb300 import _capi as A
from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W

pytestmark = pytest.mark.gpu

PLANES = ("tau", "l", "I", "Q", "U", "V")


def device_planes(torch, n_nu, npix):
    t = {k: torch.full((n_nu, npix), -1.0, dtype=torch.float64, device="cuda") for k in PLANES}
    t["status"] = torch.zeros((n_nu, npix), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()  # the fills run on torch's stream, the renders on another
    return t, A.DeviceImage(*(t[k].data_ptr() for k in PLANES), t["status"].data_ptr())


def to_host(t):
    out = {k: t[k].cpu().numpy() for k in PLANES}
    out["status"] = t["status"].cpu().numpy().astype(np.uint32)
    return out


@pytest.mark.parametrize("precision,flags", [("mixed", 0), ("mixed", A.FLAG_COMPACT_REGS), ("fp64", 0)])
def test_noalloc_matches_allocating_entry_point(lib, precision, flags):
    torch = pytest.importorskip("torch")
    from jetshow_gb300.runtime import Context, check

    jet, plane, nu, _ = W.conical_c0(scale=4)
    model, pdesc = jet.desc(), plane.desc()
    params = J.make_params(precision=precision, schedule="persistent", flags=flags, **W.ACCURATE_KW)
    nu = np.ascontiguousarray(nu, dtype=np.float64)
    npix = int(pdesc.n_across * pdesc.n_along)
    stream = torch.cuda.Stream()

    ctx = Context(0)
    ref_t, ref_img = device_planes(torch, nu.size, npix)
    check(lib, lib.jsh_observation_run_device(ctx.handle, C.byref(model), C.byref(pdesc), A.dptr(nu), nu.size,
                                              C.byref(params), C.c_void_p(stream.cuda_stream), C.byref(ref_img)))
    stream.synchronize()
    ref = to_host(ref_t)
    assert ((ref["status"] & A.ST_HIT) != 0).sum() > 0

    for call in range(2):
        out_t, out_img = device_planes(torch, nu.size, npix)
        check(lib, lib.jsh_observation_run_noalloc(C.byref(model), C.byref(pdesc), A.dptr(nu), nu.size,
                                                   C.byref(params), C.c_void_p(stream.cuda_stream),
                                                   C.byref(out_img)))
        stream.synchronize()
        got = to_host(out_t)
        for k in ("status",) + PLANES:
            assert np.array_equal(got[k], ref[k]), f"call {call}: plane {k} differs"
    ctx.close()


def test_noalloc_rejects_requests_beyond_its_limits(lib):
    jet, _, nu, _ = W.conical_c0()
    too_big = J.ImagePlane((512, 256), 17.0, 17.0, 0.1).desc()  # 131072 pixels > 65536
    params = J.make_params(**W.ACCURATE_KW)
    nu = np.ascontiguousarray(nu, dtype=np.float64)
    img = A.DeviceImage()
    st = lib.jsh_observation_run_noalloc(C.byref(jet.desc()), C.byref(too_big), A.dptr(nu), nu.size,
                                         C.byref(params), None, C.byref(img))
    assert st == A.JSH_ERR_INVALID
    assert b"no-alloc limits" in lib.jsh_last_error()
