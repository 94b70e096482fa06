"""Shared comparison helpers of the parity tests (tolerances as stated by
the transfer-path contract: hit mask and hit count bit-exact; tau within
1e-5 relative; I within 1e-4 relative where I > 1e-6 max(I); Q/U/V within
1e-4 max(I); total flux within 1e-5)."""
import numpy as np

TAU_RTOL = 1e-5
I_RTOL = 1e-4
I_FLOOR = 1e-6
QUV_ATOL_FRAC = 1e-4
FLUX_RTOL = 1e-5


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor)
    with np.errstate(divide="ignore", invalid="ignore"):
        e = np.where(den > 0, np.abs(a - b) / den, np.where(a == b, 0.0, np.inf))
    return e


def compare_images(gpu: dict, ref: dict, full: bool, tau_max=None, tau_rtol=TAU_RTOL, i_rtol=I_RTOL,
                   quv_frac=QUV_ATOL_FRAC, flux_rtol=FLUX_RTOL):
    """gpu/ref: dicts of [n_nu, npix] arrays.  Returns a dict of worst errors
    and asserts the contract."""
    out = {}
    hit_g = (gpu["status"] & 1) != 0
    hit_r = (ref["status"] & 1) != 0
    assert np.array_equal(hit_g, hit_r), "hit mask differs"
    out["n_hit"] = int(hit_g.sum())
    tau_g, tau_r = gpu["tau"], ref["tau"]
    mask = hit_r
    if tau_max is not None:
        # a ray whose tau crossed tau_max stores tau at the end of the crossing
        # step (src/Observation.cpp:208); compare those rays only for crossing
        both = (tau_g >= tau_max) & (tau_r >= tau_max)
        mask = mask & ~both
    e_tau = rel_err(tau_g[mask], tau_r[mask], 1e-300)
    out["tau"] = float(e_tau.max()) if e_tau.size else 0.0
    assert out["tau"] <= tau_rtol, f"tau rel err {out['tau']}"
    for f in range(gpu["I"].shape[0]):
        Ig, Ir = gpu["I"][f], ref["I"][f]
        imax = np.abs(Ir).max()
        sel = np.abs(Ir) > I_FLOOR * imax
        e_i = rel_err(Ig[sel], Ir[sel])
        out.setdefault("I", 0.0)
        out["I"] = max(out["I"], float(e_i.max()) if e_i.size else 0.0)
        flux_g, flux_r = Ig.sum(), Ir.sum()
        out.setdefault("flux", 0.0)
        out["flux"] = max(out["flux"], abs(flux_g - flux_r) / abs(flux_r) if flux_r != 0 else abs(flux_g))
        if full:
            for k in ("Q", "U", "V"):
                e = np.abs(gpu[k][f] - ref[k][f]).max() / imax if imax > 0 else 0.0
                out[k] = max(out.get(k, 0.0), float(e))
    assert out["I"] <= i_rtol, f"I rel err {out['I']}"
    assert out["flux"] <= flux_rtol, f"flux rel err {out['flux']}"
    if full:
        for k in ("Q", "U", "V"):
            assert out[k] <= quv_frac, f"{k} err {out[k]} of max(I)"
    return out


def flat(d: dict):
    """[n_nu, na, nl] -> [n_nu, npix]"""
    return {k: (v.reshape(v.shape[0], -1) if isinstance(v, np.ndarray) and v.ndim == 3 else v)
            for k, v in d.items()}
