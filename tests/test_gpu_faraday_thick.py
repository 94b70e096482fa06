"""The Faraday-thick mode of the mixed-precision IQUV pass
(JSH_FLAG_FARADAY_THICK: kernels built with the mode) on the ParabaloidCone jet, whose core
rays carry Faraday depths of ~2.5e7 rad: where |k_F| >= 100 k_I the pass
follows (Q, U) at its quasi-static value S / (k_I - i k_F) plus a decaying
transient and steps on I and V alone.  Checked here: it cuts the work of the
Faraday-thick rays, it meets the contract gates against the converged FP64
oracle on exactly those rays, it leaves the tau pass alone, and every form
of the mixed path gives the same bits with it; on a jet without
Faraday-thick rays the mode's kernels give the default kernels' bits."""
import numpy as np
import pytest

from jetshow_gb300 import _capi as A
from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W
from helpers import compare_images, flat

pytestmark = pytest.mark.gpu


def _render(ctx, jet, plane, nu, schedule="persistent", flags=0):
    return ctx.render(jet.desc(), plane.desc(), nu,
                      J.make_params(precision="mixed", schedule=schedule, flags=flags, **W.ACCURATE_KW))


@pytest.fixture(scope="module")
def c2_full(ctx):
    """The 1024x1024 ParabaloidCone image at 5.5 and 16.94 GHz, with the mode
    and without it, with the cost map."""
    jet, plane, nu, _ = W.parabolic_c2()
    on, s_on = _render(ctx, jet, plane, nu, flags=A.FLAG_COST_MAP | A.FLAG_FARADAY_THICK)
    off, s_off = _render(ctx, jet, plane, nu, flags=A.FLAG_COST_MAP)
    return (jet, plane, nu), (flat(on), s_on), (flat(off), s_off)


def test_mode_cuts_the_faraday_thick_rays_work(c2_full):
    _, (on, s_on), (off, s_off) = c2_full
    hit = (off["status"] & 1) != 0
    # the tau pass is untouched
    assert np.array_equal(on["tau"], off["tau"])
    assert np.array_equal(on["status"], off["status"])
    # the heaviest ray of the full integration takes ~1.2 M evaluations; the
    # mode takes it (and every other) to a few 10^4
    assert on["l"][hit].max() * 10 < off["l"][hit].max()
    assert s_on["rhs_evals"] < s_off["rhs_evals"]
    # the two integrations agree within the contract gates
    compare_images(on, off, full=True, tau_max=1e4)


def test_mode_vs_converged_oracle_on_the_heaviest_rays(c2_full, oracle):
    """The 48 rays the full integration finds heaviest (per frequency) and the
    16 deepest, against the converged oracle (rtol 1e-10)."""
    (jet, plane, nu), (on, _), (off, _) = c2_full
    hit = (off["status"] & 1) != 0
    pix = []
    for f in range(nu.size):
        cost = np.where(hit[f], off["l"][f], -1.0)
        pix.append(np.argsort(cost)[::-1][:48])
    tau0 = np.where(hit[0], off["tau"][0], -1.0)
    pix.append(np.argsort(tau0)[::-1][:16])
    pix = np.unique(np.concatenate(pix))
    ref = oracle.render(jet.desc(), plane.desc(), nu, J.make_params(**W.CONVERGED_KW), pix=pix,
                        threads=oracle.threads())
    sub = {k: v[:, pix] for k, v in on.items() if isinstance(v, np.ndarray) and v.ndim == 2}
    e = compare_images(sub, ref, full=True, tau_max=1e4)
    # the mode's approximations are held to rtol relative to I
    assert max(e["Q"], e["U"], e["V"]) < 1e-5


@pytest.mark.parametrize("flags", [A.FLAG_SERIAL_PASSES, A.FLAG_OVERLAP_PASSES, A.FLAG_SINGLE_KERNEL,
                                   A.FLAG_COMPACT_REGS, A.FLAG_GENERAL_KERNELS])
def test_mode_gives_the_same_bits_in_every_form(ctx, flags):
    """Static schedule, split form (serial and overlapped passes), single
    kernel, and each build of the kernels on the 256x256 image: every plane
    and counter bitwise the same with the mode engaged."""
    jet, plane, nu, _ = W.parabolic_c2(scale=4)
    ft = A.FLAG_FARADAY_THICK
    ref, sr = _render(ctx, jet, plane, nu, schedule="static", flags=ft | A.FLAG_COST_MAP)
    got, sg = _render(ctx, jet, plane, nu, flags=ft | flags | A.FLAG_COST_MAP)
    for k in ("tau", "l", "I", "Q", "U", "V", "status"):
        assert np.array_equal(got[k], ref[k]), k
    for k in ("rhs_evals", "steps_accepted", "steps_rejected", "status_or"):
        assert sg[k] == sr[k], k
    if flags == A.FLAG_SERIAL_PASSES:
        _, s_off = _render(ctx, jet, plane, nu)
        assert sr["rhs_evals"] < s_off["rhs_evals"]  # the mode is engaged on this image


@pytest.mark.parametrize("schedule", ["static", "persistent"])
def test_mode_kernels_give_the_default_bits_without_faraday_thick_rays(ctx, schedule):
    """The conical jet has no Faraday-thick rays: the mode never engages and
    the kernels built with it give every plane and counter of the default
    kernels."""
    jet, plane, nu, _ = W.conical_c1(scale=8)
    a, sa = _render(ctx, jet, plane, nu, schedule=schedule, flags=A.FLAG_COST_MAP)
    b, sb = _render(ctx, jet, plane, nu, schedule=schedule, flags=A.FLAG_COST_MAP | A.FLAG_FARADAY_THICK)
    for k in ("tau", "l", "I", "Q", "U", "V", "status"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("rhs_evals", "steps_accepted", "steps_rejected"):
        assert sa[k] == sb[k], k
