"""CPU check of the folded coefficient algebra of the mixed-precision path
(jsh_fields32.cuh / jsh_prepare_mixed): restated in FP64 numpy, it must
reproduce the oracle's literal coefficients (src/utils.cpp:39-143 with the
frame transforms of src/Jet.cpp:15-46) to rounding level."""
import math

import numpy as np
import pytest
from scipy.special import gamma as tgamma

from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W

PC, ME, QE, CL = 3.0856775814671913e+18, 9.10938356e-28, 4.80320467299766e-10, 29979245800.0


def folded(s, gamma_min, thermal, nu, n, b_vec, D, nlp, scalar_b=None):
    cb = QE / (2 * math.pi * ME * CL)
    cp = QE * QE / (math.pi * ME)
    fk_i = (3 ** ((s + 1) / 2) / 4) * tgamma(s / 4 + 11 / 6) * tgamma(s / 4 + 1 / 6)
    fe_i = 3 ** (s / 2) / (2 * (s + 1)) * tgamma(s / 4 + 19 / 12) * tgamma(s / 4 - 1 / 12)
    fk_v = 3 ** (s / 2) * (s + 3) * (s + 2) / (4 * (s + 1)) * tgamma(s / 4 + 11 / 12) * tgamma(s / 4 + 7 / 12)
    fe_v = 3 ** ((s - 1) / 2) * (s + 2) / (2 * s) * tgamma(s / 4 + 2 / 3) * tgamma(s / 4 + 1 / 3)
    kfr = (s + 2) * math.log(gamma_min) / ((s + 1) * gamma_min ** (s + 1))
    kcr_a, kcr_b = 2 / (s - 2), gamma_min ** (2 - s)
    Ak = math.pi * cp * cb ** ((s + 2) / 2) * fk_i / (CL * nu ** ((s + 4) / 2))
    Ae = math.pi * cp * cb ** ((s + 1) / 2) * ME * fe_i / (CL * nu ** ((s - 1) / 2))
    Av = math.pi * cp * cb ** ((s + 3) / 2) * fk_v / (CL * nu ** ((s + 5) / 2))
    Aev = math.pi * cp * cb ** (1 + s / 2) * ME * fe_v / (CL * nu ** (s / 2))
    Af = 2 * math.pi * cp * cb / (CL * nu * nu) * (kfr + thermal)
    Ac = math.pi * cp * cb * cb / (CL * nu ** 3)
    Gnu = (cb / nu) ** ((s - 2) / 2)
    c1, c2 = kcr_a * kcr_b + thermal, kcr_a * Gnu
    w = np.linalg.norm(np.cross(nlp, b_vec)) * D
    P = w ** ((s + 2) / 2)
    R = P / math.sqrt(w)
    bpar = float(np.dot(b_vec, nlp))
    kI = Ak * n * P
    eI = Ae * n * R * D
    kQ = (s + 2) / (s + 10 / 3) * kI
    eQ = (s + 1) / (s + 7 / 3) * eI
    kV = -Av * n * bpar * R * D
    eV = -Aev * n * bpar * D * D * P / w
    kF = Af * n * bpar * D
    kC = -Ac * n * (c1 * w * w - c2 * P)
    return np.array([kI, kQ, 0, kV, kF, kC, 0, eI, eQ, 0, eV])


def log_domain(s, gamma_min, thermal, nu, n0, m_n, b0, m_b, u, r, D, nlp):
    """The log-domain form of the helical / BK family (coef32_helical_log):
    k_I and eta_I as one exp2 of a sum of logs, the rest from k_I, eta_I,
    n', b and w with per-frequency ratios."""
    cb = QE / (2 * math.pi * ME * CL)
    cp = QE * QE / (math.pi * ME)
    fk_i = (3 ** ((s + 1) / 2) / 4) * tgamma(s / 4 + 11 / 6) * tgamma(s / 4 + 1 / 6)
    fe_i = 3 ** (s / 2) / (2 * (s + 1)) * tgamma(s / 4 + 19 / 12) * tgamma(s / 4 - 1 / 12)
    fk_v = 3 ** (s / 2) * (s + 3) * (s + 2) / (4 * (s + 1)) * tgamma(s / 4 + 11 / 12) * tgamma(s / 4 + 7 / 12)
    fe_v = 3 ** ((s - 1) / 2) * (s + 2) / (2 * s) * tgamma(s / 4 + 2 / 3) * tgamma(s / 4 + 1 / 3)
    kfr = (s + 2) * math.log(gamma_min) / ((s + 1) * gamma_min ** (s + 1))
    kcr_a, kcr_b = 2 / (s - 2), gamma_min ** (2 - s)
    Ak = math.pi * cp * cb ** ((s + 2) / 2) * fk_i / (CL * nu ** ((s + 4) / 2))
    Ae = math.pi * cp * cb ** ((s + 1) / 2) * ME * fe_i / (CL * nu ** ((s - 1) / 2))
    Av = math.pi * cp * cb ** ((s + 3) / 2) * fk_v / (CL * nu ** ((s + 5) / 2))
    Aev = math.pi * cp * cb ** (1 + s / 2) * ME * fe_v / (CL * nu ** (s / 2))
    Af = 2 * math.pi * cp * cb / (CL * nu * nu) * (kfr + thermal)
    Ac = math.pi * cp * cb * cb / (CL * nu ** 3)
    Gnu = (cb / nu) ** ((s - 2) / 2)
    c1, c2 = kcr_a * kcr_b + thermal, kcr_a * Gnu
    r_kv, r_ev, r_kc = Av / Ae, Aev / Ak, Ac * c2 / Ak
    pk, pk_h = (s + 2) / 2, (s + 1) / 2
    sgn = 1.0 if b0 > 0 else -1.0
    l = math.log2(r)
    uu = sgn * np.asarray(u)
    lw = math.log2(abs(b0) * D) - m_b * l + 0.5 * math.log2(float(np.dot(np.cross(nlp, uu), np.cross(nlp, uu))))
    ln = math.log2(n0) - m_n * l
    kI = Ak * 2 ** (ln + pk * lw)
    eI = Ae * D * 2 ** (ln + pk_h * lw)
    n_ = 2 ** ln
    bpar = 2 ** (math.log2(abs(b0)) - m_b * l) * float(np.dot(uu, nlp))
    w = 2 ** lw
    kQ = (s + 2) / (s + 10 / 3) * kI
    eQ = (s + 1) / (s + 7 / 3) * eI
    kV = -r_kv * bpar * eI
    eV = -r_ev * bpar * D * D * kI / w
    kF = Af * n_ * bpar * D
    kC = r_kc * kI - Ac * c1 * n_ * w * w
    return np.array([kI, kQ, 0, kV, kF, kC, 0, eI, eQ, 0, eV])


@pytest.mark.parametrize("thermal", [0.0, 0.1])
def test_folded_algebra_matches_oracle(oracle, thermal):
    jet, plane, nu, kw = W.conical_c0()
    jet.thermal_fraction = thermal
    m = jet.desc()
    _, d, _ = oracle.plane_rays(plane.desc())
    nl = -d
    g = 10.0
    beta = math.sqrt(1 - 1 / g ** 2)
    D = 1 / (g * (1 - beta * nl[2]))
    nlp = D * nl - (D + 1) * (g / (g + 1)) * beta * np.array([0, 0, 1.0])
    rng = np.random.default_rng(3)
    for _ in range(20):
        p = rng.normal(size=3) * 3 * J.pc
        p[2] = abs(p[2]) + 0.5 * J.pc
        ref = oracle.coefficients(m, p, nl, nu[0])
        r = np.linalg.norm(p) / J.pc
        b = 0.1 * r ** -1.0
        rc = math.hypot(p[0], p[1])
        bvec = b * np.array([math.sin(math.pi / 4) * -p[1] / rc, math.sin(math.pi / 4) * p[0] / rc,
                             math.cos(math.pi / 4)])
        n = 500.0 * r ** -2.0
        got = folded(2.5, 10.0, thermal, nu[0], n, bvec, D, nlp)
        u = bvec / b
        logd = log_domain(2.5, 10.0, thermal, nu[0], 500.0, 2.0, 0.1, 1.0, u, r, D, nlp)
        for i in range(11):
            assert abs(got[i] - ref[i]) <= 1e-10 * max(abs(ref[i]), 1e-300), (i, got[i], ref[i])
            assert abs(logd[i] - ref[i]) <= 1e-10 * max(abs(ref[i]), 1e-300), (i, logd[i], ref[i])
        # a negative b0 reverses B: k_V, k_F, eta_V change sign, the rest do not
        neg = log_domain(2.5, 10.0, thermal, nu[0], 500.0, 2.0, -0.1, 1.0, u, r, D, nlp)
        sign = np.array([1, 1, 1, -1, -1, 1, 1, 1, 1, 1, -1])
        np.testing.assert_allclose(neg, sign * logd, rtol=1e-12)
