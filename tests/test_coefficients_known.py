"""Known answers of the transfer coefficients: the oracle's eleven lab-frame
coefficients against an independent restatement of the reference's
formulas, at points, lines of sight and frequencies where the field laws
(themselves pinned by test_field_laws_known.py) give B, n and v.

Restated from the reference (CGS constants of include/utils.h:22-36):
* nu_p, nu_b, k_0, eta_0 and the power-law coefficients k_i, k_q, k_v,
  k_F_c, k_C_c, k_F_r, k_C_r, eta_i, eta_q, eta_v (src/utils.cpp:8-144),
  with the random-field factors of the scalar-B forms (:46-51, :125-130);
* the plasma-frame kinematics getG, getD, get_n_los_prime, getBprime
  (src/utils.cpp:145-170) and the lab-frame conversion k = k'/D,
  eta = eta' D^2 with nu' = nu/D, n' = n/Gamma for densities given in the
  lab frame (src/Jet.cpp:15-46, :218-237);
* the builder-defined thermal share: cold k_F_c and k_C_c of n_th = f n'
  added to the relativistic k_F_r and k_C_r.
"""
import math

import numpy as np
import pytest

from jetshow_gb300 import jet as J

PC = 3.0856775814913673e18
M_E = 9.10938356e-28
Q_E = 4.80320467299766e-10
C_LIGHT = 29979245800.0
PI = math.pi
G = math.gamma


def plasma_frame(b, n, v, nl, nu, b_lab, n_lab):
    beta = np.asarray(v) / C_LIGHT
    gamma = 1.0 / math.sqrt(1.0 - beta @ beta)
    D = 1.0 / (gamma * (1.0 - beta @ nl))
    nlp = D * nl - (D + 1.0) * (gamma / (gamma + 1.0)) * beta
    if b_lab and b is not None:
        b = b / gamma + gamma / ((1.0 + gamma) * C_LIGHT ** 2) * np.asarray(v) * (np.asarray(v) @ b)
    return b, (n / gamma if n_lab else n), nlp, nu / D, D


def expected(b, n, v, nl, nu, s, gamma_min, thermal, b_lab, n_lab, scalar_b=False):
    """The eleven lab-frame coefficients (k_I, k_Q, k_U, k_V, k_F, k_C, h_Q,
    eta_I, eta_Q, eta_U, eta_V) from the reference's formulas."""
    out = np.zeros(11)
    b, n, nlp, nup, D = plasma_frame(None if scalar_b else np.asarray(b, float), n, v, np.asarray(nl, float), nu,
                                     b_lab, n_lab)
    nu_p2 = n * Q_E ** 2 / (PI * M_E)
    if scalar_b:
        bb = float(scalar_b)
        nub = Q_E * bb / (2 * PI * M_E * C_LIGHT)
        fk = 3 ** ((s + 1) / 2) / 4 * G(s / 4 + 11 / 6) * G(s / 4 + 1 / 6) * math.sqrt(PI / 4) * G((6 + s) / 4) / G(
            (8 + s) / 4)
        fe = 3 ** (s / 2) / (2 * (s + 1)) * G(s / 4 + 19 / 12) * G(s / 4 - 1 / 12) * math.sqrt(PI / 4) * G(
            (5 + s) / 4) / G((7 + s) / 4)
        out[0] = PI * nu_p2 * nub / (C_LIGHT * nup ** 2) * (nub / nup) ** (s / 2) * fk / D
        out[7] = PI * nu_p2 * nub * M_E / C_LIGHT * (nub / nup) ** ((s - 1) / 2) * fe * D * D
        return out
    bn = math.sqrt(b @ b)
    nub = Q_E * np.linalg.norm(np.cross(nlp, b)) / (2 * PI * M_E * C_LIGHT)
    nubv = Q_E * bn / (2 * PI * M_E * C_LIGHT)
    cos_t = (b @ nlp) / bn
    k0 = PI * nu_p2 * nub / (C_LIGHT * nup ** 2)
    k0v = PI * nu_p2 * nubv / (C_LIGHT * nup ** 2)
    e0 = PI * nu_p2 * nub * M_E / C_LIGHT
    e0v = PI * nu_p2 * nubv * M_E / C_LIGHT
    ki = k0 * (nub / nup) ** (s / 2) * 3 ** ((s + 1) / 2) / 4 * G(s / 4 + 11 / 6) * G(s / 4 + 1 / 6)
    kq = (s + 2) / (s + 10 / 3) * ki
    kv = -k0v * cos_t * (nub / nup) ** ((s + 1) / 2) * 3 ** (s / 2) * (s + 3) * (s + 2) / (4 * (s + 1)) * G(
        s / 4 + 11 / 12) * G(s / 4 + 7 / 12)

    def kfc(npl2):
        return 2 * PI * npl2 * nubv * cos_t / (C_LIGHT * nup ** 2)

    def kcc(npl2):
        return -PI * npl2 * nub ** 2 / (C_LIGHT * nup ** 3)

    kf = (s + 2) * math.log(gamma_min) / ((s + 1) * gamma_min ** (s + 1)) * kfc(nu_p2)
    kc = 2 / (s - 2) * (gamma_min ** (2 - s) - (nub / nup) ** ((s - 2) / 2)) * kcc(nu_p2)
    if thermal:
        kf += kfc(thermal * nu_p2)
        kc += kcc(thermal * nu_p2)
    ei = e0 * (nub / nup) ** ((s - 1) / 2) * 3 ** (s / 2) / (2 * (s + 1)) * G(s / 4 + 19 / 12) * G(s / 4 - 1 / 12)
    eq = (s + 1) / (s + 7 / 3) * ei
    ev = -e0v * cos_t * (nub / nup) ** (s / 2) * 3 ** ((s - 1) / 2) * (s + 2) / (2 * s) * G(s / 4 + 2 / 3) * G(
        s / 4 + 1 / 3)
    out[[0, 1, 3, 4, 5]] = np.array([ki, kq, kv, kf, kc]) / D
    out[[7, 8, 10]] = np.array([ei, eq, ev]) * D * D
    return out


CONE = J.Cone((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.1, 100 * PC)
MODELS = {
    # B and n given in the plasma frame, radial flow, thermal share, gamma_min 10
    "helical_plasma": (J.Jet(CONE, J.ConstCentralVField(8.0), J.HelicalConicalBField(0.5, 1.0, 0.7, True),
                             J.BKNField(1e3, 2.0, True), s=2.5, gamma_min=10.0, thermal_fraction=0.1),
                       False, False, False),
    # B and n given in the lab frame (Lorentz-transformed B, n / Gamma), flat flow
    "toroidal_lab": (J.Jet(CONE, J.ConstFlatVField(3.0), J.ToroidalBField(0.2, 1.0, False),
                           J.BKNFieldZ(300.0, 2.0, False), s=3.42, gamma_min=100.0),
                     True, True, False),
    # scalar (tangled) B: k_I and eta_I with the random-field factors only
    "scalar_random": (J.Jet(CONE, J.ConstFlatVField(5.0), J.RandomScalarBFieldZ(0.3, 1.0),
                            J.ConstNField(50.0, False), s=3.42, gamma_min=100.0),
                      False, True, True),
}
POINTS = [(0.01, 0.02, 1.0), (-0.05, 0.03, 3.0), (0.2, -0.1, 7.5)]
LOS = [(math.sin(0.1), 0.0, math.cos(0.1)), (0.3, -0.5, 0.812403840463596), (math.sin(1.2), 0.0, math.cos(1.2))]
FREQS = [5e9, 15.4e9, 43e9]


@pytest.mark.parametrize("name", list(MODELS))
def test_coefficients_match_the_reference_formulas(oracle, name):
    jet, b_lab, n_lab, scalar = MODELS[name]
    m = jet.desc()
    worst = 0.0
    for pt in POINTS:
        p = np.array(pt) * PC
        f = oracle.fields(m, p)
        b, n, v = f[:3], f[3], f[4:7]
        for los in LOS:
            nl = np.array(los) / np.linalg.norm(los)
            for nu in FREQS:
                got = oracle.coefficients(m, p, nl, nu)
                exp = expected(b, n, v, nl, nu, jet.s, jet.gamma_min, jet.thermal_fraction, b_lab, n_lab,
                               scalar_b=b[0] if scalar else False)
                for i in range(11):
                    if exp[i] == 0.0:
                        assert got[i] == 0.0, (name, i)
                    else:
                        worst = max(worst, abs(got[i] - exp[i]) / abs(exp[i]))
    assert worst < 1e-12, worst


def test_lab_frame_conversion_is_exercised(oracle):
    """The restatement's frames matter: the flow is relativistic (D far from
    1) and the lab-frame B differs from the plasma-frame B."""
    jet, *_ = MODELS["toroidal_lab"]
    p = np.array(POINTS[1]) * PC
    f = oracle.fields(jet.desc(), p)
    nl = np.array(LOS[0])
    bp, npr, _, _, D = plasma_frame(f[:3], f[3], f[4:7], nl, 15.4e9, True, True)
    assert D > 2.0 and abs(npr - f[3] / 3.0) < 1e-12 * f[3]
    assert np.linalg.norm(bp - f[:3]) > 0.1 * np.linalg.norm(f[:3])
