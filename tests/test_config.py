"""The legacy config.json driver (jetshow_gb300.config, the config-driven
observation of src/main.cpp:69-225) on the CPU: a config in the reference
file's layout becomes the descriptors, plane, frequency, integration
arguments and output maps the driver used."""
import json
import math

import pytest

from jetshow_gb300 import _capi as A
from jetshow_gb300 import config as CF
from jetshow_gb300 import jet as J
from jetshow_gb300.runtime import mas_to_pc

CFG = {
    "observation": {"redshift": 0.2, "frequency_ghz": 8.0, "los_angle": 0.15},
    "jet": {"geometry": {"type": "cone", "parameters": {"angle": 0.04, "scale_pc": 50.0}},
            "bfield": {"type": "spiral_conical", "parameters": {"pitch_angle": 0.7, "random_fraction": 0.0,
                                                                 "b_1": 0.5, "n_b": 1}},
            "vfield": {"type": "const_central", "parameters": {"gamma": 7}},
            "nfield": {"type": "bk", "parameters": {"n_n": 2.0, "n_1": 300}}},
    "image": {"pixel_size_mas": 0.002, "number_of_pixels": 64},
    "integration": {"step_type": "adaptive",
                    "parameters": {"n_tau_max": 500, "log10_abs_error_I": -10.0, "tau_max": 100.0,
                                   "log10_tau_min": -6.0, "n": 50, "dl_max_pc": 0.01,
                                   "log10_rel_error_tau": -8.0, "log10_abs_error_tau": -4.0, "tau_n_min": 0.1,
                                   "log10_rel_error_I": -6.0}},
    "output": {"file_tau": "t.txt", "file_i": "i.txt", "file_length": "l.txt", "file_q": "q.txt",
               "file_u": "u.txt", "file_v": "v.txt"},
    "calculate": "full",
}


def test_config_builds_the_drivers_observation(lib, tmp_path):
    path = tmp_path / "config.json"
    path.write_text(json.dumps(CFG))
    for src in (CFG, str(path), json.dumps(CFG)):
        b = CF.build(src)
        m = b["jet"].desc()
        assert m.geometry.kind == A.GEO_CONE and m.geometry.angle == 0.04
        assert m.geometry.big_scale == 50.0 * J.pc
        assert m.bfield.kind == A.B_SPIRAL_CONICAL and list(m.bfield.p[:2]) == [0.5, 0.7]
        assert m.vfield.kind == A.V_CONST_CENTRAL and m.vfield.p[0] == 7.0
        assert m.nfield.kind == A.N_BK and list(m.nfield.p[:2]) == [300.0, 2.0]
        pl = b["plane"].desc()
        assert (pl.n_across, pl.n_along) == (64, 64)
        assert pl.lg_pixel_size_start_cm == pytest.approx(math.log10(0.002 * 0.25 * mas_to_pc(0.2) * J.pc), rel=1e-15)
        assert b["nu"] == pytest.approx(8e9 * 1.2)
        r = b["run"]
        assert (r["n"], r["tau_max"], r["dt_max"], r["output_type"]) == (50, 100.0, 0.01, "full")
        assert r["tau_min"] == pytest.approx(1e-6) and r["rtol"] == pytest.approx(1e-6)
        assert [mp[0] for mp in b["maps"]] == ["tau", "I", "l", "Q", "U", "V"]
        jy = dict((mp[0], mp[2]) for mp in b["maps"])["I"]
        assert jy == pytest.approx(1e-23 / (0.002 * J.mas_to_rad) ** 2)


def test_config_random_fraction_wraps_the_field(lib):
    # the driver's PointsRandomVectorBField(bfield, random_fraction, 123)
    cfg = json.loads(json.dumps(CFG))
    cfg["jet"]["bfield"]["parameters"]["random_fraction"] = 0.3
    d = CF.build(cfg)["jet"].desc()
    assert (d.random.kind, d.random.fraction, d.random.seed) == (A.RND_POINTS, 0.3, 123)
    assert d.bfield.kind == A.B_SPIRAL_CONICAL


def test_config_rejects_what_the_driver_cannot_render(lib):
    bad = json.loads(json.dumps(CFG))
    bad["jet"]["geometry"]["type"] = "cylinder"
    with pytest.raises(ValueError):
        CF.build(bad)
    bad = json.loads(json.dumps(CFG))
    bad["calculate"] = "QU"
    with pytest.raises(ValueError):
        CF.build(bad)
