"""Host side of the serving stream (no GPU): the seeded request stream
follows the model-fitting priors and Poisson arrivals, and the server
entry points reject bad arguments before touching a device."""
import ctypes as C
import math

import numpy as np

from jetshow_gb300 import _capi as A
from jetshow_gb300 import jet as J
from jetshow_gb300 import serving as S


def test_stream_is_seeded_and_poisson():
    a = S.request_stream(400, rate_hz=200.0, seed=42)
    b = S.request_stream(400, rate_hz=200.0, seed=42)
    assert [r.t_arrival for r in a] == [r.t_arrival for r in b]
    gaps = np.diff([0.0] + [r.t_arrival for r in a])
    assert np.all(gaps > 0)
    # exponential inter-arrivals with mean 5 ms: mean within 4 sigma, CV near 1
    assert abs(gaps.mean() - 0.005) < 4 * 0.005 / math.sqrt(gaps.size)
    assert 0.8 < gaps.std() / gaps.mean() < 1.2


def test_stream_priors():
    rng = np.random.default_rng(0)
    labels, kinds = [], []
    for _ in range(300):
        jet, plane, nu, label = S.sample_request(rng)
        m, p = jet.desc(), plane.desc()
        labels.append(label)
        kinds.append(m.geometry.kind)
        assert 0.02 <= p.los_angle <= 0.3
        assert 1 <= nu.size <= 4 and np.all(np.diff(nu) >= 0)
        assert np.all(nu >= 5e9) and np.all(nu <= 43e9 * 1.1 + 1)
        b0 = m.bfield.p[0]
        assert 0.01 <= b0 <= 1.0
        assert 10.0 <= m.nfield.p[0] <= 1e4
        assert 2.0 <= m.vfield.p[0] <= 20.0
        if label == "512x1024log":
            assert (p.n_across, p.n_along) == (512, 1024) and p.lg_pixel_size_stop_cm > p.lg_pixel_size_start_cm
        else:
            n = int(label.split("x")[0])
            assert (p.n_across, p.n_along) == (n, n)
    assert set(labels) == set(S.SIZES)
    assert set(kinds) == {A.GEO_CONE, A.GEO_PARABALOID_CONE}


def test_server_rejects_null_arguments():
    lib = A.load_library()
    cfg = A.ServerConfig(max_inflight_batches=2, max_batch_requests=8, precision=A.PREC_MIXED, use_graphs=1)
    out = C.c_void_p()
    assert lib.jsh_server_create(None, C.byref(cfg), C.byref(out)) == A.JSH_ERR_INVALID
    assert not out.value
    rid = C.c_uint64()
    p = J.make_params()
    assert lib.jsh_server_submit(None, None, None, None, 0, C.byref(p), C.byref(rid)) == A.JSH_ERR_INVALID
    assert lib.jsh_server_poll(None, 1) == A.JSH_ERR_INVALID
    assert lib.jsh_server_cancel(None, 1) == A.JSH_ERR_INVALID
