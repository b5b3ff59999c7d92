"""Request stream of the serving workload (host logic, no GPU)."""
import numpy as np

from dlbc_gb300 import serve


def test_stream_distributions():
    reqs = serve.request_stream(400, rate=50.0, seed=7)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0)
    assert abs(len(reqs) / arr[-1] - 50.0) < 10.0
    for r in reqs:
        x, y, z = r.gn
        assert 48 <= x <= 256 and 32 <= y <= 128 and y == z
        assert 6.0 <= r.radius <= y / 4.0
        assert 2000 <= r.steps <= 20000
        assert 0.0 <= r.acc <= 1e-5
        assert r.p.dimension_has_wall[2] == [True, True] and r.p.mask_init == 5
    again = serve.request_stream(400, rate=50.0, seed=7)
    assert [r.gn for r in again] == [r.gn for r in reqs]


def test_step_scale():
    reqs = serve.request_stream(20, seed=1, step_scale=0.1)
    assert all(200 <= r.steps <= 2000 for r in reqs)
