"""Serving loop: requests admitted by memory budget into a running batch,
leaving when done.  Each request's result must equal the same simulation
run alone."""
import numpy as np
import pytest

from dlbc_gb300 import lbgpu, serve

pytestmark = pytest.mark.gpu


def small_requests():
    specs = [((48, 32, 32), 7.0, 40, 3e-6), ((40, 36, 36), 6.0, 25, 0.0), ((64, 32, 32), 8.0, 55, 1e-5),
             ((32, 40, 40), 6.5, 10, 5e-6), ((56, 34, 34), 7.5, 33, 2e-6)]
    out = []
    for i, (gn, r, steps, acc) in enumerate(specs):
        req = serve.Request(i, 0.001 * i, gn, r, steps, acc)
        req.p = serve.droplet_channel_params(gn, r, acc)
        out.append(req)
    return out


@pytest.mark.parametrize("precision", [lbgpu.FP16, lbgpu.FP32])
def test_results_in_the_mix_equal_results_alone(precision):
    reqs = small_requests()
    per = max(2 * 2 * 19 * r.sites * (2 if precision == lbgpu.FP16 else 4) + r.sites for r in reqs)
    # room for about two members at a time: later requests wait and join as others leave
    srv = serve.Server(precision=precision, budget_bytes=2.2 * per, max_chunk=8, keep_state=True)
    out = srv.run(reqs, realtime=False)
    assert out["requests"] == len(reqs)
    assert out["peak_members"] >= 2
    assert any(r["queue"] > 0 for r in out["results"])
    for rec in out["results"]:
        req = reqs[rec["rid"]]
        g = lbgpu.GPULattice(req.p, precision=precision)
        g.init_device()
        g.step(req.steps)
        alone = g.population()
        for c in range(2):
            assert np.array_equal(rec["population"][c], alone[c]), (rec["rid"], c)


def test_request_larger_than_budget_is_refused():
    reqs = small_requests()[:1]
    srv = serve.Server(precision=lbgpu.FP16, budget_bytes=1e5)
    with pytest.raises(lbgpu.BudgetExceeded):
        srv.run(reqs, realtime=False)
