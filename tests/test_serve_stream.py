"""Request stream of the serving workload and the serving loop's admission
and chunking against a fake batch (host logic, no GPU)."""
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


class _FakeMember:
    def reduce(self):
        return np.zeros(2), np.zeros((2, 3))


class _FakeBatch:
    """The batch interface the server uses, with a byte budget of `sites`
    units and the launches recorded (no GPU)."""

    def __init__(self, budget_sites):
        from dlbc_gb300 import lbgpu

        self.err = lbgpu.BudgetExceeded
        self.budget = budget_sites
        self.members = {}  # sid -> [request sites, steps done]
        self.next_sid = 0
        self.admitted = []  # rids in admission order
        self.chunks = []

    @property
    def device_bytes(self):
        return sum(v[0] for v in self.members.values())

    def add_device(self, p):
        sites = int(np.prod(p.gn[:3]))
        if self.device_bytes + sites > self.budget:
            raise self.err("budget")
        sid = self.next_sid
        self.next_sid += 1
        self.members[sid] = [sites, 0]
        self.admitted.append(p.rid)
        return sid

    def step(self, k):
        assert k >= 1 and self.members
        self.chunks.append(k)
        for v in self.members.values():
            v[1] += k

    def synchronize(self):
        pass

    def member(self, sid):
        return _FakeMember()

    def remove(self, sid):
        del self.members[sid]


def _server(budget_sites, age_limit_s=5.0, max_chunk=500):
    s = object.__new__(serve.Server)
    s.batch = _FakeBatch(budget_sites)
    s.max_chunk, s.min_chunk, s.age_limit_s, s.keep_state = max_chunk, 25, age_limit_s, False
    return s


def _requests(specs):
    out = []
    for rid, (n, steps) in enumerate(specs):
        r = serve.Request(rid, 0.0, (n, n, n), 4.0, steps, 0.0)
        r.p = serve.droplet_channel_params(r.gn, 4.0, 0.0)
        r.p.rid = rid
        out.append(r)
    return out


def test_server_admits_fit_first_and_completes_every_request():
    """A large request at the head that does not fit yet does not hold back
    smaller ones behind it; every request does exactly its steps; chunks end
    when a member finishes."""
    # budget 30 000 sites: the first (8 000) runs; the second (27 000, more
    # than the room left) waits; the small ones behind it (1 000, 1 000,
    # 1 728) are admitted meanwhile, the second once the first has finished
    reqs = _requests([(20, 300), (30, 100), (10, 50), (10, 80), (12, 120)])
    s = _server(budget_sites=30_000)
    out = s.run(reqs, realtime=False)
    assert out["requests"] == 5
    b = s.batch
    assert b.admitted[:4] == [0, 2, 3, 4] and b.admitted[4] == 1
    assert sorted(r["rid"] for r in out["results"]) == [0, 1, 2, 3, 4]
    # every chunk ended at a member's completion: the chunk boundaries are
    # exactly the completion step counts of the members that ran together
    assert b.chunks == [50, 30, 40, 180, 100]
    assert out["site_steps"] == sum(r.sites * r.steps for r in reqs)
    assert out["peak_members"] == 4 and out["peak_device_bytes"] <= 30_000


def test_server_aging_stops_overtaking():
    """Once the waiting head has aged past the limit, nothing overtakes it."""
    reqs = _requests([(20, 400), (30, 100), (10, 50), (10, 50)])
    s = _server(budget_sites=30_000, age_limit_s=-1.0)
    s.run(reqs, realtime=False)
    # the head (rid 1) does not fit beside rid 0 and has aged at once: rids
    # 2 and 3 wait behind it (without aging they would run beside rid 0)
    assert s.batch.admitted == [0, 1, 2, 3] and s.batch.chunks[0] == 400
