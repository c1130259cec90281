"""Host-side tests of the serving loop: the request stream and the
scheduler (first come first served, slots, HBM budget, continuous
admission), against a simulated processor-sharing device."""
import math

import numpy as np
import pytest

from astr_gb300 import serve


def test_request_stream():
    reqs = serve.make_requests(2000, rate=50.0, seed=20261203)
    assert [r.rid for r in reqs] == list(range(2000))
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0)
    assert abs(len(reqs) / arr[-1] - 50.0) < 5.0  # Poisson rate
    n3 = [r.n for r in reqs if r.kind == "tgv3d"]
    n2 = [r.n for r in reqs if r.kind == "vortex2d"]
    assert 0.4 < len(n3) / len(reqs) < 0.6
    assert min(n3) >= 32 and max(n3) <= 192 and min(n2) >= 64 and max(n2) <= 1024
    # log-uniform edges: the median near the geometric mean
    assert abs(math.log(np.median(n3)) - 0.5 * math.log(32 * 192)) < 0.15
    assert all(100 <= r.reynolds <= 3000 and 0.05 <= r.mach <= 0.3 and 50 <= r.steps <= 500
               for r in reqs)
    again = serve.make_requests(2000, rate=50.0, seed=20261203)
    assert again == reqs


def _run(reqs, budget, slots, rate=1e6):
    dev = serve.FakeDevice(rate=rate)
    be = serve.FakeBackend(dev)
    srv = serve.Server(be, budget, max_active=slots)
    recs = serve.serve(reqs, srv, clock=serve.FakeClock(dev), poll_interval=1e-3)
    return srv, be, recs


def test_scheduler_fifo_budget_slots():
    reqs = serve.make_requests(60, rate=50.0, seed=7, edge3d=(8, 24), edge2d=(16, 64),
                               steps=(5, 20))
    budget = int(max(serve.request_points(r) for r in reqs) * 100 * 3)
    srv, be, recs = _run(reqs, budget, slots=4)
    assert len(recs) == 60 and all(r.finished >= r.admitted >= r.arrival for r in recs)
    assert be.started == sorted(be.started)  # admitted in arrival order
    assert srv.peak_active <= 4 and srv.peak_used <= budget
    assert srv.used == 0 and not srv.active


def test_continuous_admission_overlaps_work():
    # slow device: the second request arrives while the first is running and
    # is admitted before the first finishes
    reqs = [serve.Request(0, "tgv3d", 32, 1000.0, 0.1, 100, 0.0),
            serve.Request(1, "vortex2d", 64, 1000.0, 0.1, 50, 0.05)]
    srv, be, recs = _run(reqs, budget=10**12, slots=8, rate=2e6)
    assert recs[1].admitted < recs[0].finished
    # sharing the device: the first case takes longer than alone
    alone = serve.request_points(reqs[0]) * 3 * reqs[0].steps / 2e6
    assert recs[0].latency > alone


def test_sequential_baseline_and_summary():
    reqs = serve.make_requests(20, rate=50.0, seed=3, edge3d=(8, 16), edge2d=(16, 32),
                               steps=(5, 10))
    dev = serve.FakeDevice(rate=1e5)
    recs = serve.serve_sequential(reqs, serve.FakeBackend(dev), clock=serve.FakeClock(dev),
                                  poll_interval=1e-3)
    for a, b in zip(recs, recs[1:]):
        assert b.admitted >= a.finished - 1e-12
    s = serve.summarize(reqs, recs)
    assert s["cases"] == 20 and s["latency_p99_s"] >= s["latency_p50_s"] > 0


def test_oversize_request_rejected():
    dev = serve.FakeDevice()
    srv = serve.Server(serve.FakeBackend(dev), hbm_budget=1000)
    with pytest.raises(ValueError):
        srv.submit(serve.Request(0, "tgv3d", 64, 100.0, 0.1, 10, 0.0))


def test_partition_across_gpus():
    reqs = serve.make_requests(50, rate=50.0, seed=11)
    parts = [serve.partition(reqs, r, 4) for r in range(4)]
    assert sorted(q.rid for p in parts for q in p) == list(range(50))
    assert all(q.rid % 4 == r for r, p in enumerate(parts) for q in p)


class _PreparingBackend(serve.FakeBackend):
    """A backend with host-side preparation: the server must hand each case
    the inputs prepared for it."""

    def __init__(self, device):
        super().__init__(device)
        self.prepared = []

    def prepare(self, req):
        self.prepared.append(req.rid)
        return ("inputs", req.rid)

    def start(self, req, inputs=None):
        assert inputs == ("inputs", req.rid)
        return super().start(req)


def test_scheduler_prefetches_inputs():
    reqs = serve.make_requests(40, rate=50.0, seed=11, edge3d=(8, 24), edge2d=(16, 64),
                               steps=(5, 20))
    dev = serve.FakeDevice(rate=1e6)
    be = _PreparingBackend(dev)
    budget = int(sum(be.footprint(r) for r in reqs) * 0.3)
    srv = serve.Server(be, budget, max_active=4, prefetch=3)
    recs = serve.serve(reqs, srv, clock=serve.FakeClock(dev), poll_interval=1e-3)
    srv.close()
    assert [r.rid for r in recs] == [q.rid for q in reqs]
    # first come first served, every case prepared exactly once before it started
    assert be.started == sorted(be.started)
    assert sorted(be.prepared) == be.started


class _FakeBatch:
    """Stands in for capi.Batch: a call of k steps finishes at the next
    poll; a case added while a call is in flight is refused as the C ABI
    refuses it."""

    def __init__(self, precision):
        self.members = []
        self.calls = []
        self.inflight = None

    def add(self, g):
        from astr_gb300 import capi
        if self.inflight is not None:
            raise capi.AstrError(capi.ASTR_ERR_STATE, "a batched call is in flight")
        self.members.append(g)

    def remove(self, g):
        self.members.remove(g)

    def __len__(self):
        return len(self.members)

    def step_async(self, k):
        assert self.inflight is None and k > 0
        self.inflight = k
        self.calls.append((k, list(self.members)))

    def poll(self):
        return True

    def wait(self):
        from astr_gb300 import capi
        k, self.inflight = self.inflight, None
        return capi.ASTR_OK, k


def test_batch_group_joins_and_leaves_between_calls(monkeypatch):
    """Calls of min(chunk, fewest remaining steps); a case leaves when its
    steps are done and a case that arrives during a call joins after it."""
    from astr_gb300 import capi
    monkeypatch.setattr(capi, "Batch", _FakeBatch)
    grp = serve._Group(capi.FP32_STORAGE, chunk=20)
    a, b, c = (serve._BatchCase(name, 1.0) for name in ("a", "b", "c"))
    a.remaining, b.remaining, c.remaining = 50, 7, 30
    for h in (a, b):
        grp.batch.add(h.g)
        grp.members.append(h)
    grp.tick()                                  # starts a call of 7 steps
    assert grp.batch.calls[-1] == (7, ["a", "b"])
    grp.joining.append(c)                       # arrives during the call
    grp.tick()                                  # harvest: b done; c joins; next call
    assert b.finished and not a.finished and (a.remaining, c.remaining) == (43, 30)
    assert grp.batch.calls[-1] == (20, ["a", "c"])
    for _ in range(4):
        grp.tick()
    assert a.finished and c.finished and a.remaining == 0 and c.remaining == 0
    assert [k for k, _ in grp.batch.calls] == [7, 20, 10, 13]
    assert grp.batch.members == []


class _FakeSolver:
    """A case's solver for BatchBackend host tests: records graph steps."""

    def __init__(self, name, batchable=True):
        self.name, self.batchable = name, batchable
        self.graph_steps = 0

    def step_async(self, n):
        self.graph_steps += n

    def poll(self):
        return True


class _RefusingBatch(_FakeBatch):
    def add(self, g):
        from astr_gb300 import capi
        if not g.batchable:
            raise capi.AstrError(capi.ASTR_ERR_UNSUPPORTED, "not batchable")
        super().add(g)


def test_batch_backend_routes_cases(monkeypatch):
    """A batchable case joins the batch (or waits for the call in flight);
    a case the batch refuses runs on its own graphs; one above max_points
    too; the call cycle finishes every batched case."""
    from astr_gb300 import capi
    monkeypatch.setattr(capi, "Batch", _RefusingBatch)
    be = serve.BatchBackend.__new__(serve.BatchBackend)
    be.groups = [serve._Group(capi.FP32_STORAGE, 8)]
    be.max_points = 1000.0
    a = serve._BatchCase(_FakeSolver("a"), 500.0)
    b = serve._BatchCase(_FakeSolver("b", batchable=False), 500.0)
    big = serve._BatchCase(_FakeSolver("big"), 5000.0)
    be.enqueue(a, 12)
    be.enqueue(b, 5)
    be.enqueue(big, 7)
    assert a.group is be.groups[0] and b.group is None and big.group is None
    assert (b.g.graph_steps, big.g.graph_steps) == (5, 7)
    assert be.done(b) and be.done(big)          # own graphs: their stream's poll
    assert not be.done(a)                        # starts a call of 8 steps
    c = serve._BatchCase(_FakeSolver("c"), 100.0)
    be.enqueue(c, 3)                             # call in flight: joins after it
    assert c in be.groups[0].joining
    while not (be.done(a) and be.done(c)):
        pass
    calls = [(k, [g.name for g in m]) for k, m in be.groups[0].batch.calls]
    assert calls == [(8, ["a"]), (3, ["a", "c"]), (1, ["a"])]
    assert be.calls == 3
