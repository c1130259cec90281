"""Request loop that serves many independent periodic cases on one GPU.

Requests (a 3-D Taylor-Green vortex or a 2-D isentropic vortex, each with its
own grid edge, Reynolds number, Mach number and step count) arrive over time.
The server admits them first come, first served, while a slot is free and
the case's HBM footprint fits under the budget.  An admitted case gets its
own context and stream; all of its RK3 steps are enqueued at once as CUDA
graph launches (astr_gpu_step_async), so the kernels of every admitted case
run concurrently on the device, and a case that arrives while others run
starts as soon as a slot and memory free up (continuous batching).  Finished
cases are downloaded and their memory released at the next scheduling pass.
BatchBackend instead steps the admitted cases together in one batch of
persistent kernels (astr_batch_*), cases joining and leaving between calls
of a few steps.

Nothing here has a counterpart in the reference, which runs one case per
MPI job; the cases themselves are the reference's TGV set-up (tgvini,
src/initialisation.F90:621-691) and the analytic isentropic vortex, at CFL
0.5 measured as cflcal does (src/commcal.F90:27-87).
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import capi, cases

PI = math.pi
GAMMA = 1.4


@dataclass
class Request:
    rid: int
    kind: str          # "tgv3d" or "vortex2d"
    n: int             # grid edge (intervals)
    reynolds: float
    mach: float
    steps: int
    arrival: float     # seconds after the start of the stream


def make_requests(count, rate=50.0, seed=20261203, edge3d=(32, 192), edge2d=(64, 1024),
                  re=(100.0, 3000.0), mach=(0.05, 0.3), steps=(50, 500), frac3d=0.5):
    """A Poisson stream of `count` requests at `rate` per second: half 3-D
    TGV, half 2-D vortex; grid edge log-uniform in edge3d / edge2d, Reynolds
    number log-uniform in `re`, Mach number uniform in `mach`, steps uniform
    over the integers in `steps` (numpy PCG64 stream of `seed`)."""
    rng = np.random.default_rng(seed)
    arrival = np.cumsum(rng.exponential(1.0 / rate, count))
    is3d = rng.random(count) < frac3d
    u_edge = rng.random(count)
    u_re = rng.random(count)
    u_mach = rng.random(count)
    nsteps = rng.integers(steps[0], steps[1] + 1, count)
    out = []
    for i in range(count):
        lo, hi = edge3d if is3d[i] else edge2d
        n = int(round(math.exp(math.log(lo) + u_edge[i] * (math.log(hi) - math.log(lo)))))
        r = math.exp(math.log(re[0]) + u_re[i] * (math.log(re[1]) - math.log(re[0])))
        m = mach[0] + u_mach[i] * (mach[1] - mach[0])
        out.append(Request(i, "tgv3d" if is3d[i] else "vortex2d", n, r, m, int(nsteps[i]),
                           float(arrival[i])))
    return out


def partition(requests, rank: int, world: int):
    """The requests one of `world` independent servers (one per GPU) takes:
    every world-th request of the stream, so each server sees the same
    arrival process thinned by `world`."""
    return [r for r in requests if r.rid % world == rank]


def request_points(req: Request) -> float:
    """Unique grid points of a request (periodic: edge^3 or edge^2)."""
    return float(req.n) ** (3 if req.kind == "tgv3d" else 2)


def _uniform_diag_metrics(dims, lengths):
    """dxi(d,d) = 1/spacing and jacob = cell volume (area in 2-D) on a
    uniform periodic grid, halo layout."""
    im, jm, km = dims
    full = (im + 11, jm + 11, km + 11)
    sp = [lengths[d] / dims[d] if dims[d] > 0 else 1.0 for d in range(3)]
    diag = [np.full(full, 1.0 / sp[d], order="F") if dims[d] > 0 else np.zeros(full, order="F")
            for d in range(3)]
    vol = sp[0] * sp[1] * (sp[2] if km > 0 else 1.0)
    return diag, np.full(full, vol, order="F")


def case_inputs(req: Request):
    """Dimensions, solver keyword arguments, diagonal metrics and initial
    state of one request."""
    if req.kind == "tgv3d":
        n = req.n
        L = 2.0 * PI
        x, y, z = cases.gridcube(n, n, n, L, L, L)
        st = cases.tgv_state(n, n, n, mach=req.mach, x=x, y=y, z=z)
        dims = (n, n, n)
        diag, J = _uniform_diag_metrics(dims, (L, L, L))
        kw = dict(mach=req.mach, reynolds=req.reynolds, diffterm=True)
    else:
        n = req.n
        st = cases.vortex_state(n, mach=req.mach)
        dims = (n, n, 0)
        diag, J = _uniform_diag_metrics(dims, (10.0, 10.0, 0.0))
        kw = dict(mach=req.mach, reynolds=req.reynolds, diffterm=False)
    kw["deltat"] = cases.cfl_deltat(st, diag, req.mach, 0.5)
    return dims, kw, diag, J, st


class GpuBackend:
    """One context and stream per case on the GPU."""

    def __init__(self, precision=capi.FP32_STORAGE):
        self.precision = precision
        self.L = capi.load()

    def footprint(self, req: Request) -> int:
        n = req.n
        dims = capi.AstrDims(n, n, n if req.kind == "tgv3d" else 0, n, n,
                             n if req.kind == "tgv3d" else 0, 3, 3, 3)
        p = capi.AstrParams()
        p.precision = self.precision
        return int(self.L.astr_gpu_footprint(dims, p))

    def prepare(self, req: Request):
        """Host-side inputs of a case (grid metrics, initial state, time
        step); thread-safe, run ahead of admission by the server."""
        return case_inputs(req)

    def start(self, req: Request, inputs=None):
        from .solver import GpuSolver
        dims, kw, diag, J, st = inputs if inputs is not None else case_inputs(req)
        g = GpuSolver(*dims, precision=self.precision, **kw)
        g.set_metrics_diag(diag[0], diag[1], diag[2], J)
        g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
        return g

    def enqueue(self, h, nsteps: int):
        h.step_async(nsteps)

    def done(self, h) -> bool:
        return h.poll()

    def finish(self, h):
        out = h.download_state()
        launches = h.launches
        h.close()
        return out, launches


class _BatchCase:
    """A case of the BatchBackend: its solver, the steps it still needs, its
    group (None: it runs on its own graphs) and whether it has finished."""

    def __init__(self, g, points):
        self.g = g
        self.points = points
        self.remaining = 0
        self.group = None
        self.finished = False


class _Group:
    """One batch, its stream and its call cycle: calls of up to `chunk`
    steps; between calls, cases that reached their step count leave and
    waiting cases join."""

    def __init__(self, precision, chunk):
        self.batch = capi.Batch(precision)
        self.chunk = chunk
        self.members: list = []
        self.joining: list = []
        self.inflight = 0
        self.calls = 0

    def load(self) -> float:
        return sum(h.points for h in self.members + self.joining)

    def tick(self):
        if self.inflight:
            if not self.batch.poll():
                return
            code, n = self.batch.wait()
            if code != capi.ASTR_OK:
                raise capi.AstrError(code, capi.batch_error(self.batch.h))
            self.inflight = 0
            for h in self.members:
                h.remaining -= n
            for h in [h for h in self.members if h.remaining <= 0]:
                self.batch.remove(h.g)
                self.members.remove(h)
                h.finished = True
        for h in self.joining:
            self.batch.add(h.g)
            self.members.append(h)
        self.joining = []
        if self.members:
            k = min(self.chunk, min(h.remaining for h in self.members))
            self.batch.step_async(k)
            self.inflight = k
            self.calls += 1


class BatchBackend(GpuBackend):
    """Cases step together in batches (astr_batch_*): every launch of a step
    is a persistent kernel over the (case, block) items of all the cases of
    a batch.  `groups` batches, each on its own stream, split the admitted
    cases by points (timed on a 32-case mix, more than one batch gained
    nothing: balanced batches run their phases in step).
    Each batch runs calls of up to `chunk` steps; between calls, cases that
    reached their step count leave and admitted cases join
    (iteration-level continuous batching).  A case the batch kernels do not
    take (a line longer than the tiled chunk lengths, for instance) runs on
    its own context's graphs as in GpuBackend, and so does a case of more
    than `max_points` points when that is set (large cases gain more from
    running concurrently with the others than from sharing launches)."""

    def __init__(self, precision=capi.FP32_STORAGE, chunk: int = 20, groups: int = 1,
                 max_points=None):
        super().__init__(precision)
        self.groups = [_Group(precision, int(chunk)) for _ in range(max(1, int(groups)))]
        self.max_points = max_points

    def start(self, req: Request, inputs=None):
        return _BatchCase(super().start(req, inputs), request_points(req))

    def enqueue(self, h, nsteps: int):
        h.remaining = int(nsteps)
        if h.remaining <= 0:
            h.finished = True
            return
        if self.max_points is not None and h.points > self.max_points:
            h.g.step_async(nsteps)
            return
        grp = min(self.groups, key=lambda q: q.load())
        try:
            grp.batch.add(h.g)
        except capi.AstrError as e:
            if e.code == capi.ASTR_ERR_UNSUPPORTED:
                h.g.step_async(nsteps)      # not batchable: own graphs
                return
            if e.code != capi.ASTR_ERR_STATE:
                raise
            h.group = grp
            grp.joining.append(h)           # a call is in flight: join after it
            return
        h.group = grp
        grp.members.append(h)

    def tick(self):
        """Harvest each batch's call in flight when it has finished and
        start its next call."""
        for grp in self.groups:
            grp.tick()

    def done(self, h) -> bool:
        if h.group is None:
            return h.finished or h.g.poll()
        self.tick()
        return h.finished

    def finish(self, h):
        out = h.g.download_state()
        launches = h.g.launches
        h.g.close()
        return out, launches

    @property
    def calls(self) -> int:
        return sum(q.calls for q in self.groups)

    @property
    def batch_launches(self) -> int:
        return sum(q.batch.launches for q in self.groups)

    def close(self):
        for q in self.groups:
            q.batch.close()


@dataclass
class _Slot:
    req: Request
    handle: object
    nbytes: int
    admitted: float


@dataclass
class Record:
    rid: int
    arrival: float
    admitted: float
    finished: float
    result: object = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


class Server:
    """First-come-first-served admission by free slots and HBM budget.  The
    host-side inputs of the next `prefetch` queued requests are prepared on
    worker threads while the admitted cases run, when the backend offers
    prepare()."""

    def __init__(self, backend, hbm_budget: int, max_active: int = 32, prefetch: int = 4):
        self.b = backend
        self.budget = int(hbm_budget)
        self.max_active = int(max_active)
        self.queue: collections.deque = collections.deque()
        self.active: dict = {}
        self.used = 0
        self.peak_used = 0
        self.peak_active = 0
        self.launches = 0
        self.prefetch = int(prefetch) if hasattr(backend, "prepare") else 0
        self._pool = cf.ThreadPoolExecutor(max_workers=2) if self.prefetch else None
        self._prepared: dict = {}

    def close(self):
        if self._pool:
            self._pool.shutdown(wait=True)
            self._pool = None

    def _prefetch(self):
        for req in list(self.queue)[: self.prefetch]:
            if req.rid not in self._prepared:
                self._prepared[req.rid] = self._pool.submit(self.b.prepare, req)

    def submit(self, req: Request):
        if self.b.footprint(req) > self.budget:
            raise ValueError(f"request {req.rid} needs more HBM than the whole budget")
        self.queue.append(req)

    def idle(self) -> bool:
        return not self.queue and not self.active

    def poll(self, now: float):
        """One scheduling pass: harvest finished cases, then admit from the
        head of the queue.  Returns the Records finished in this pass."""
        done = []
        for rid in list(self.active):
            s = self.active[rid]
            if self.b.done(s.handle):
                res, launches = self.b.finish(s.handle)
                self.launches += launches
                self.used -= s.nbytes
                del self.active[rid]
                done.append(Record(rid, s.req.arrival, s.admitted, now, res))
        while self.queue and len(self.active) < self.max_active:
            req = self.queue[0]
            nb = self.b.footprint(req)
            if self.used + nb > self.budget:
                break
            self.queue.popleft()
            if self.prefetch:
                fut = self._prepared.pop(req.rid, None)
                h = self.b.start(req, fut.result() if fut is not None else self.b.prepare(req))
            else:
                h = self.b.start(req)
            self.b.enqueue(h, req.steps)
            self.active[req.rid] = _Slot(req, h, nb, now)
            self.used += nb
            self.peak_used = max(self.peak_used, self.used)
            self.peak_active = max(self.peak_active, len(self.active))
        if self.prefetch:
            self._prefetch()
        if hasattr(self.b, "tick"):
            self.b.tick()   # a batching backend starts its next call
        return done


class WallClock:
    def __init__(self):
        self.t0 = time.perf_counter()

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def sleep(self, dt: float):
        time.sleep(dt)


def serve(requests, server: Server, clock=None, poll_interval=2e-4):
    """Feed the requests to the server at their arrival times and run its
    scheduling passes until every request has finished.  Returns the
    Records in request order."""
    clock = clock or WallClock()
    reqs = sorted(requests, key=lambda r: r.arrival)
    recs = {}
    i = 0
    while len(recs) < len(reqs):
        now = clock.now()
        while i < len(reqs) and reqs[i].arrival <= now:
            server.submit(reqs[i])
            i += 1
        for r in server.poll(now):
            recs[r.rid] = r
        if len(recs) < len(reqs):
            wait = poll_interval
            if server.idle() and i < len(reqs):
                wait = max(poll_interval, reqs[i].arrival - clock.now())
            clock.sleep(wait)
    return [recs[r.rid] for r in requests]


def serve_sequential(requests, backend, clock=None, poll_interval=2e-4):
    """The baseline: one case at a time in arrival order, each started when
    it has arrived and the previous one has finished."""
    clock = clock or WallClock()
    recs = []
    for req in sorted(requests, key=lambda r: r.arrival):
        while clock.now() < req.arrival:
            clock.sleep(min(poll_interval * 10, req.arrival - clock.now()))
        start = clock.now()
        h = backend.start(req)
        backend.enqueue(h, req.steps)
        while not backend.done(h):
            clock.sleep(poll_interval)
        res, _ = backend.finish(h)
        recs.append(Record(req.rid, req.arrival, start, clock.now(), res))
    order = {r.rid: k for k, r in enumerate(recs)}
    return [recs[order[r.rid]] for r in requests]


def summarize(requests, records):
    lat = np.array([r.latency for r in records])
    makespan = max(r.finished for r in records) - min(r.arrival for r in requests)
    pts = sum(request_points(q) * 3 * q.steps for q in requests)
    return {"cases": len(records), "makespan_s": round(float(makespan), 3),
            "cases_per_s": round(len(records) / makespan, 3),
            "latency_p50_s": round(float(np.percentile(lat, 50)), 4),
            "latency_p99_s": round(float(np.percentile(lat, 99)), 4),
            "latency_mean_s": round(float(lat.mean()), 4),
            "mpts_stages_per_s": round(pts / makespan / 1e6, 3)}


# -- a simulated device for host-side tests ---------------------------------
@dataclass
class _FakeCase:
    work: float
    enqueued: bool = False


@dataclass
class FakeDevice:
    """Processor sharing: the device completes `rate` units of work per
    second, split evenly among the cases with work in flight."""
    rate: float = 1.0
    cases: list = field(default_factory=list)

    def advance(self, dt: float):
        live = [c for c in self.cases if c.enqueued and c.work > 0]
        while dt > 0 and live:
            share = self.rate / len(live)
            t_min = min(c.work / share for c in live)
            step = min(dt, t_min)
            for c in live:
                c.work -= share * step
            dt -= step
            live = [c for c in live if c.work > 1e-12]


class FakeBackend:
    """Stands in for the GPU in scheduler tests: a case's work is its point
    stages; its footprint is proportional to its points."""

    def __init__(self, device: FakeDevice, bytes_per_point=100):
        self.dev = device
        self.bpp = bytes_per_point
        self.started = []

    def footprint(self, req):
        return int(request_points(req) * self.bpp)

    def start(self, req, inputs=None):
        c = _FakeCase(work=request_points(req) * 3 * req.steps)
        self.dev.cases.append(c)
        self.started.append(req.rid)
        return c

    def enqueue(self, h, nsteps):
        h.enqueued = True

    def done(self, h):
        return h.enqueued and h.work <= 1e-12

    def finish(self, h):
        self.dev.cases.remove(h)
        return None, 0


class FakeClock:
    def __init__(self, device: FakeDevice):
        self.t = 0.0
        self.dev = device

    def now(self):
        return self.t

    def sleep(self, dt):
        self.dev.advance(dt)
        self.t += dt
