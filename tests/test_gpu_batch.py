"""Batches (astr_batch_*): persistent kernels over the (case, block) items of
many cases, one launch per phase of an RK3 stage.

- A mix of cases (3-D viscous boxes of several sizes and chunk lengths, one
  small enough to spread its variables over blocks, a 2-D inviscid vortex,
  each with its own time step) advances bit for bit as each case alone, in
  both precision forms.
- The deadline: a budget that has run out before the first gate leaves
  every case untouched; a budget that runs out part-way stops at a step
  boundary, and the cases equal that many steps run alone.
- The cancel word, set by another host thread during a call, does the same.
- Cases outside what the batch kernels run are refused with a reason.
- The serving loop on the batch gives every case the result it has alone.
"""
import threading
import time

import numpy as np
import pytest

from astr_gb300 import capi

pytestmark = pytest.mark.gpu

FIELDS = ("q", "rho", "vel", "prs", "tmp")


def _tgv(dims, precision, dt, reynolds=1600.0, **kw):
    from astr_gb300 import cases
    from astr_gb300.solver import GpuSolver
    im, jm, km = dims
    L = 2 * np.pi
    x, y, z = cases.gridcube(im, jm, km, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.tgv_state(im, jm, km, x=x, y=y, z=z)
    g = GpuSolver(im, jm, km, precision=precision, deltat=dt, reynolds=reynolds, **kw)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    return g


def _vortex(n, precision):
    from astr_gb300 import cases
    from astr_gb300.solver import GpuSolver
    mach = 1.0 / np.sqrt(1.4)
    st = cases.vortex_state(n)
    x, y, z = cases.vortex_grid(n)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    dt = cases.cfl_deltat(st, (d11, d22, d33), mach)
    g = GpuSolver(n, n, 0, precision=precision, diffterm=False, mach=mach, reynolds=1e4, deltat=dt)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    return g


# (builder, arguments): 40^3 spreads its variables over blocks; 64^3 and
# the anisotropic box run whole lines per block with other chunk lengths
MIX = [
    (_tgv, ((40, 40, 40), 2e-3)),
    (_tgv, ((64, 64, 64), 1e-3)),
    (_tgv, ((72, 40, 56), 1.5e-3, 800.0)),
    (_vortex, (64,)),
]


def _make(k, precision):
    f, a = MIX[k]
    if f is _vortex:
        return _vortex(a[0], precision)
    return _tgv(a[0], precision, *a[1:])


def _alone(k, precision, steps):
    g = _make(k, precision)
    if steps:
        g.time_integration_rk(steps, stats=False)
    out = g.download_state()
    g.close()
    return out


def _same(a, b):
    return all(np.array_equal(a[f], b[f]) for f in FIELDS)


@pytest.mark.parametrize("precision", [capi.FP32_STORAGE, capi.FP64])
def test_batch_equals_alone(gpu_lib, monkeypatch, precision):
    if precision == capi.FP64:
        monkeypatch.setenv("ASTR_V2", "2")   # the FP64 form on the tiled sweeps
    steps = 4
    b = capi.Batch(precision)
    gs = [_make(k, precision) for k in range(len(MIX))]
    for g in gs:
        b.add(g)
    assert len(b) == len(MIX)
    code, n = b.step(steps)
    assert (code, n) == (capi.ASTR_OK, steps)
    assert b.launches > 0
    # a second call continues from where the first stopped
    code, n = b.step(1)
    assert (code, n) == (capi.ASTR_OK, 1)
    for k, g in enumerate(gs):
        got = g.download_state()
        want = _alone(k, precision, steps + 1)
        assert _same(got, want), k
        g.close()
    assert len(b) == 0   # destroying a context removes it from its batch
    b.close()


def test_deadline_before_first_step_leaves_cases_untouched(gpu_lib):
    b = capi.Batch(capi.FP32_STORAGE)
    gs = [_make(k, capi.FP32_STORAGE) for k in (1, 3)]
    before = [g.download_state() for g in gs]
    for g in gs:
        b.add(g)
    code, n = b.step(50, budget_ms=1e-6)
    assert code == capi.ASTR_ERR_TIMEOUT and n == 0
    for g, s in zip(gs, before):
        assert _same(g.download_state(), s)
        g.close()
    b.close()


def test_deadline_part_way_stops_at_a_step_boundary(gpu_lib):
    b = capi.Batch(capi.FP32_STORAGE)
    probe = _make(1, capi.FP32_STORAGE)
    b.add(probe)
    t0 = time.perf_counter()
    assert b.step(10)[0] == capi.ASTR_OK
    t_step = (time.perf_counter() - t0) / 10 * 1e3
    probe.close()
    g = _make(1, capi.FP32_STORAGE)
    b.add(g)
    total = 400
    code, n = b.step(total, budget_ms=40 * t_step)
    assert code == capi.ASTR_ERR_TIMEOUT, (code, n)
    assert 0 < n < total
    assert _same(g.download_state(), _alone(1, capi.FP32_STORAGE, n))
    g.close()
    b.close()


def test_cancel_from_another_thread(gpu_lib):
    b = capi.Batch(capi.FP32_STORAGE)
    g = _make(1, capi.FP32_STORAGE)
    b.add(g)
    total = 1000
    t = threading.Timer(0.03, b.cancel)
    t.start()
    b.step_async(total)
    code, n = b.wait()
    t.join()
    assert code == capi.ASTR_ERR_CANCELLED, (code, n)
    assert 0 < n < total
    assert _same(g.download_state(), _alone(1, capi.FP32_STORAGE, n))
    # the next call starts with the cancel word clear
    assert b.step(1) == (capi.ASTR_OK, 1)
    g.close()
    b.close()


def test_refusals(gpu_lib, monkeypatch):
    b = capi.Batch(capi.FP32_STORAGE)
    g64 = _tgv((32, 32, 32), capi.FP64, 1e-3)          # FP64 on the register-window sweeps
    with pytest.raises(capi.AstrError) as e:
        b.add(g64)
    assert e.value.code == capi.ASTR_ERR_UNSUPPORTED and "precision" in str(e.value)
    g64.close()
    wall = _tgv((32, 32, 32), capi.FP32_STORAGE, 1e-3, npdc=(3, 4, 3), bctype=(0, 0, 41, 41, 0, 0))
    with pytest.raises(capi.AstrError) as e:
        b.add(wall)
    assert e.value.code == capi.ASTR_ERR_UNSUPPORTED
    wall.close()
    g = _tgv((32, 32, 32), capi.FP32_STORAGE, 1e-3)
    b.add(g)
    with pytest.raises(capi.AstrError) as e:
        b.add(g)
    assert e.value.code == capi.ASTR_ERR_STATE
    b.remove(g)
    assert len(b) == 0
    g.close()
    b.close()
    b64 = capi.Batch(capi.FP64)
    g = _tgv((32, 32, 32), capi.FP64, 1e-3)             # created without ASTR_V2=2
    with pytest.raises(capi.AstrError) as e:
        b64.add(g)
    assert e.value.code == capi.ASTR_ERR_UNSUPPORTED and "tiled" in str(e.value)
    g.close()
    b64.close()


def test_serving_on_the_batch_equals_alone(gpu_lib):
    from astr_gb300 import serve
    from test_gpu_serve import MIX as REQS, _alone as serve_alone
    be = serve.BatchBackend(capi.FP32_STORAGE, chunk=5, groups=2)
    srv = serve.Server(be, hbm_budget=8 << 30, max_active=4)
    recs = serve.serve(REQS, srv)
    assert srv.peak_active >= 2 and be.calls > 1 and be.batch_launches > 0
    for req, rec in zip(REQS, recs):
        ref = serve_alone(req, capi.FP32_STORAGE)
        for k in FIELDS:
            assert np.array_equal(rec.result[k], ref[k]), (req.rid, k)
    be.close()
