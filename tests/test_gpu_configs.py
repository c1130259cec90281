"""Parity on the reference configurations themselves, GPU against the oracle.

- Plain-method TGV: 64^3, main-solver ordering, dt fixed from cflcal's
  measure at CFL 0.5, 100 RK3 steps, FP64: every state field and the
  kinetic-energy / enstrophy history within 1e-12 (max-norm relative), on
  the register-window sweeps and on the tiled sweeps.
- Isentropic vortex: 512^2, inviscid, CFL 0.5; FP64 against the oracle over
  200 steps (1e-12), and the FP32-storage form against FP64 over the full
  1000 steps (relative L2 1e-5).
- Channel: 256 x 192 x 128, tanh-stretched walls, body force and
  controller; FP64 against the oracle over 20 steps (1e-12) and the
  FP32-storage form against FP64 (relative L2 1e-5).
"""
import numpy as np
import pytest

from conftest import relerr
from oracle import pyoracle as po
from test_gpu_parity import TOL, compare_state, gpu_from_oracle

pytestmark = pytest.mark.gpu

L2_TOL = 1e-5


def _rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def tgv64_oracle():
    """The 64^3 TGV at CFL 0.5 after 100 oracle steps, with its initial state."""
    import bench
    _, st = bench.tgv_inputs(64)
    dt = st["deltat"]
    o = po.tgv_main(64, deltat=dt)
    init = {k: o.field(k).copy() for k in ("q", "rho", "vel", "prs", "tmp")}
    hist = o.rk3_steps(100)
    return o, init, hist, dt


@pytest.mark.parametrize("tiled", [False, True])
def test_c0_tgv64_cfl05_100_steps(gpu_lib, tgv64_oracle, monkeypatch, tiled):
    from astr_gb300 import capi
    from astr_gb300.solver import GpuSolver
    if tiled:
        monkeypatch.setenv("ASTR_V2", "2")
    o, init, hist_o, dt = tgv64_oracle
    c = o.cfg
    g = GpuSolver(64, 64, 64, order=capi.ORDER_MAIN, mach=c.mach, reynolds=c.reynolds, deltat=dt)
    g.set_metrics(o.field("dxi"), o.field("jacob"))
    g.upload_state(init["q"], init["rho"], init["vel"], init["prs"], init["tmp"])
    hist_g = g.time_integration_rk(100)
    st = g.download_state()
    g.close()
    compare_state(o, st, full=True)
    e = relerr(hist_g, hist_o)
    print(f"TGV 64^3, 100 steps at CFL 0.5 (dt {dt:.4e}): KE/enstrophy history rel err {e:.2e}")
    assert e <= TOL


def test_c1_vortex512_fp64_200_steps(gpu_lib):
    from astr_gb300 import capi
    from test_gpu_vortex import MACH, _gpu, _setup, _sl
    n, steps = 512, 200
    st, metrics, dt = _setup(n)
    o = po.from_state(st, (n, n, 0), lx=10.0, ly=10.0, lz=0.0, diffterm=False, mach=MACH,
                      reynolds=1e4, deltat=dt)
    o.rk3_steps(steps)
    g = _gpu(n, capi.FP64, st, metrics, dt, steps)
    sl = _sl(n)
    errs = {}
    for m in (0, 1, 2, 4):
        errs[f"q{m + 1}"] = relerr(g["q"][sl + (m,)], o.field("q")[sl + (m,)])
    for name in ("prs", "tmp", "rho"):
        errs[name] = relerr(g[name][sl], o.field(name)[sl])
    print("vortex 512^2, 200 steps, FP64 vs oracle: " + " ".join(f"{k} {v:.1e}" for k, v in errs.items()))
    assert max(errs.values()) <= TOL, errs


def test_c1_vortex512_fp32_storage_1000_steps(gpu_lib):
    from astr_gb300 import capi
    from test_gpu_vortex import _gpu, _setup, _sl
    n, steps = 512, 1000
    st, metrics, dt = _setup(n)
    g64 = _gpu(n, capi.FP64, st, metrics, dt, steps)
    g32 = _gpu(n, capi.FP32_STORAGE, st, metrics, dt, steps)
    sl = _sl(n)
    e = {"rho": _rel_l2(g32["q"][sl + (0,)], g64["q"][sl + (0,)]),
         "mom": _rel_l2(g32["q"][sl + (slice(1, 3),)], g64["q"][sl + (slice(1, 3),)]),
         "E": _rel_l2(g32["q"][sl + (4,)], g64["q"][sl + (4,)])}
    print("vortex 512^2, 1000 steps, FP32 storage vs FP64 rel L2: " +
          " ".join(f"{k} {v:.2e}" for k, v in e.items()))
    assert max(e.values()) <= L2_TOL


def test_c3_channel_full_size_20_steps(gpu_lib):
    from astr_gb300 import capi
    from test_gpu_channel import _case, gpu_channel
    im, jm, km = 256, 192, 128
    steps = 20
    o, dxi = _case(im, jm, km)
    out = {}
    for name, prec in (("fp64", capi.FP64), ("fp32", capi.FP32_STORAGE)):
        g = gpu_channel(o, dxi, prec)
        g.time_integration_rk(steps)
        out[name] = (g.download_state(), g.channel_state())
        g.close()
    o.rk3_steps(steps)
    h = po.HM
    sl = (slice(h, h + im + 1), slice(h, h + jm + 1), slice(h, h + km + 1))
    s64 = out["fp64"][0]
    errs = {f"q{m + 1}": relerr(s64["q"][sl + (m,)], o.field("q")[sl + (m,)]) for m in range(5)}
    for name in ("prs", "tmp", "rho"):
        errs[name] = relerr(s64[name][sl], o.field(name)[sl])
    print(f"channel {im}x{jm}x{km}, {steps} steps, FP64 vs oracle: " +
          " ".join(f"{k} {v:.1e}" for k, v in errs.items()))
    assert max(errs.values()) <= TOL, errs
    oc, cs = o.chan_state(), out["fp64"][1]
    for k in (1, 2, 3):
        assert abs(cs[k] - oc[k]) <= TOL * abs(oc[k]), (k, cs[k], oc[k])
    a, b = out["fp32"][0]["q"][sl], s64["q"][sl]
    e = {"rho": _rel_l2(a[..., 0], b[..., 0]), "mom": _rel_l2(a[..., 1:4], b[..., 1:4]),
         "E": _rel_l2(a[..., 4], b[..., 4])}
    print("channel FP32 storage vs FP64 rel L2: " + " ".join(f"{k} {v:.2e}" for k, v in e.items()))
    assert max(e.values()) <= L2_TOL
