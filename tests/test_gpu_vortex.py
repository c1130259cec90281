"""2-D isentropic vortex on the GPU: FP64 form against the oracle (same
inputs, 1e-12), FP32-storage form against the FP64 form and both against
the analytic translated vortex."""
import numpy as np
import pytest

from astr_gb300 import cases

pytestmark = pytest.mark.gpu

GAMMA = 1.4
MACH = 1.0 / np.sqrt(GAMMA)
H = 5


def _setup(n):
    st = cases.vortex_state(n)
    x, y, z = cases.vortex_grid(n)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    dt = cases.cfl_deltat(st, (d11, d22, d33), MACH)
    return st, (d11, d22, d33, J), dt


def _gpu(n, precision, st, metrics, dt, steps):
    from astr_gb300.solver import GpuSolver
    g = GpuSolver(n, n, 0, precision=precision, diffterm=False, mach=MACH, reynolds=1e4,
                  deltat=dt)
    g.set_metrics_diag(*metrics)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    g.time_integration_rk(steps)
    out = g.download_state()
    g.close()
    return out


def _sl(n):
    return (slice(H, H + n + 1), slice(H, H + n + 1), H)


@pytest.mark.parametrize("n", [64, 96])
def test_vortex_fp64_matches_oracle(gpu_lib, n):
    from astr_gb300 import capi
    from oracle import pyoracle as po
    st, metrics, dt = _setup(n)
    steps = 5
    o = po.from_state(st, (n, n, 0), lx=10.0, ly=10.0, lz=0.0, diffterm=False, mach=MACH,
                      reynolds=1e4, deltat=dt)
    o.rk3_steps(steps)
    g = _gpu(n, capi.FP64, st, metrics, dt, steps)
    sl = _sl(n)
    assert not np.any(g["q"][sl + (3,)])  # rho*w stays zero in 2-D
    for m in (0, 1, 2, 4):
        ref = o.field("q")[sl + (m,)]
        err = np.abs(g["q"][sl + (m,)] - ref).max() / np.abs(ref).max()
        assert err <= 1e-12, (m, err)
    for name in ("prs", "tmp", "rho"):
        ref = o.field(name)[sl]
        err = np.abs(g[name][sl] - ref).max() / np.abs(ref).max()
        assert err <= 1e-12, (name, err)


def test_vortex_fp32_storage_error(gpu_lib):
    from astr_gb300 import capi
    n, t_end = 128, 1.0
    st, metrics, dt = _setup(n)
    steps = int(round(t_end / dt))
    dt = t_end / steps
    g64 = _gpu(n, capi.FP64, st, metrics, dt, steps)
    g32 = _gpu(n, capi.FP32_STORAGE, st, metrics, dt, steps)
    ex = cases.vortex_state(n, t=t_end)
    sl = _sl(n)

    def l2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    e32 = l2(g32["q"][sl + (slice(0, 4),)], g64["q"][sl + (slice(0, 4),)])
    ea64 = float(np.sqrt(np.mean((g64["rho"][sl] - ex["rho"][sl]) ** 2)))
    ea32 = float(np.sqrt(np.mean((g32["rho"][sl] - ex["rho"][sl]) ** 2)))
    print(f"vortex 128^2, t=1: FP32-storage vs FP64 rel L2 {e32:.2e}; rho RMS error vs analytic "
          f"FP64 {ea64:.2e} FP32-storage {ea32:.2e}")
    assert e32 <= 1e-5
    assert ea64 < 1e-6 and ea32 < 1e-6
