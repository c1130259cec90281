"""Device monitors: cflcal (src/commcal.F90:27-87) against the host
restatement, and crashcheck (src/mainloop.F90:709-812) on a state poisoned
on the host (no GPU fault is provoked)."""
import numpy as np
import pytest

from astr_gb300 import capi, cases

pytestmark = pytest.mark.gpu
H = 5


def _tgv(n, precision):
    from astr_gb300.solver import GpuSolver
    L = 2 * np.pi
    x, y, z = cases.gridcube(n, n, n, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.tgv_state(n, n, n, x=x, y=y, z=z)
    g = GpuSolver(n, n, n, precision=precision)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    return g, st, (d11, d22, d33)


@pytest.mark.parametrize("precision,tol", [(capi.FP64, 1e-13), (capi.FP32_STORAGE, 1e-6)])
def test_cflcal_matches_host(gpu_lib, precision, tol):
    g, st, diag = _tgv(32, precision)
    dt = cases.cfl_deltat(st, diag, 0.1, 0.5)
    cfl, d3 = g.cflcal(dt)
    g.close()
    assert abs(cfl - 0.5) <= tol * 0.5, cfl
    assert np.all(d3 > 0)


def test_cflcal_vortex_2d(gpu_lib):
    from astr_gb300.solver import GpuSolver
    mach = 1.0 / np.sqrt(1.4)
    st = cases.vortex_state(64)
    x, y, z = cases.vortex_grid(64)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    dt = cases.cfl_deltat(st, (d11, d22, d33), mach, 0.5)
    g = GpuSolver(64, 64, 0, diffterm=False, mach=mach, deltat=dt)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    cfl, d3 = g.cflcal(dt)
    g.close()
    assert abs(cfl - 0.5) <= 1e-13 and d3[2] == 0.0


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32_STORAGE])
def test_crashcheck(gpu_lib, precision):
    g, st, _ = _tgv(24, precision)
    assert g.crashcheck() == (0, None)
    g.close()
    q = st["q"].copy(order="F")
    q[H + 3, H + 4, H + 5, 0] = -1.0
    q[H + 10, H + 2, H + 7, 0] = np.nan
    from astr_gb300.solver import GpuSolver
    L = 2 * np.pi
    x, y, z = cases.gridcube(24, 24, 24, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    g = GpuSolver(24, 24, 24, precision=precision)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(q, st["rho"], st["vel"], st["prs"], st["tmp"])
    n, ijk = g.crashcheck()
    g.close()
    assert n == 2
    # the node with the smaller interior index i + (im+1)(j + (jm+1)k) is reported
    assert ijk == min(((3, 4, 5), (10, 2, 7)), key=lambda t: t[0] + 25 * (t[1] + 25 * t[2]))
