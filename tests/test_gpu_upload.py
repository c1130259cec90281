"""astr_gpu_upload_q: uploading q alone (primitives recomputed on the device)
gives the same steps as uploading the whole state, in both forms."""
import numpy as np
import pytest

from astr_gb300 import capi, cases

pytestmark = pytest.mark.gpu
H = 5


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32_STORAGE])
def test_upload_q_matches_full_state(gpu_lib, prec):
    from astr_gb300.solver import GpuSolver
    n = 32
    L = 2.0 * np.pi
    x, y, z = cases.gridcube(n, n, n, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.tgv_state(n, n, n, mach=0.1, x=x, y=y, z=z)
    dt = cases.cfl_deltat(st, (d11, d22, d33), 0.1, 0.5)
    out = []
    for full in (True, False):
        g = GpuSolver(n, n, n, precision=prec, mach=0.1, reynolds=1600.0, deltat=dt)
        g.set_metrics_diag(d11, d22, d33, J)
        if full:
            g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
        else:
            g.upload_q(st["q"])
        g.time_integration_rk(3)
        out.append(g.download_state())
        g.close()
    # FP32 storage: the recomputed primitives are q2fvar of the FP32 copy of
    # q (as at the end of every step of that form), the uploaded ones were
    # the host's FP64 values rounded once; the difference is that form's own
    # rounding level
    tol = 1e-12 if prec == capi.FP64 else 1e-6
    sl = (slice(H, H + n + 1),) * 3
    for name in ("q", "rho", "prs", "tmp"):
        a, b = out[1][name][sl], out[0][name][sl]
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err <= tol, (name, err)
