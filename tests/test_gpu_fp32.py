"""The FP32-storage form against the plain FP64 form.

The FP32-storage form streams every field in FP32 and computes the sweeps
in FP32, keeping the RK3 base (qsave) and a master copy of the conserved
variables in FP64.  Its bar is a relative L2 error <= 1e-5 against the FP64
form on the Taylor-Green vortex; the measured errors are printed.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L2_TOL = 1e-5


def _case(n, precision, order=0, steps=10):
    from astr_gb300 import capi, cases
    from astr_gb300.solver import GpuSolver
    L = 2 * np.pi
    x, y, z = cases.gridcube(n, n, n, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.tgv_state(n, n, n, x=x, y=y, z=z)
    g = GpuSolver(n, n, n, order=order, precision=precision)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    hist = g.time_integration_rk(steps)
    out = g.download_state()
    g.close()
    return out, hist


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("n", [48, 64])
def test_fp32_storage_tgv_error(gpu_lib, n):
    from astr_gb300 import capi
    s64, h64 = _case(n, capi.FP64)
    s32, h32 = _case(n, capi.FP32_STORAGE)
    h = 5
    sl = (slice(h, h + n + 1),) * 3
    errs = {}
    # scalars field by field; momentum and velocity as vectors (the TGV's
    # w starts at exactly zero, so a per-component norm of rho*w is empty)
    errs["rho"] = rel_l2(s32["q"][sl + (0,)], s64["q"][sl + (0,)])
    errs["mom"] = rel_l2(s32["q"][sl + (slice(1, 4),)], s64["q"][sl + (slice(1, 4),)])
    errs["E"] = rel_l2(s32["q"][sl + (4,)], s64["q"][sl + (4,)])
    for name in ("prs", "tmp"):
        errs[name] = rel_l2(s32[name][sl], s64[name][sl])
    errs["vel"] = rel_l2(s32["vel"][sl], s64["vel"][sl])
    ke = float(np.max(np.abs(h32[:, 0] - h64[:, 0]) / np.abs(h64[:, 0])))
    en = float(np.max(np.abs(h32[:, 1] - h64[:, 1]) / np.abs(h64[:, 1])))
    print(f"FP32-storage vs FP64, TGV {n}^3, 10 steps: "
          + " ".join(f"{k} {v:.2e}" for k, v in errs.items()) + f"; KE {ke:.2e} enstrophy {en:.2e}")
    assert max(errs.values()) <= L2_TOL
    assert ke <= L2_TOL and en <= L2_TOL


def test_fp32_storage_golden_history(gpu_lib):
    """Mini-app ordering in the FP32-storage form against the reference's
    golden 128^3 history (first 20 steps), at the FP32 bar."""
    import os
    from astr_gb300 import capi
    from oracle import pyoracle as po
    from test_gpu_parity import gpu_from_oracle
    ref = np.loadtxt(os.path.join(os.path.dirname(__file__), "golden", "tgv128_state_ref.txt"))
    o = po.tgv_miniapp(128)
    g = gpu_from_oracle(o, precision=capi.FP32_STORAGE)
    hist = g.time_integration_rk(20)
    ke = float(np.max(np.abs(hist[:, 0] - ref[:20, 2]) / ref[:20, 2]))
    en = float(np.max(np.abs(hist[:, 1] - ref[:20, 3]) / ref[:20, 3]))
    print(f"FP32-storage mini-app vs state.ref_128 (20 steps): KE {ke:.2e} enstrophy {en:.2e}")
    assert ke <= L2_TOL and en <= L2_TOL
