"""General (non-diagonal) metrics on the GPU against the oracle: the
channel with the reference's own metrics (gridgeom's off-diagonal rounding
residue included) and a periodic curvilinear grid."""
import numpy as np
import pytest

from astr_gb300 import capi, cases

pytestmark = pytest.mark.gpu
H = 5


def _cmp(o, s, dims, tol=1e-12):
    im, jm, km = dims
    sl = (slice(H, H + im + 1), slice(H, H + jm + 1), slice(H, H + km + 1))
    qo = o.field("q")[sl]
    mom = np.abs(qo[..., 1:4]).max()  # momentum components against the vector's scale
    for m in range(5):
        ref = qo[..., m]
        scale = mom if 1 <= m <= 3 else np.abs(ref).max()
        err = np.abs(s["q"][sl + (m,)] - ref).max() / scale
        assert err <= tol, (m, err)
    for name in ("prs", "tmp", "rho"):
        ref = o.field(name)[sl]
        err = np.abs(s[name][sl] - ref).max() / np.abs(ref).max()
        assert err <= tol, (name, err)


def test_channel_full_metrics_match_oracle(gpu_lib):
    from test_channel import channel_oracle
    from test_gpu_channel import gpu_channel
    im, jm, km = 24, 40, 16
    o, _, _, _ = channel_oracle(im, jm, km, zero_offdiag=False)
    dxi = o.field("dxi")
    offdiag = [d + 3 * m for d in range(3) for m in range(3) if d != m]
    assert np.any(dxi[..., offdiag] != 0)  # the residue is there
    g = gpu_channel(o, dxi.copy(order="F"), capi.FP64)
    o.rk3_steps(5)
    g.time_integration_rk(5)
    s = g.download_state()
    g.close()
    _cmp(o, s, (im, jm, km))


def _wavy_case(n, amp=0.1, **kw):
    """Oracle on the periodic grid x = xi + a sin(eta) sin(zeta) (and
    cyclic), metrics by gridgeom, TGV fields at the physical coordinates."""
    from oracle import pyoracle as po
    L = 2.0 * np.pi
    xi = L / n * np.arange(n + 1)
    Xi, Et, Ze = np.meshgrid(xi, xi, xi, indexing="ij")
    X = Xi + amp * np.sin(Et) * np.sin(Ze)
    Y = Et + amp * np.sin(Xi) * np.sin(Ze)
    Z = Ze + amp * np.sin(Xi) * np.sin(Et)
    o = po.Oracle(n, n, n, mode=po.MODE_MAIN, **kw)
    x = o.field("x")
    sl = (slice(H, H + n + 1),) * 3
    x[sl + (0,)] = X
    x[sl + (1,)] = Y
    x[sl + (2,)] = Z
    o.call("gridgeom")
    c = cases.refcal(0.1, 1600.0)
    rho = np.ones_like(X)
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(X)
    p = c["pinf"] + rho / 16.0 * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0)
    T = p / rho * c["const2"]
    q5 = rho * (T * c["const1"] + 0.5 * (u * u + v * v + w * w))
    st = cases._pack_state(n, n, n, rho, u, v, w, p, T, q5)
    for name in ("q", "rho", "vel", "prs", "tmp"):
        o.field(name)[...] = st[name]
    return o


def _gpu_from(o, precision):
    from astr_gb300.solver import GpuSolver
    c = o.cfg
    g = GpuSolver(o.im, o.jm, o.km, precision=precision, mach=c.mach, reynolds=c.reynolds,
                  deltat=c.deltat)
    g.set_metrics(o.field("dxi").copy(order="F"), o.field("jacob").copy(order="F"))
    g.upload_state(o.field("q"), o.field("rho"), o.field("vel"), o.field("prs"), o.field("tmp"))
    return g


def test_curvilinear_fp64_matches_oracle(gpu_lib):
    n = 24
    o = _wavy_case(n, deltat=2e-3)
    dxi = o.field("dxi")
    assert np.abs(dxi[..., 1]).max() > 0.1 * np.abs(dxi[..., 0]).max()  # truly skewed
    g = _gpu_from(o, capi.FP64)
    hist_o = o.rk3_steps(3)
    hist_g = g.time_integration_rk(3)
    s = g.download_state()
    g.close()
    _cmp(o, s, (n, n, n))
    np.testing.assert_allclose(hist_g, hist_o, rtol=1e-12)


def test_curvilinear_fp32_storage(gpu_lib):
    n = 32
    o = _wavy_case(n, deltat=2e-3)
    outs = {}
    for name, prec in (("fp64", capi.FP64), ("fp32", capi.FP32_STORAGE)):
        g = _gpu_from(o, prec)
        g.time_integration_rk(10)
        outs[name] = g.download_state()
        g.close()
    sl = (slice(H, H + n + 1),) * 3
    a, b = outs["fp32"]["q"][sl], outs["fp64"]["q"][sl]
    e = float(np.linalg.norm(a[..., 1:4] - b[..., 1:4]) / np.linalg.norm(b[..., 1:4]))
    print(f"curvilinear 32^3, 10 steps: FP32-storage vs FP64 momentum rel L2 {e:.2e}")
    assert e <= 1e-5
