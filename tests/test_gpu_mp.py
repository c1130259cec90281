"""Compact MP convective scheme (conschm 543c) on the GPU against the oracle
(FP64, 1e-12): a Sod tube with physical x ends and a density that varies in
y, with and without the characteristic decomposition; a periodic 3-D case
with a pressure jump and the viscous terms; a skewed curvilinear grid with
the filter on; the rhscal drop-in; and the Sod solution against the exact
Riemann solution."""
import numpy as np
import pytest

from astr_gb300 import capi, cases

pytestmark = pytest.mark.gpu
H = 5
TOL = 1e-12


def _gpu_from(o):
    from astr_gb300.solver import GpuSolver
    c = o.cfg
    g = GpuSolver(o.im, o.jm, o.km, npdc=(c.npdci, c.npdcj, c.npdck), mach=c.mach,
                  reynolds=c.reynolds, deltat=c.deltat, lfilter=bool(c.lfilter),
                  diffterm=bool(c.diffterm), conschm="543c", lchardecomp=bool(c.lchardecomp),
                  bfacmpld=c.bfacmpld, shkcrt=c.shkcrt)
    g.set_metrics(o.field("dxi").copy(order="F"), o.field("jacob").copy(order="F"))
    g.upload_state(o.field("q"), o.field("rho"), o.field("vel"), o.field("prs"), o.field("tmp"))
    return g


def _cmp(o, s, tol=TOL):
    im, jm, km = o.im, o.jm, o.km
    sl = (slice(H, H + im + 1), slice(H, H + jm + 1), slice(H, H + km + 1))
    qo = o.field("q")[sl]
    mom = np.abs(qo[..., 1:4]).max()  # momentum components against the vector's scale
    errs = {}
    for m in range(5):
        ref = qo[..., m]
        scale = mom if 1 <= m <= 3 else np.abs(ref).max()
        errs[f"q{m + 1}"] = float(np.abs(s["q"][sl + (m,)] - ref).max() / scale)
    for name in ("prs", "tmp", "rho"):
        ref = o.field(name)[sl]
        errs[name] = float(np.abs(s[name][sl] - ref).max() / np.abs(ref).max())
    print(" ".join(f"{k} {v:.1e}" for k, v in errs.items()))
    assert max(errs.values()) <= tol, errs


def _zero_offdiag(o):
    D = o.field("dxi")
    for d in range(3):
        for m in range(3):
            if d != m:
                D[..., d + 3 * m] = 0.0


def _sod(im, jm, dt, amp, **kw):
    from oracle import pyoracle as po
    st = cases.shock_tube_state("sod", im, jm, amp=amp)
    o = po.from_state(st, (im, jm, 0), grid=cases.grid1d(im, jm), npdc=(4, 3, 3), mach=3.0,
                      conschm="543c", lfilter=False, diffterm=False, deltat=dt, **kw)
    _zero_offdiag(o)
    return o


@pytest.mark.parametrize("chard", [True, False])
def test_mp_sod_matches_oracle(gpu_lib, chard):
    o = _sod(96, 12, 0.01, 0.1, lchardecomp=chard)
    g = _gpu_from(o)
    o.rk3_steps(25)
    g.time_integration_rk(25)
    s = g.download_state()
    g.close()
    if chard:
        ls = o.lshock()
        assert ls.any() and not ls.all()  # both limiter branches are taken
    _cmp(o, s)


def _jump3d(n, mach=0.3, **kw):
    """The periodic shock box: TGV fields at Mach 0.3 with the pressure
    raised by half in z < pi (two plane discontinuities)."""
    from oracle import pyoracle as po
    L = 2.0 * np.pi
    st = cases.shock_box_state(n, mach=mach, jump=0.5)
    o = po.from_state(st, (n, n, n), lx=L, ly=L, lz=L, mach=mach, conschm="543c", **kw)
    _zero_offdiag(o)
    return o


def test_mp_periodic_3d_viscous_matches_oracle(gpu_lib):
    o = _jump3d(24, lfilter=False, diffterm=True, reynolds=400.0, deltat=2e-3)
    g = _gpu_from(o)
    hist_o = o.rk3_steps(4)
    hist_g = g.time_integration_rk(4)
    s = g.download_state()
    g.close()
    ls = o.lshock()
    assert ls.any() and not ls.all()
    _cmp(o, s)
    np.testing.assert_allclose(hist_g, hist_o, rtol=1e-11)


def _skew_case(n, amp=0.15, mach=0.3, **kw):
    """Oracle on the periodic skewed grid x = xi + a sin(eta) sin(zeta),
    y = eta + a sin(zeta), z = zeta (metrics by gridgeom: every off-diagonal
    but d(eta)/dx, d(zeta)/dx, d(zeta)/dy is nonzero), TGV fields at the
    physical coordinates.  chardecomp picks its eigenvector branch by the
    first metric component of the interface above 1e-12 in magnitude
    (src/solver.F90:2058-2130) and divides by it; on this grid that component
    is O(1) at every interface and for all three branches, whereas a grid
    where it passes near zero (above the threshold) makes the eigenvector
    pair ill-conditioned, with rounding noise of order eps/|g| in any
    arithmetic, the reference's included."""
    from oracle import pyoracle as po
    L = 2.0 * np.pi
    xi = L / n * np.arange(n + 1)
    Xi, Et, Ze = np.meshgrid(xi, xi, xi, indexing="ij")
    X = Xi + amp * np.sin(Et) * np.sin(Ze)
    Y = Et + amp * np.sin(Ze)
    Z = Ze
    o = po.Oracle(n, n, n, mode=po.MODE_MAIN, mach=mach, conschm="543c", **kw)
    x = o.field("x")
    sl = (slice(H, H + n + 1),) * 3
    x[sl + (0,)] = X
    x[sl + (1,)] = Y
    x[sl + (2,)] = Z
    o.call("gridgeom")
    c = cases.refcal(mach, 1600.0)
    rho = 1.0 + 0.2 * (np.cos(X) * np.cos(Z) > 0.3)  # density jumps for the limiter
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(X)
    p = c["pinf"] + 1.0 / 16.0 * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0)
    T = p / rho * c["const2"]
    q5 = rho * (T * c["const1"] + 0.5 * (u * u + v * v + w * w))
    st = cases._pack_state(n, n, n, rho, u, v, w, p, T, q5)
    for name in ("q", "rho", "vel", "prs", "tmp"):
        o.field(name)[...] = st[name]
    return o


@pytest.mark.parametrize("chard", [True, False])
def test_mp_curvilinear_filtered_matches_oracle(gpu_lib, chard):
    # without the characteristic decomposition the MP5 limiter acts at
    # every interface (no sensor)
    o = _skew_case(16, deltat=2e-3, lfilter=True, lchardecomp=chard)
    D = o.field("dxi")
    assert np.abs(D[..., 0 + 3 * 1]).max() > 0.1  # d(xi)/dy: truly skewed
    g = _gpu_from(o)
    o.rk3_steps(3)
    g.time_integration_rk(3)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_mp_rhscal_dropin(gpu_lib):
    o = _sod(64, 10, 0.01, 0.1)
    g = _gpu_from(o)
    o.rk3_steps(5)
    g.time_integration_rk(5)
    for x in (o,):
        x.call("qswap")
        x.call("gradcal")
    g.qswap()
    g.gradcal()
    o.field("qrhs")[...] = 0.0
    o.call("rhscal")
    g.rhscal()
    r = g.download_rhs()
    g.close()
    ref = o.field("qrhs")
    for m in range(5):
        scale = max(np.abs(ref[..., m]).max(), np.abs(ref[..., 1:4]).max() if 1 <= m <= 3 else 0.0)
        if scale == 0.0:
            assert np.all(r["qrhs"][..., m] == 0.0)
            continue
        e = np.abs(r["qrhs"][..., m] - ref[..., m]).max() / scale
        assert e <= TOL, (m, e)


def test_mp_sod_exact_solution(gpu_lib):
    from astr_gb300.solver import GpuSolver
    im, jm, dt, t_end = 400, 8, 0.004, 1.5
    st = cases.shock_tube_state("sod", im, jm)
    x, y, z = cases.grid1d(im, jm)
    dxi, J = cases.rect_metrics(x, y, z, npdc=(4, 3, 3))
    g = GpuSolver(im, jm, 0, npdc=(4, 3, 3), mach=3.0, deltat=dt, lfilter=False,
                  diffterm=False, conschm="543c")
    g.set_metrics(dxi, J)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    g.time_integration_rk(int(round(t_end / dt)))
    s = g.download_state()
    g.close()
    rho = s["rho"][H:H + im + 1, H:H + jm + 1, H]
    assert np.max(np.abs(rho - rho[:, :1])) < 1e-12
    re, _, _ = cases.riemann_exact((1.0, 0.0, 1.0), (0.125, 0.0, 0.1), x, t_end)
    l1 = float(np.mean(np.abs(rho[:, 0] - re)))
    print(f"Sod 400 points, t = 1.5: density L1 error {l1:.2e}")
    assert l1 < 3e-3
    assert rho.min() > 0.125 * 0.98 and rho.max() < 1.02


def test_mp_needs_fp64_main_order(gpu_lib):
    from astr_gb300.solver import GpuSolver
    with pytest.raises(capi.AstrError) as e:
        GpuSolver(16, 16, 16, precision=capi.FP32_STORAGE, conschm="543c")
    assert e.value.code == capi.ASTR_ERR_UNSUPPORTED


def test_mp_graph_steps_match_plain_steps(gpu_lib):
    """The compact MP step captured as a CUDA graph (astr_gpu_step_async):
    the flagged-interface count lives on the device, so the replayed steps
    are the plain steps."""
    o = _sod(96, 12, 0.01, 0.1)
    out = []
    for graph in (False, True):
        g = _gpu_from(o)
        if graph:
            g.step_async(6)
            while not g.poll():
                pass
        else:
            g.time_integration_rk(6, stats=False)
        out.append(g.download_state()["q"])
        g.close()
    assert np.array_equal(out[0], out[1])


def test_mp_with_walls_matches_oracle(gpu_lib):
    """The compact MP scheme with boundary routines: a 2-D box with
    adiabatic no-slip x-walls and symmetry y-planes, the viscous terms and a
    pressure jump in x (a shock running between the walls)."""
    from oracle import pyoracle as po
    from test_bc import box_state
    im, jm = 64, 32
    st, grid = box_state((im, jm, 0))
    sl = (slice(H, H + im + 1), slice(H, H + jm + 1), H)
    x = grid[0]
    st["prs"][sl] *= (1.0 + 0.8 * (x < np.pi)).reshape(-1, 1)
    c = cases.refcal(0.3, 1600.0)
    rho, p = st["rho"][sl], st["prs"][sl]
    u, v = st["vel"][sl + (0,)], st["vel"][sl + (1,)]
    st["tmp"][sl] = p / rho * c["const2"]
    st["q"][sl + (4,)] = rho * (st["tmp"][sl] * c["const1"] + 0.5 * (u * u + v * v))
    o = po.from_state(st, (im, jm, 0), grid=grid, npdc=(4, 4, 3), mach=0.3, reynolds=400.0,
                      deltat=2e-3, conschm="543c", lfilter=False, bctype=(42, 42, 60, 60, 0, 0))
    _zero_offdiag(o)
    from astr_gb300.solver import GpuSolver
    g = GpuSolver(im, jm, 0, npdc=(4, 4, 3), mach=0.3, reynolds=400.0, deltat=2e-3,
                  lfilter=False, conschm="543c", bctype=(42, 42, 60, 60, 0, 0))
    g.set_metrics(o.field("dxi").copy(order="F"), o.field("jacob").copy(order="F"))
    g.upload_state(o.field("q"), o.field("rho"), o.field("vel"), o.field("prs"), o.field("tmp"))
    o.rk3_steps(8)
    g.time_integration_rk(8)
    s = g.download_state()
    g.close()
    ls = o.lshock()
    assert ls.any() and not ls.all()
    _cmp(o, s)
