"""Boundary routines of boucon on the GPU against the oracle (FP64, 1e-12):
a 3-D box with a different routine on each face (isothermal and adiabatic
no-slip, symmetry, zero-gradient extrapolation), slip walls (isothermal with
a slip region, adiabatic) on the y faces, outflow on xmax and ymax, farfield on the y and z faces, the
viscous terms and the
filter; a skewed curvilinear box where the symmetry faces project on the
metric normal; inflow on xmin (freestream and a profile) with outflow on
xmax; inflow_nscbc on xmin (its residual and steps); gcnscbc on xmax and
ymax; and the FP32-storage form against FP64."""
import numpy as np
import pytest

from astr_gb300 import capi, cases
from test_bc import H, MACH, bc_oracle

pytestmark = pytest.mark.gpu


def _gpu_from(o, precision=capi.FP64, **kw):
    from astr_gb300.solver import GpuSolver
    c = o.cfg
    g = GpuSolver(o.im, o.jm, o.km, precision=precision, npdc=(c.npdci, c.npdcj, c.npdck),
                  mach=c.mach, reynolds=c.reynolds, deltat=c.deltat, lfilter=bool(c.lfilter),
                  diffterm=bool(c.diffterm), twall=c.twall, bctype=tuple(c.bctype),
                  twall_face=tuple(c.twall6), **kw)
    g.set_metrics(o.field("dxi").copy(order="F"), o.field("jacob").copy(order="F"))
    g.upload_state(o.field("q"), o.field("rho"), o.field("vel"), o.field("prs"), o.field("tmp"))
    return g


def _cmp(o, s, tol=1e-12):
    sl = (slice(H, H + o.im + 1), slice(H, H + o.jm + 1), slice(H, H + o.km + 1))
    qo = o.field("q")[sl]
    mom = np.abs(qo[..., 1:4]).max()
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


def _mixed_box():
    return bc_oracle((24, 20, 16), (4, 4, 4), (41, 42, 60, 50, 60, 41),
                     twall6=(1.3, 0, 0, 0, 0, 0.9), twall=1.0, deltat=2e-3, lfilter=True)


def test_mixed_faces_match_oracle(gpu_lib):
    o = _mixed_box()
    g = _gpu_from(o)
    o.rk3_steps(4)
    g.time_integration_rk(4)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_slip_adiabatic_walls_match_oracle(gpu_lib):
    """421 on both y faces (ymax keeps the extrapolated v), isothermal and
    adiabatic no-slip on the x faces, z periodic."""
    o = bc_oracle((24, 20, 16), (4, 4, 3), (41, 42, 421, 421, 0, 0), twall6=(1.2, 0, 0, 0, 0, 0),
                  deltat=2e-3, lfilter=True)
    g = _gpu_from(o)
    o.rk3_steps(4)
    g.time_integration_rk(4)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_slip_isothermal_walls_match_oracle(gpu_lib):
    """411 on both y faces: ymin slips up to x = xslip (the node mask comes
    from the grid, astr_gpu_set_grid), isothermal no-slip beyond and on
    ymax; stepping refuses to start before the grid is set."""
    o = bc_oracle((24, 20, 16), (4, 4, 3), (41, 42, 411, 411, 0, 0),
                  twall6=(1.2, 0, 1.1, 0.9, 0, 0), xslip=3.0, deltat=2e-3, lfilter=True)
    g = _gpu_from(o, xslip=3.0)
    with pytest.raises(capi.AstrError, match="grid not set"):
        g.time_integration_rk(1)
    g.set_grid(o.field("x").copy(order="F"))
    o.rk3_steps(4)
    g.time_integration_rk(4)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_outflow_faces_match_oracle(gpu_lib):
    """21 on xmax (the i-1 copy) and ymax (supersonic extrapolation or the
    subsonic pressure relaxation: a bulk v of 3.5 at Mach 0.3 puts both on
    the face), walls on xmin and ymin, z periodic."""
    o = bc_oracle((24, 20, 16), (4, 4, 3), (41, 21, 42, 21, 0, 0), twall6=(1.2, 0, 0, 0, 0, 0),
                  vbulk=3.5, deltat=2e-3, lfilter=True)
    g = _gpu_from(o)
    o.rk3_steps(3)
    g.time_integration_rk(3)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_outflow_only_matches_oracle(gpu_lib):
    """Outflow faces as the only boundary routines (xmin and ymin without
    one): boucon still runs."""
    o = bc_oracle((24, 20, 16), (4, 4, 3), (0, 21, 0, 21, 0, 0), vbulk=3.5, deltat=2e-3,
                  lfilter=True)
    g = _gpu_from(o)
    o.rk3_steps(2)
    g.time_integration_rk(2)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_farfield_faces_match_oracle(gpu_lib):
    """51 on the y and z faces (both the inflow and the outflow branch on
    ymin, zmin and zmax), walls on the x faces."""
    o = bc_oracle((24, 20, 16), (4, 4, 4), (41, 42, 51, 51, 51, 51), twall6=(1.2, 0, 0, 0, 0, 0),
                  deltat=2e-3, lfilter=True)
    g = _gpu_from(o)
    o.rk3_steps(3)
    g.time_integration_rk(3)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_skewed_symmetry_faces_match_oracle(gpu_lib):
    from oracle import pyoracle as po
    from test_bc import box_state
    n = 16
    L = 2.0 * np.pi
    st, _ = box_state((n, n, n))
    xi = L / n * np.arange(n + 1)
    Xi, Et, Ze = np.meshgrid(xi, xi, xi, indexing="ij")
    o = po.Oracle(n, n, n, npdc=(4, 3, 4), bctype=(60, 60, 0, 0, 50, 60), mach=MACH,
                  reynolds=400.0, deltat=2e-3)
    x = o.field("x")
    sl = (slice(H, H + n + 1),) * 3
    x[sl + (0,)] = Xi + 0.15 * np.sin(Et) * np.sin(Ze)
    x[sl + (1,)] = Et + 0.15 * np.sin(Ze)
    x[sl + (2,)] = Ze
    o.call("gridgeom")
    for name in ("q", "rho", "vel", "prs", "tmp"):
        o.field(name)[...] = st[name]
    D = o.field("dxi")
    assert np.abs(D[..., 0 + 3 * 1]).max() > 0.1  # x faces: the metric row is skewed
    g = _gpu_from(o)
    o.rk3_steps(3)
    g.time_integration_rk(3)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_mixed_faces_fp32_storage(gpu_lib):
    o = _mixed_box()
    out = {}
    for name, prec in (("fp64", capi.FP64), ("fp32", capi.FP32_STORAGE)):
        g = _gpu_from(o, prec)
        g.time_integration_rk(10)
        out[name] = g.download_state()
        g.close()
    sl = (slice(H, H + o.im + 1), slice(H, H + o.jm + 1), slice(H, H + o.km + 1))
    a, b = out["fp32"]["q"][sl], out["fp64"]["q"][sl]
    e = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    print(f"mixed faces, 10 steps: FP32-storage vs FP64 rel L2 {e:.2e}")
    assert e <= 1e-5


def test_boundary_routine_checks(gpu_lib):
    from astr_gb300.solver import GpuSolver
    with pytest.raises(capi.AstrError):   # a routine on a periodic direction
        GpuSolver(16, 16, 16, bctype=(41, 0, 0, 0, 0, 0))
    with pytest.raises(capi.AstrError):   # adiabatic no-slip exists for x and y faces only
        GpuSolver(16, 16, 16, npdc=(3, 3, 4), bctype=(0, 0, 0, 0, 42, 0))
    with pytest.raises(capi.AstrError):   # not built (outflow_nscbc)
        GpuSolver(16, 16, 16, npdc=(4, 3, 3), bctype=(22, 21, 0, 0, 0, 0))


@pytest.mark.parametrize("profile", [False, True])
def test_inflow_outflow_match_oracle(gpu_lib, profile):
    """11 on xmin (freestream arrays, or a profile through
    astr_gpu_set_inflow), 21 on xmax, y and z periodic, viscous with the
    filter."""
    from test_bc import _inflow_profile
    o = bc_oracle((24, 20, 16), (4, 3, 3), (11, 21, 0, 0, 0, 0), deltat=2e-3, lfilter=True)
    g = _gpu_from(o)
    if profile:
        f = _inflow_profile(o)
        g.set_inflow(f["vel_in"], f["tmp_in"], f["tmp_prof"], f["prs_in"])
    o.rk3_steps(4)
    g.time_integration_rk(4)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_inflow_arguments(gpu_lib):
    """bctype 11 exists on xmin only; set_inflow needs an inflow face and
    positive temperatures."""
    from astr_gb300.solver import GpuSolver
    with pytest.raises(capi.AstrError, match="xmin"):
        GpuSolver(16, 16, 16, npdc=(4, 4, 3), bctype=(0, 0, 11, 0, 0, 0))
    g = GpuSolver(16, 16, 16, npdc=(4, 3, 3), bctype=(11, 21, 0, 0, 0, 0))
    with pytest.raises(capi.AstrError, match="> 0"):
        g.set_inflow(tmp_prof=np.zeros(17))
    g.close()
    g = GpuSolver(16, 16, 16)
    with pytest.raises(capi.AstrError, match="no inflow face"):
        g.set_inflow()
    g.close()


def _gcnscbc_box():
    return bc_oracle((24, 20, 16), (4, 4, 3), (41, 23, 42, 23, 0, 0), twall6=(1.2, 0, 0, 0, 0, 0),
                     vbulk=-1.0, deltat=2e-3, lfilter=True)


def test_gcnscbc_routine_matches_oracle(gpu_lib):
    """23 (gcnscbc) on xmax and ymax (both of ymax's branches on the face),
    walls on xmin and ymin: one boucon call on the same state, every face
    value ≤1e-14; the face routine needs the grid first."""
    o = _gcnscbc_box()
    g = _gpu_from(o)
    with pytest.raises(capi.AstrError, match="grid not set"):
        g.time_integration_rk(1)
    g.set_grid(o.field("x").copy(order="F"))
    o.call("boucon")
    g.boucon()
    s = g.download_state()
    g.close()
    _cmp(o, s, tol=1e-14)


def test_gcnscbc_steps_match_oracle(gpu_lib):
    """Three steps of the same box.  The routine builds the face from
    one-sided differences of the first interior nodes, which magnify the
    rounding differences of the interior by |v| / |v(dim-1) - v(dim-2)|, so
    the bar is 5e-12 here (measured 1.8e-12) against 1e-12 elsewhere."""
    o = _gcnscbc_box()
    g = _gpu_from(o)
    g.set_grid(o.field("x").copy(order="F"))
    o.rk3_steps(3)
    g.time_integration_rk(3)
    s = g.download_state()
    g.close()
    _cmp(o, s, tol=5e-12)


def _nscbc_box(profile):
    from test_bc import _inflow_profile
    o = bc_oracle((24, 20, 16), (4, 3, 3), (12, 21, 0, 0, 0, 0), deltat=2e-3, lfilter=True)
    f = None
    if profile:
        _inflow_profile(o)
        f = o.inflow()
        f["prs_in"][...] = cases.refcal(MACH, 400.0)["pinf"] * (1.0 + 0.02 * f["tmp_in"])
        f = {k: v.copy() for k, v in f.items()}
    return o, f


def _nscbc_gpu(o, f):
    g = _gpu_from(o)
    with pytest.raises(capi.AstrError, match="grid not set"):
        g.time_integration_rk(1)
    g.set_grid(o.field("x").copy(order="F"))
    if f is not None:
        g.set_inflow(f["vel_in"], f["tmp_in"], f["tmp_prof"], f["prs_in"])
    return g


def test_inflow_nscbc_residual_matches_oracle(gpu_lib):
    """12 (inflow_nscbc) on xmin, outflow on xmax, y and z periodic: the
    routine chain boucon, qswap, gradcal, rhscal gives the oracle's residual
    (the routine's LODI and tangential terms at i = 0 added under rhscal's
    negation), every node."""
    o, f = _nscbc_box(True)
    g = _nscbc_gpu(o, f)
    for name in ("boucon", "qswap", "gradcal", "rhscal"):
        o.call(name)
        getattr(g, name)()
    r = g.download_rhs()["qrhs"]
    g.close()
    ro = o.field("qrhs")
    for m in range(5):
        scale = np.abs(ro[..., m]).max()
        err = np.abs(r[..., m] - ro[..., m]).max() / scale
        face = np.abs(r[0, ..., m] - ro[0, ..., m]).max() / np.abs(ro[0, ..., m]).max()
        print(f"q{m + 1}: {err:.1e} (face {face:.1e})")
        assert err <= 1e-12 and face <= 1e-12


@pytest.mark.parametrize("profile", [False, True])
def test_inflow_nscbc_steps_match_oracle(gpu_lib, profile):
    o, f = _nscbc_box(profile)
    g = _nscbc_gpu(o, f)
    o.rk3_steps(4)
    g.time_integration_rk(4)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_inflow_nscbc_fp32_storage_against_fp64(gpu_lib):
    """The FP32-storage form with inflow_nscbc (profile) against FP64, 10
    steps: relative L2 ≤1e-5 (measured ≤4.7e-7)."""
    o, f = _nscbc_box(True)
    out = {}
    for name, prec in (("fp64", capi.FP64), ("fp32", capi.FP32_STORAGE)):
        g = _gpu_from(o, precision=prec)
        g.set_grid(o.field("x").copy(order="F"))
        g.set_inflow(f["vel_in"], f["tmp_in"], f["tmp_prof"], f["prs_in"])
        g.time_integration_rk(10)
        out[name] = g.download_state()["q"]
        g.close()
    sl = (slice(H, H + o.im + 1), slice(H, H + o.jm + 1), slice(H, H + o.km + 1))
    a, b = out["fp32"][sl], out["fp64"][sl]
    for m in range(5):
        e = np.linalg.norm(a[..., m] - b[..., m]) / np.linalg.norm(b[..., m])
        assert e <= 1e-5, (m, e)
