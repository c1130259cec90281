"""Boundary routines of boucon (src/bc.F90:327-409) in the oracle, on CPU:
the face values each routine sets (41 isothermal no-slip, 42 adiabatic
no-slip, 411 isothermal slip/no-slip wall, 421 adiabatic slip wall, 21
outflow, 51 farfield, 11 inflow, 23 gcnscbc, 50
zero-gradient extrapolation, 60 symmetry), and a closed box
stepping stably with walls on every face."""
import numpy as np
import pytest

from astr_gb300 import cases

H = 5
MACH = 0.3


def box_state(dims, lengths=(2.0 * np.pi, 2.0 * np.pi, 2.0 * np.pi), mach=MACH, vbulk=0.0):
    """TGV fields at Mach 0.3 on a box whose nodes include both ends of every
    direction (non-periodic layout), shifted by a quarter period so that the
    velocity does not vanish on the faces; vbulk is added to v."""
    im, jm, km = dims
    x, y, z = cases.gridcube(im, jm, km, *lengths)
    X = x.reshape(-1, 1, 1) + 0.7
    Y = y.reshape(1, -1, 1) + 0.4
    Z = z.reshape(1, 1, -1) + 0.3
    c = cases.refcal(mach, 1600.0)
    shape = (im + 1, jm + 1, km + 1)
    rho = (1.0 + 0.1 * np.sin(X) * np.cos(Y)) * np.ones(shape)
    u = np.sin(X) * np.cos(Y) * np.cos(Z) * np.ones(shape)
    v = vbulk - np.cos(X) * np.sin(Y) * np.cos(Z) * np.ones(shape)
    w = (0.2 * np.sin(Z) * np.cos(X) if km > 0 else 0.0) * np.ones(shape)
    p = c["pinf"] + 1.0 / 16.0 * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0)
    T = p / rho * c["const2"]
    q5 = rho * (T * c["const1"] + 0.5 * (u * u + v * v + w * w))
    return cases._pack_state(im, jm, km, rho, u, v, w, p, T, q5), (x, y, z)


def bc_oracle(dims, npdc, bctype, twall6=(0.0,) * 6, vbulk=0.0, **kw):
    from oracle import pyoracle as po
    st, grid = box_state(dims, vbulk=vbulk)
    kw.setdefault("mach", MACH)
    kw.setdefault("reynolds", 400.0)
    return po.from_state(st, dims, grid=grid, npdc=npdc, bctype=bctype, twall6=twall6, **kw)


def _face(a, n, l=0):
    """Face n at distance l from it, without its edges (edge nodes belong to
    two faces; the later face in boucon's order sets them)."""
    d, side = n // 2, n % 2
    dim = a.shape[d] - 2 * H - 1
    idx = [slice(H + 1, H + a.shape[m] - 2 * H - 1) for m in range(3)]
    idx[d] = H + (dim - l if side else l)
    return a[tuple(idx)]


def test_face_values():
    dims = (24, 20, 16)
    o = bc_oracle(dims, (4, 4, 4), (41, 42, 60, 50, 60, 41), twall6=(1.3, 0, 0, 0, 0, 0.9),
                  twall=1.0)
    before = {k: o.field(k).copy() for k in ("vel", "prs", "tmp", "rho")}
    o.call("boucon")
    vel, prs, tmp, rho, q = (o.field(k) for k in ("vel", "prs", "tmp", "rho", "q"))
    ex = lambda a, n: (4.0 * _face(a, n, 1) - _face(a, n, 2)) / 3.0
    # 41 on xmin (T_w 1.3) and zmax (0.9): u = 0, T = T_w, p extrapolated
    for n, tw in ((0, 1.3), (5, 0.9)):
        assert np.all(_face(vel, n) == 0.0) and np.all(_face(tmp, n) == tw)
        np.testing.assert_allclose(_face(prs, n), ex(before["prs"], n), rtol=1e-14)
    # 42 on xmax: p and T extrapolated, u = 0
    assert np.all(_face(vel, 1) == 0.0)
    np.testing.assert_allclose(_face(tmp, 1), ex(before["tmp"], 1), rtol=1e-14)
    # 60 on ymin: v = 0, u and w extrapolated; 60 on zmin: w = 0
    assert np.all(_face(vel[..., 1], 2) == 0.0)
    assert np.all(_face(vel[..., 2], 4) == 0.0)
    # 50 on ymax: every primitive extrapolated (T from p and the extrapolated rho)
    np.testing.assert_allclose(_face(vel, 3), ex(before["vel"], 3), rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(_face(rho, 3), ex(before["rho"], 3), rtol=1e-14)
    # q consistent with the primitives on every face
    for n in range(6):
        np.testing.assert_allclose(_face(q[..., 1], n), _face(rho, n) * _face(vel[..., 0], n), rtol=1e-14,
                                   atol=1e-15)
        e = _face(prs, n) * 2.5 + 0.5 * _face(rho, n) * (_face(vel, n) ** 2).sum(axis=-1)
        np.testing.assert_allclose(_face(q[..., 4], n), e, rtol=1e-12)


def test_slip_adiabatic_wall_face_values():
    """421 (slipadibwall, src/bc.F90:7231-7430) on both y faces: p, T and u
    extrapolated, w = 0; v = 0 on ymin and extrapolated on ymax, as the
    reference writes the two faces; rho from p and T."""
    o = bc_oracle((24, 20, 16), (3, 4, 3), (0, 0, 421, 421, 0, 0))
    before = {k: o.field(k).copy() for k in ("vel", "prs", "tmp")}
    o.call("boucon")
    vel, prs, tmp, rho, q = (o.field(k) for k in ("vel", "prs", "tmp", "rho", "q"))
    ex = lambda a, n: (4.0 * _face(a, n, 1) - _face(a, n, 2)) / 3.0
    const2 = cases.refcal(MACH, 400.0)["const2"]
    for n in (2, 3):
        np.testing.assert_allclose(_face(prs, n), ex(before["prs"], n), rtol=1e-14)
        np.testing.assert_allclose(_face(tmp, n), ex(before["tmp"], n), rtol=1e-14)
        np.testing.assert_allclose(_face(vel[..., 0], n), ex(before["vel"][..., 0], n), rtol=1e-13,
                                   atol=1e-14)
        assert np.all(_face(vel[..., 2], n) == 0.0)
        np.testing.assert_allclose(_face(rho, n), _face(prs, n) / _face(tmp, n) * const2,
                                   rtol=1e-14)
        e = _face(prs, n) * 2.5 + 0.5 * _face(rho, n) * (_face(vel, n) ** 2).sum(axis=-1)
        np.testing.assert_allclose(_face(q[..., 4], n), e, rtol=1e-12)
    assert np.all(_face(vel[..., 1], 2) == 0.0)
    np.testing.assert_allclose(_face(vel[..., 1], 3), ex(before["vel"][..., 1], 3), rtol=1e-13,
                               atol=1e-14)


def test_slip_isothermal_wall_face_values():
    """411 (slipisotwall, src/bc.F90:7038-7229) on both y faces: on ymin the
    nodes at x <= xslip slip (u and T extrapolated, v = w = 0), the others
    are isothermal no-slip walls; ymax is an isothermal no-slip wall; p
    extrapolated everywhere, rho from p and T."""
    o = bc_oracle((24, 20, 16), (3, 4, 3), (0, 0, 411, 411, 0, 0), twall6=(0, 0, 1.1, 0.9, 0, 0),
                  xslip=3.0)
    before = {k: o.field(k).copy() for k in ("vel", "prs", "tmp")}
    o.call("boucon")
    vel, prs, tmp, rho = (o.field(k) for k in ("vel", "prs", "tmp", "rho"))
    ex = lambda a, n: (4.0 * _face(a, n, 1) - _face(a, n, 2)) / 3.0
    const2 = cases.refcal(MACH, 400.0)["const2"]
    slip = _face(o.field("x")[..., 0], 2) <= 3.0
    assert 0.2 < slip.mean() < 0.8
    np.testing.assert_allclose(_face(tmp, 2)[slip], ex(before["tmp"], 2)[slip], rtol=1e-14)
    np.testing.assert_allclose(_face(vel[..., 0], 2)[slip], ex(before["vel"][..., 0], 2)[slip],
                               rtol=1e-13, atol=1e-14)
    assert np.all(_face(tmp, 2)[~slip] == 1.1) and np.all(_face(vel[..., 0], 2)[~slip] == 0.0)
    assert np.all(_face(vel[..., 1:], 2) == 0.0)
    assert np.all(_face(vel, 3) == 0.0) and np.all(_face(tmp, 3) == 0.9)
    for n in (2, 3):
        np.testing.assert_allclose(_face(prs, n), ex(before["prs"], n), rtol=1e-14)
        np.testing.assert_allclose(_face(rho, n), _face(prs, n) / _face(tmp, n) * const2, rtol=1e-15)


def test_outflow_face_values():
    """21 (outflow, src/bc.F90:3404-3617) on xmax and ymax.  xmax copies the
    i-1 node; ymax extrapolates where the face is supersonic (v >= sqrt(T)/M)
    and else relaxes p towards pinf, taking T extrapolated for rho and then
    T from p and rho.  A bulk v of 3.5 at Mach 0.3 puts both branches on the
    ymax face."""
    o = bc_oracle((24, 20, 16), (4, 4, 3), (0, 21, 0, 21, 0, 0), vbulk=3.5, deltat=2e-3)
    before = {k: o.field(k).copy() for k in ("vel", "prs", "tmp", "rho")}
    o.call("boucon")
    vel, prs, tmp, rho, q = (o.field(k) for k in ("vel", "prs", "tmp", "rho", "q"))
    c = cases.refcal(MACH, 400.0)
    const2, pinf = c["const2"], c["pinf"]
    # xmax: the i-1 node, all nodes of the face (edges included: ymax comes later)
    for f in ("vel", "prs", "tmp"):
        assert np.array_equal(_face(o.field(f), 1), _face(before[f], 1, 1))
    np.testing.assert_allclose(_face(rho, 1), _face(prs, 1) / _face(tmp, 1) * const2, rtol=1e-15)
    np.testing.assert_allclose(_face(q[..., 4], 1),
                               _face(rho, 1) * (_face(tmp, 1) * c["const1"] +
                                                0.5 * (_face(vel, 1) ** 2).sum(axis=-1)), rtol=1e-14)
    # ymax
    ex = lambda a: (4.0 * _face(a, 3, 1) - _face(a, 3, 2)) / 3.0
    vf, tf, pf, rf = (_face(before[k], 3) for k in ("vel", "tmp", "prs", "rho"))
    vf = vf[..., 1]
    css = np.sqrt(tf) / MACH
    sup = vf >= css
    assert 0.1 < sup.mean() < 0.9, sup.mean()
    np.testing.assert_allclose(_face(vel, 3), ex(before["vel"]), rtol=1e-13, atol=1e-14)
    adt = 0.25 * 2e-3
    p_sub = (pf + adt * pinf + rf * css * (ex(before["vel"])[..., 1] - vf)) / (1.0 + adt)
    p_exp = np.where(sup, ex(before["prs"]), p_sub)
    r_exp = np.where(sup, ex(before["rho"]), p_sub / ex(before["tmp"]) * const2)
    np.testing.assert_allclose(_face(prs, 3), p_exp, rtol=1e-14)
    np.testing.assert_allclose(_face(rho, 3), r_exp, rtol=1e-14)
    np.testing.assert_allclose(_face(tmp, 3), p_exp / r_exp * const2, rtol=1e-14)
    e = _face(prs, 3) * 2.5 + 0.5 * _face(rho, 3) * (_face(vel, 3) ** 2).sum(axis=-1)
    np.testing.assert_allclose(_face(q[..., 4], 3), e, rtol=1e-12)


def test_farfield_face_values():
    """51 (farfield, src/bc.F90:3008-3392) on the y and z faces.  ymax is
    extrapolated (its characteristic treatment is commented out); ymin, zmin
    and zmax take the free stream through the Riemann invariants where the
    normal velocity points into the domain, else pinf with the outgoing
    invariant.  The TGV box has both signs of v on ymin and of w on the z
    faces."""
    o = bc_oracle((24, 20, 16), (4, 4, 4), (0, 0, 51, 51, 51, 51), deltat=2e-3)
    before = {k: o.field(k).copy() for k in ("vel", "prs", "tmp", "rho")}
    o.call("boucon")
    vel, prs, tmp, rho, q = (o.field(k) for k in ("vel", "prs", "tmp", "rho", "q"))
    c = cases.refcal(MACH, 400.0)
    const2, pinf = c["const2"], c["pinf"]
    # ymax: extrapolated, T from p and rho, q with temperature
    ex = lambda a, n: (4.0 * _face(a, n, 1) - _face(a, n, 2)) / 3.0
    for f in ("vel", "prs", "rho"):
        np.testing.assert_allclose(_face(o.field(f), 3), ex(before[f], 3), rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(_face(tmp, 3), _face(prs, 3) / _face(rho, 3) * const2, rtol=1e-15)
    for n, m in ((2, 1), (4, 2), (5, 2)):
        sgn = -1.0 if n % 2 else 1.0
        vf = _face(before["vel"], n)[..., m]
        inflow = sgn * vf >= 0.0
        assert 0.1 < inflow.mean() < 0.9, (n, inflow.mean())
        css = np.sqrt(_face(before["tmp"], n)) / MACH
        rf = _face(before["rho"], n)
        vne, pe, roe = ex(before["vel"], n)[..., m], ex(before["prs"], n), ex(before["rho"], n)
        csse = (4.0 * np.sqrt(_face(before["tmp"], n, 1)) / MACH -
                np.sqrt(_face(before["tmp"], n, 2)) / MACH) / 3.0
        p_in = 0.5 * (pinf + pe) - sgn * 0.5 * rf * css * vne
        vn_in = sgn * 0.5 * (pinf - pe) / (rf * css) + 0.5 * vne
        p_exp = np.where(inflow, p_in, pinf)
        r_exp = np.where(inflow, (p_in / pinf) ** (1.0 / 1.4), roe + (pinf - pe) / csse ** 2)
        vn_exp = np.where(inflow, vn_in, vne - sgn * (pe - pinf) / roe / csse)
        np.testing.assert_allclose(_face(prs, n), p_exp, rtol=1e-14)
        np.testing.assert_allclose(_face(rho, n), r_exp, rtol=1e-13)
        np.testing.assert_allclose(_face(vel, n)[..., m], vn_exp, rtol=1e-12, atol=1e-14)
        assert np.all(_face(vel, n)[..., 0][inflow] == 1.0)
        np.testing.assert_allclose(_face(tmp, n), p_exp / r_exp * const2, rtol=1e-13)
        e = _face(prs, n) * 2.5 + 0.5 * _face(rho, n) * (_face(vel, n) ** 2).sum(axis=-1)
        np.testing.assert_allclose(_face(q[..., 4], n), e, rtol=1e-12)


def test_closed_box_steps():
    """A 2-D box with walls on all four faces (isothermal, adiabatic and a
    symmetry plane) and the viscous terms steps stably."""
    o = bc_oracle((32, 24, 0), (4, 4, 3), (41, 42, 41, 60, 0, 0), twall=1.0, deltat=2e-3,
                  lfilter=True)
    o.rk3_steps(10)
    q = o.field("q")
    assert np.isfinite(q).all()
    # boucon runs at the start of each stage: apply it to see the faces
    o.call("boucon")
    vel = o.field("vel")
    assert np.all(_face(vel, 0) == 0.0) and np.all(_face(vel, 1) == 0.0)
    assert np.all(_face(vel[..., 1], 3) == 0.0)


def _inflow_profile(o):
    """A non-uniform inflow (vel_in, tmp_in, tmp_prof) in the oracle's
    arrays, returned as copies."""
    f = o.inflow()
    nj, nk = f["tmp_in"].shape
    J = np.arange(nj).reshape(-1, 1) * (2 * np.pi / (nj - 1))
    K = np.arange(nk).reshape(1, -1) * (2 * np.pi / max(nk - 1, 1))
    f["vel_in"][..., 0] = 1.0 + 0.1 * np.sin(J) * np.cos(K)
    f["vel_in"][..., 1] = 0.05 * np.cos(K) * np.ones_like(J)
    f["vel_in"][..., 2] = 0.02 * np.sin(J + K)
    f["tmp_in"][...] = 1.0 + 0.05 * np.sin(J + 0.3) * np.ones_like(K)
    f["tmp_prof"][...] = 1.0 + 0.03 * np.cos(np.arange(nj) * 0.4)
    return {k: v.copy() for k, v in f.items()}


@pytest.mark.parametrize("profile", [False, True])
def test_inflow_face_values(profile):
    """11 (inflow, src/bc.F90:1366-1562) on xmin: v, w, T from the inflow
    arrays; p from the incoming characteristic against pinf, blended towards
    pinf by tanh of the inflow Mach number (speed of sound of the profile
    temperature); u = u_in + (pinf - p)/(rho_1 css); rho from p and T; q in
    temperature form.  Freestream arrays (u 1, T 1) or a profile."""
    o = bc_oracle((24, 20, 16), (4, 3, 3), (11, 21, 0, 0, 0, 0), deltat=2e-3)
    if profile:
        f = _inflow_profile(o)
    else:
        f = {k: v.copy() for k, v in o.inflow().items()}
        assert np.all(f["vel_in"][..., 0] == 1.0) and np.all(f["vel_in"][..., 1:] == 0.0)
        assert np.all(f["tmp_in"] == 1.0) and np.all(f["tmp_prof"] == 1.0)
    before = {k: o.field(k).copy() for k in ("vel", "prs", "tmp", "rho")}
    o.call("boucon")
    c = cases.refcal(MACH, 400.0)
    const1, const2, pinf = c["const1"], c["const2"], c["pinf"]
    sl0 = (H, slice(H, H + o.jm + 1), slice(H, H + o.km + 1))
    sl1 = (H + 1,) + sl0[1:]
    sl2 = (H + 2,) + sl0[1:]
    ex = lambda a: (4.0 * a[sl1] - a[sl2]) / 3.0
    vin = f["vel_in"]
    css = (np.sqrt(f["tmp_prof"]) / MACH).reshape(-1, 1)
    rho_ref = before["rho"][sl1]
    pe, ue = ex(before["prs"]), ex(before["vel"][..., 0])
    blend = 0.5 * (np.tanh((vin[..., 0] / css - 1.0) * 6.0) + 1.0)
    p = (0.5 * (pinf + pe) + 0.5 * rho_ref * css * (vin[..., 0] - ue)) * (1.0 - blend) + pinf * blend
    vel, prs, tmp, rho, q = (o.field(k) for k in ("vel", "prs", "tmp", "rho", "q"))
    np.testing.assert_allclose(prs[sl0], p, rtol=1e-14)
    np.testing.assert_allclose(vel[sl0 + (0,)], vin[..., 0] + (pinf - p) / rho_ref / css, rtol=1e-14)
    assert np.array_equal(vel[sl0 + (1,)], vin[..., 1]) and np.array_equal(vel[sl0 + (2,)], vin[..., 2])
    assert np.array_equal(tmp[sl0], f["tmp_in"])
    np.testing.assert_allclose(rho[sl0], p / f["tmp_in"] * const2, rtol=1e-15)
    e = rho[sl0] * (tmp[sl0] * const1 + 0.5 * (vel[sl0] ** 2).sum(axis=-1))
    np.testing.assert_allclose(q[sl0 + (4,)], e, rtol=1e-14)
    assert blend.max() < 1e-3  # subsonic inflow: the characteristic branch dominates


def _gcnscbc_expected(before, x, n, mach, pinf, const2, extent):
    """gcnscbc (src/bc.F90:8024-8254) on face n (1 xmax, 3 ymax) restated in
    numpy from the state before the call, with the reference's INTEGER css,
    css2 and vnorm (truncated; mavg an integer division; lambda(5) = vnorm
    since lambda(5:numq) = vnorm follows lambda(5) = vnorm + css)."""
    d = n // 2
    on, ot = d, 1 - d
    f1 = lambda a: _face(a, n, 1)
    f2 = lambda a: _face(a, n, 2)
    r1, t1, p1 = f1(before["rho"]), f1(before["tmp"]), f1(before["prs"])
    v1, v2 = f1(before["vel"]), f2(before["vel"])
    css = np.trunc(np.sqrt(t1) / mach).astype(np.int64)
    css2 = css * css
    vnorm = np.trunc(v1[..., on]).astype(np.int64)
    mavg = np.trunc(vnorm / css).astype(np.float64)
    lam = [(vnorm - css) + 1e-10] + [vnorm + 1e-10] * 4
    dx = f1(x[..., d]) - f2(x[..., d])
    dr = lambda a, b: -(-a + b) / dx
    dvel = [dr(v1[..., m], v2[..., m]) for m in range(3)]
    dprs = dr(p1, f2(before["prs"]))
    drho = dr(r1, f2(before["rho"]))
    lodi = [lam[0] * (dprs - r1 * css * dvel[on]), lam[1] * (css2 * drho - dprs), lam[2] * dvel[ot],
            lam[3] * dvel[2], lam[4] * (dprs + r1 * css * dvel[on])]
    soft = 0.25 * css * (1.0 - mavg * mavg) / extent * (p1 - pinf)
    if d == 0:
        lodi[0] = soft
    else:
        eta, inflow = 0.25, vnorm < 0
        lodi[0] = np.where(inflow, eta * r1 * css2 * (1.0 - mavg * mavg) / extent * v1[..., 1], soft)
        lodi[1] = np.where(inflow, eta * r1 * css2 / 1.4 / extent * (t1 - 1.0), lodi[1])
        lodi[2] = np.where(inflow, eta * css / extent * (v1[..., 0] - 1.0), lodi[2])
        lodi[3] = np.where(inflow, eta * css / extent * v1[..., 2], lodi[3])
    lodi = [lodi[m] / lam[m] for m in range(5)]
    dtmp = t1 / r1 / css * (-lodi[1] + 0.5 * (1.4 - 1.0) * (lodi[0] + lodi[4]))
    dprs = 0.5 * (lodi[0] + lodi[4])
    dv = [None] * 3
    dv[on] = 1.0 / (2.0 * r1 * css) * (lodi[4] - lodi[0])
    dv[ot], dv[2] = lodi[2], lodi[3]
    t = t1 + 2.0 * dx * dtmp
    p = p1 + 2.0 * dx * dprs
    vel = np.stack([v1[..., m] + 2.0 * dx * dv[m] for m in range(3)], axis=-1)
    return {"tmp": t, "prs": p, "vel": vel, "rho": p / t * const2}


def test_gcnscbc_face_values():
    """23 (gcnscbc) on xmax and ymax against a numpy restatement; a bulk v
    of -1 puts both of ymax's branches (vnorm >= 0: soft outflow towards
    pinf; vnorm < 0: the waves relaxed towards the free stream) on the
    face."""
    o = bc_oracle((24, 20, 16), (4, 4, 3), (41, 23, 42, 23, 0, 0), twall6=(1.2, 0, 0, 0, 0, 0),
                  vbulk=-1.0, deltat=2e-3)
    before = {k: o.field(k).copy() for k in ("vel", "prs", "tmp", "rho")}
    x = o.field("x").copy()
    o.call("boucon")
    c = cases.refcal(MACH, 400.0)
    extent = 2.0 * np.pi
    vnorm_y = np.trunc(_face(before["vel"], 3, 1)[..., 1])
    assert 0.05 < (vnorm_y < 0).mean() < 0.95
    for n in (1, 3):
        want = _gcnscbc_expected(before, x, n, MACH, c["pinf"], c["const2"], extent)
        for k in ("prs", "tmp", "rho"):
            np.testing.assert_allclose(_face(o.field(k), n), want[k], rtol=1e-13, err_msg=(n, k))
        np.testing.assert_allclose(_face(o.field("vel"), n), want["vel"], rtol=1e-12, atol=1e-13)
        q, rho, vel, prs = (o.field(k) for k in ("q", "rho", "vel", "prs"))
        e = _face(prs, n) * 2.5 + 0.5 * _face(rho, n) * (_face(vel, n) ** 2).sum(axis=-1)
        np.testing.assert_allclose(_face(q[..., 4], n), e, rtol=1e-12)


def _pmatrix(rho, u, v, w, t, ddi, inv, mach):
    """pmatrix (src/bc.F90:5516-5611) on arrays: shape (..., 5, 5)."""
    g = 1.4
    c = np.sqrt(t) / mach
    var1 = 1.0 / np.sqrt(ddi[0] ** 2 + ddi[1] ** 2 + ddi[2] ** 2)
    nx, ny, nz = ddi[0] * var1, ddi[1] * var1, ddi[2] * var1
    phi = 0.5 * (g - 1.0) * (u * u + v * v + w * w)
    VV = nx * u + ny * v + nz * w
    a1, a2, a3 = g - 1.0, 1.0 / (np.sqrt(2.0) * rho * c), rho / (c * np.sqrt(2.0))
    a4, a5, a6 = (phi + c * c) / (g - 1.0), 1.0 - phi / (c * c), phi / (g - 1.0)
    c2 = c * c
    if inv:
        rows = [[nx * a5 - (nz * v - ny * w) / rho, nx * a1 * u / c2, nx * a1 * v / c2 + nz / rho,
                 nx * a1 * w / c2 - ny / rho, -nx * a1 / c2],
                [ny * a5 - (nx * w - nz * u) / rho, ny * a1 * u / c2 - nz / rho, ny * a1 * v / c2,
                 ny * a1 * w / c2 + nx / rho, -ny * a1 / c2],
                [nz * a5 - (ny * u - nx * v) / rho, nz * a1 * u / c2 + ny / rho, nz * a1 * v / c2 - nx / rho,
                 nz * a1 * w / c2, -nz * a1 / c2],
                [a2 * (phi - c * VV), -a2 * (a1 * u - nx * c), -a2 * (a1 * v - ny * c),
                 -a2 * (a1 * w - nz * c), a1 * a2],
                [a2 * (phi + c * VV), -a2 * (a1 * u + nx * c), -a2 * (a1 * v + ny * c),
                 -a2 * (a1 * w + nz * c), a1 * a2]]
    else:
        rows = [[nx, ny, nz, a3, a3],
                [nx * u, ny * u - nz * rho, nz * u + ny * rho, a3 * (u + nx * c), a3 * (u - nx * c)],
                [nx * v + nz * rho, ny * v, nz * v - nx * rho, a3 * (v + ny * c), a3 * (v - ny * c)],
                [nx * w - ny * rho, ny * w + nx * rho, nz * w, a3 * (w + nz * c), a3 * (w - nz * c)],
                [nx * a6 + rho * (nz * v - ny * w), ny * a6 + rho * (nx * w - nz * u),
                 nz * a6 + rho * (ny * u - nx * v), a3 * (a4 + c * VV), a3 * (a4 - c * VV)]]
    return np.stack([np.stack([np.broadcast_to(x, np.shape(rho)) for x in r], -1) for r in rows], -2)


def _row_flux(o, sl, d):
    """J (q u_d + dxi(d,:) p) at the halo-array slice sl (inflow_nscbc's Ecs / fcs)."""
    X = o.field("dxi")[sl]
    x = [X[..., d + 3 * m] for m in range(3)]
    V, Q = o.field("vel")[sl], o.field("q")[sl]
    J, p = o.field("jacob")[sl], o.field("prs")[sl]
    uu = x[0] * V[..., 0] + x[1] * V[..., 1] + x[2] * V[..., 2]
    return np.stack([J * Q[..., 0] * uu, J * (Q[..., 1] * uu + x[0] * p), J * (Q[..., 2] * uu + x[1] * p),
                     J * (Q[..., 3] * uu + x[2] * p), J * (Q[..., 4] + p) * uu], -1)


def _inflow_nscbc_expected(o, mach, extent):
    """inflow_nscbc (src/bc.F90:2114-2344) in numpy: the residual added at
    i = 0 (periodic y and z), shape (jm+1, km+1, 5)."""
    jm, km = o.jm, o.km
    inner = (slice(H, H + o.im + 1), slice(H, H + jm + 1), slice(H, H + km + 1))
    V, T = o.field("vel")[inner], o.field("tmp")[inner]
    gm2 = ((V[..., 0] ** 2 + V[..., 1] ** 2 + V[..., 2] ** 2) / (np.sqrt(T) / mach) / (np.sqrt(T) / mach)).max()
    f0 = (H, slice(H, H + jm + 1), slice(H, H + km + 1))
    f1 = (H + 1,) + f0[1:]
    rho, vel, t, pr, J = (o.field(k)[f0] for k in ("rho", "vel", "tmp", "prs", "jacob"))
    Q, X = o.field("q")[f0], o.field("dxi")[f0]
    u, v, w = vel[..., 0], vel[..., 1], vel[..., 2]
    ddi = [X[..., 0], X[..., 3], X[..., 6]]
    pnor, pinv = (_pmatrix(rho, u, v, w, t, ddi, inv, mach) for inv in (False, True))
    dE = -_row_flux(o, f0, 0) + _row_flux(o, f1, 0)
    E = np.stack([Q[..., 1], Q[..., 1] * u + pr, Q[..., 2] * u, Q[..., 3] * u, (Q[..., 4] + pr) * u], -1)
    F = np.stack([Q[..., 2], Q[..., 1] * v, Q[..., 2] * v + pr, Q[..., 3] * v, (Q[..., 4] + pr) * v], -1)
    G = np.stack([Q[..., 3], Q[..., 1] * w, Q[..., 2] * w, Q[..., 3] * w + pr, (Q[..., 4] + pr) * w], -1)
    Xa, Ja = o.field("dxi")[f1], o.field("jacob")[f1]
    jcbi = [-(X[..., 3 * m] * J) + Xa[..., 3 * m] * Ja for m in range(3)]
    rest = E * jcbi[0][..., None] + F * jcbi[1][..., None] + G * jcbi[2][..., None]
    lodi = np.einsum("...rc,...c->...r", pinv, dE - rest) / J[..., None]
    css = np.sqrt(t) / mach
    kin = 0.25 * (1.0 - gm2) * css / extent
    var1 = 1.0 / np.sqrt(ddi[0] ** 2 + ddi[1] ** 2 + ddi[2] ** 2)
    f = o.inflow()
    ui, vi, wi = f["vel_in"][..., 0], f["vel_in"][..., 1], f["vel_in"][..., 2]
    lodi[..., 0] = 0.0
    lodi[..., 1] = kin * 0.5 * (ddi[0] * var1 * (w - wi) - ddi[2] * var1 * (u - ui))
    lodi[..., 2] = kin * 0.5 * (-ddi[0] * var1 * (v - vi) + ddi[1] * var1 * (u - ui))
    lodi[..., 3] = kin * (ddi[0] * var1 * (u - ui) + ddi[1] * var1 * (v - vi) + ddi[2] * var1 * (w - wi) +
                          (pr - f["prs_in"]) / rho / css)
    out = np.einsum("...rc,...c->...r", pnor, lodi) * J[..., None] + rest
    ym = (H, slice(H - 1, H + jm), slice(H, H + km + 1))
    yp = (H, slice(H + 1, H + jm + 2), slice(H, H + km + 1))
    out = out + 0.5 * (_row_flux(o, yp, 1) - _row_flux(o, ym, 1))
    if km > 0:
        zm = (H, slice(H, H + jm + 1), slice(H - 1, H + km))
        zp = (H, slice(H, H + jm + 1), slice(H + 1, H + km + 2))
        out = out + 0.5 * (_row_flux(o, zp, 2) - _row_flux(o, zm, 2))
    return out


@pytest.mark.parametrize("profile", [False, True])
def test_inflow_nscbc_residual(profile):
    """12 (inflow_nscbc) on xmin, y and z periodic: boucon adds to qrhs at
    i = 0 the LODI residual and the face's tangential flux derivatives;
    against a numpy restatement (pmatrix, the one-sided normal flux
    difference, the relaxation of the incoming waves towards the inflow
    arrays at the rate kin of the domain-wide Mach number)."""
    o = bc_oracle((24, 20, 16), (4, 3, 3), (12, 21, 0, 0, 0, 0), deltat=2e-3)
    if profile:
        _inflow_profile(o)
        f = o.inflow()
        f["prs_in"][...] = cases.refcal(MACH, 400.0)["pinf"] * (1.0 + 0.02 * f["tmp_in"])
    before = o.field("q").copy()
    o.call("boucon")
    assert np.array_equal(o.field("q")[H], before[H])  # the face's state is not touched
    want = _inflow_nscbc_expected(o, MACH, 2.0 * np.pi)
    got = o.field("qrhs")[0]
    scale = np.abs(want).max(axis=(0, 1))
    np.testing.assert_allclose(got / scale, want / scale, rtol=0, atol=1e-13)
    assert np.all(o.field("qrhs")[1:] == 0.0)


def test_pmatrix_inverse_pair():
    """pmatrix's two forms (src/bc.F90:5516-5611) are inverse to each other
    for any state and metric row (the check the reference leaves commented
    out as Pmult = MatMul(Pinv, pnor)): the restated entries hold."""
    rng = np.random.default_rng(7)
    n = 64
    rho = 0.5 + rng.random(n)
    u, v, w = (rng.standard_normal(n) for _ in range(3))
    t = 0.5 + rng.random(n)
    ddi = [rng.standard_normal(n) for _ in range(3)]
    pnor = _pmatrix(rho, u, v, w, t, ddi, False, MACH)
    pinv = _pmatrix(rho, u, v, w, t, ddi, True, MACH)
    eye = np.broadcast_to(np.eye(5), pnor.shape)
    np.testing.assert_allclose(pinv @ pnor, eye, atol=1e-12)
    np.testing.assert_allclose(pnor @ pinv, eye, atol=1e-12)
