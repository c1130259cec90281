"""Host-side set-up of the configurations the hot path is measured on.

Grid metrics and initial states are inputs of the hot path: a Fortran host
passes its own (``astr_gpu_set_metrics``); the benchmark and the serving loop
build them here.  ``rect_metrics`` restates ``gridgeom`` (src/geom.F90:
99-930) for rectilinear grids, x = x(i), y = y(j), z = z(k), with the same
floating-point operations in the same order: arrays are held with singleton
axes where a field is constant, and numpy broadcasting applies the
reference's element-wise arithmetic.  The compact derivative along an axis
is ``fd_scheme_initiate`` + ``df_compact`` (src/derivative.F90:63-306) with
the Thomas recurrences of src/commfunc.F90:752-813, vectorised over lines.
"""
from __future__ import annotations

import numpy as np

HM = 5
PI = 4.0 * np.arctan(1.0)
NUM1D3 = 1.0 / 3.0
NUM7D9 = 7.0 / 9.0
NUM1D36 = 1.0 / 36.0
NUM1D60 = 1.0 / 60.0


# ---------------------------------------------------------------------------
# compact first derivative along one axis (arrays hold halo nodes -5..dim+5)
# ---------------------------------------------------------------------------
def _scheme(ntype: int, dim: int):
    """fd_scheme_initiate ('643c') + tridiagonal_thomas_proprocess."""
    i0, imx = (0, dim) if ntype == 4 else (-1, dim + 1)
    n = imx - i0 + 1
    a = np.full(n, NUM1D3)
    c = np.full(n, NUM1D3)
    a[0] = c[0] = 0.0
    a[-1] = c[-1] = 0.0
    if ntype == 4:
        a[0] = c[0] = 2.0
        a[1] = c[1] = 0.25
        a[-1] = c[-1] = 2.0
        a[-2] = c[-2] = 0.25
    ac1 = np.zeros(n)
    ac2 = np.zeros(n)
    ac3 = np.zeros(n)
    ac1[0] = c[0]
    for i in range(1, n):
        ac1[i] = c[i] / (1.0 - a[i] * ac1[i - 1])
        ac2[i] = 1.0 / (1.0 - a[i] * ac1[i - 1])
        ac3[i] = a[i] / (1.0 - a[i] * ac1[i - 1])
    return i0, n, ac1, ac2, ac3


def compact_deriv(f: np.ndarray, axis: int, ntype: int, dim: int) -> np.ndarray:
    """Index-space derivative of f along `axis` (length dim+11, halo first)
    at nodes 0..dim, exactly as df_compact (src/derivative.F90:171-306)."""
    f = np.moveaxis(np.asarray(f, dtype=np.float64), axis, 0)
    i0, n, ac1, ac2, ac3 = _scheme(ntype, dim)

    def F(j):  # node j -> array slab
        return f[j + HM]

    d = np.empty((n,) + f.shape[1:])
    rows = range(n)
    for r in rows:
        j = i0 + r
        if ntype == 4 and r == 0:
            d[r] = -2.5 * F(j) + 2.0 * F(j + 1) + 0.5 * F(j + 2)
        elif ntype == 4 and (r == 1 or r == n - 2):
            d[r] = 0.75 * (F(j + 1) - F(j - 1))
        elif ntype == 4 and r == n - 1:
            d[r] = 2.5 * F(j) - 2.0 * F(j - 1) - 0.5 * F(j - 2)
        elif ntype != 4 and (r == 0 or r == n - 1):
            d[r] = 0.75 * (F(j + 1) - F(j - 1)) - 0.15 * (F(j + 2) - F(j - 2)) + \
                NUM1D60 * (F(j + 3) - F(j - 3))
        else:
            d[r] = NUM7D9 * (F(j + 1) - F(j - 1)) + NUM1D36 * (F(j + 2) - F(j - 2))
    for i in range(1, n):
        d[i] = d[i] * ac2[i] - d[i - 1] * ac3[i]
    x = np.empty_like(d)
    x[n - 1] = d[n - 1]
    for i in range(n - 2, -1, -1):
        x[i] = d[i] - ac1[i] * x[i + 1]
    out = x[-i0: -i0 + dim + 1]
    return np.moveaxis(out, 0, axis)


# ---------------------------------------------------------------------------
# grids
# ---------------------------------------------------------------------------
def gridcube(ia, ja, ka, lx, ly, lz):
    """gridcube (src/gridgeneration.F90:233-267), single rank: 1-D node
    coordinates x(0:ia), y(0:ja), z(0:ka)."""
    x = np.array([lx / float(ia) * float(i) for i in range(ia + 1)])
    y = np.array([ly] if ja == 0 else [ly / float(ja) * float(j) for j in range(ja + 1)])
    z = np.array([0.0] if ka == 0 else [lz / float(ka) * float(k) for k in range(ka + 1)])
    return x, y, z


def _extend(c: np.ndarray, dim: int, flat: bool) -> np.ndarray:
    """gridsendrecv single-rank halo extension (src/parallel.F90:2861-2866,
    2930-2960, 3010-3030): nodes -5..dim+5."""
    h = np.zeros(dim + 2 * HM + 1)
    if flat:
        for n in range(-HM, HM + 1):
            h[n + HM] = c[0] + float(n)
        return h
    h[HM:HM + dim + 1] = c
    for n in range(1, HM + 1):
        h[dim + n + HM] = c[dim] + (c[n] - c[0])
        h[-n + HM] = c[0] - (c[dim] - c[dim - n])
    return h


def grid_halo(x, y, z):
    """x(-hm:..,1:3) in the halo layout (Fortran order) for rectilinear node
    vectors, halos filled as gridsendrecv does on one rank
    (src/parallel.F90:2861-2866, 2930-2960, 3010-3030)."""
    im, jm, km = len(x) - 1, len(y) - 1, len(z) - 1
    X = _extend(x, im, False).reshape(-1, 1, 1)
    Y = _extend(y, jm, jm == 0).reshape(1, -1, 1)
    Z = _extend(z, km, km == 0).reshape(1, 1, -1)
    full = (im + 2 * HM + 1, jm + 2 * HM + 1, km + 2 * HM + 1)
    out = np.zeros(full + (3,), order="F")
    out[..., 0] = np.broadcast_to(X, full)
    out[..., 1] = np.broadcast_to(Y, full)
    out[..., 2] = np.broadcast_to(Z, full)
    return out


def _wrap_halo(a: np.ndarray, dims, per) -> np.ndarray:
    """dataswap of an interior-valued array onto halo layout: periodic axes
    copy im-5..im-1 / 1..5 into the halos; other halos are zero."""
    out = a
    for ax in range(3):
        n = out.shape[ax]
        if n == 1:
            continue
        dim = dims[ax]
        if per[ax]:
            idx = np.concatenate([np.arange(dim - HM, dim), np.arange(0, dim + 1), np.arange(1, HM + 1)])
            out = np.take(out, idx, axis=ax)
        else:
            pad = [(0, 0)] * out.ndim
            pad[ax] = (HM, HM)
            out = np.pad(out, pad)
    return out


def rect_metrics(x, y, z, npdc=(3, 3, 3), diag_only=False):
    """gridgeom (src/geom.F90:99-930) for a rectilinear grid.

    Returns (dxi, jacob) in the halo layout: dxi shape (im+11, jm+11, km+11,
    3, 3) in Fortran order (or a tuple of the three diagonal components when
    diag_only and every off-diagonal is zero), jacob (im+11, jm+11, km+11).
    """
    im, jm, km = len(x) - 1, len(y) - 1, len(z) - 1
    ndims = 3 if km > 0 else 2
    per = [p == 3 for p in npdc]
    dims = (im, jm, km)
    # coordinates with halos, broadcast along the axes they do not vary on
    X = [
        _extend(x, im, False).reshape(-1, 1, 1),
        _extend(y, jm, jm == 0).reshape(1, -1, 1),
        _extend(z, km, km == 0).reshape(1, 1, -1),
    ]
    full = (im + 2 * HM + 1, jm + 2 * HM + 1, km + 2 * HM + 1)

    def D(f, axis):
        """fds%central along `axis` for every transverse line: f holds nodes
        -5..dim+5 along `axis` (or is constant there: singleton axis) and
        interior nodes (or a singleton) on the other axes."""
        f = np.asarray(f, dtype=np.float64)
        if f.shape[axis] == 1:
            if npdc[axis] == 3:
                # every row of a periodic system differences equal values
                return np.zeros(f.shape)
            f = np.broadcast_to(f, tuple(full[axis] if a == axis else f.shape[a] for a in range(3)))
        return compact_deriv(f, axis, npdc[axis], dims[axis])

    def transverse_interior(a, axis):
        sl = [slice(HM, HM + dims[b] + 1) if (b != axis and a.shape[b] > 1) else slice(None)
              for b in range(3)]
        return a[tuple(sl)]

    # dx(m,d): derivative of coordinate m along d on interior lines, then dataswap
    dxm = [[None] * 3 for _ in range(3)]
    for d in range(3):
        for m in range(3):
            dxm[m][d] = D(transverse_interior(X[m], d), d)
    dxh = [[_wrap_halo(dxm[m][d], dims, per) for d in range(3)] for m in range(3)]

    def A(m, d):  # dx(m,d) on interior nodes, 1-based indices
        return dxm[m - 1][d - 1]

    if ndims == 3:
        J = (A(1, 1) * A(2, 2) * A(3, 3) + A(1, 2) * A(2, 3) * A(3, 1) +
             A(1, 3) * A(2, 1) * A(3, 2) - A(1, 3) * A(2, 2) * A(3, 1) -
             A(1, 2) * A(2, 1) * A(3, 3) - A(1, 1) * A(2, 3) * A(3, 2))
    else:
        J = A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)
    J = np.broadcast_to(J, (im + 1, jm + 1, km + 1))

    dxi = [[0.0] * 3 for _ in range(3)]  # dxi[d][m], 0-based
    if ndims == 3:
        def Xh(m):
            return X[m - 1]

        def DXh(m, d):
            return dxh[m - 1][d - 1]

        terms = {
            0: [(2, 1, 2, 3, 3, 3, 3, 2), (2, 2, 3, 3, 1, 1, 3, 3), (2, 3, 1, 3, 2, 2, 3, 1),
                (3, 1, 3, 2, 2, 2, 2, 3), (3, 2, 1, 2, 3, 3, 2, 1), (3, 3, 2, 2, 1, 1, 2, 2)],
            1: [(1, 1, 3, 3, 2, 2, 3, 3), (1, 2, 1, 3, 3, 3, 3, 1), (1, 3, 2, 3, 1, 1, 3, 2),
                (3, 1, 2, 1, 3, 3, 1, 2), (3, 2, 3, 1, 1, 1, 1, 3), (3, 3, 1, 1, 2, 2, 1, 1)],
            2: [(1, 1, 2, 2, 3, 3, 2, 2), (1, 2, 3, 2, 1, 1, 2, 3), (1, 3, 1, 2, 2, 2, 2, 1),
                (2, 1, 3, 1, 2, 2, 1, 3), (2, 2, 1, 1, 3, 3, 1, 1), (2, 3, 2, 1, 1, 1, 1, 2)],
        }
        for s in range(3):
            for (dd, mm, am, ad, bm, cm, cd, dm) in terms[s]:
                # phi over nodes -hm..dim+hm of lines at interior transverse nodes
                phi = 0.5 * (DXh(am, ad) * Xh(bm) - DXh(cm, cd) * Xh(dm))
                dxi[dd - 1][mm - 1] = dxi[dd - 1][mm - 1] + D(transverse_interior(phi, s), s)
    else:
        dxi[0][0] = A(2, 2)
        dxi[0][1] = -A(1, 2)
        dxi[1][0] = -A(2, 1)
        dxi[1][1] = A(1, 1)
    out = [[None] * 3 for _ in range(3)]
    for d in range(3):
        for m in range(3):
            v = np.asarray(dxi[d][m], dtype=np.float64)
            if not np.any(v):
                out[d][m] = np.zeros((1, 1, 1))  # 0/J is exactly 0
            else:
                out[d][m] = np.broadcast_to(v, (im + 1, jm + 1, km + 1)) / J
    def to_halo(a):
        return np.asfortranarray(np.broadcast_to(_wrap_halo(np.ascontiguousarray(a), dims, per), full))

    Jh = to_halo(J)
    offdiag_zero = all(not np.any(out[d][m]) for d in range(3) for m in range(3) if d != m)
    if diag_only and offdiag_zero:
        diag = tuple(to_halo(out[d][d]) for d in range(3))
        return diag, Jh
    dxi_h = np.zeros(full + (3, 3), order="F")
    for d in range(3):
        for m in range(3):
            dxi_h[..., d, m] = _wrap_halo(np.ascontiguousarray(out[d][m]), dims, per)
    return dxi_h, Jh


# ---------------------------------------------------------------------------
# initial states
# ---------------------------------------------------------------------------
def refcal(mach, reynolds, prandtl=0.72, gamma=1.4):
    """Nondimensional constants of refcal (src/solver.F90:102-128)."""
    c = {}
    c["const1"] = 1.0 / (gamma * (gamma - 1.0) * (mach * mach))
    c["const2"] = gamma * (mach * mach)
    c["const6"] = 1.0 / (gamma - 1.0)
    c["pinf"] = 1.0 * 1.0 / c["const2"]
    return c


def cfl_deltat(st, dxi_diag, mach, cfl=0.5, im=None, jm=None, km=None):
    """Time step at a given CFL number, as cflcal (src/commcal.F90:27-87)
    measures it: CFL = dt * (Di + Dj + Dk), D the largest contravariant
    velocity plus sound speed along each computational direction over the
    interior nodes, sos = sqrt(T)/mach (nondimensional, src/fludyna.F90:
    832-859).  Diagonal metrics: dxi_diag = (dxi11, dxi22, dxi33)."""
    q = st["q"]
    im = q.shape[0] - 2 * HM - 1 if im is None else im
    jm = q.shape[1] - 2 * HM - 1 if jm is None else jm
    km = q.shape[2] - 2 * HM - 1 if km is None else km
    sl = (slice(HM, HM + im + 1), slice(HM, HM + jm + 1), slice(HM, HM + km + 1))
    css = np.sqrt(st["tmp"][sl]) / mach
    total = 0.0
    for d in range(3 if km > 0 else 2):
        x = np.asarray(dxi_diag[d])[sl]
        ubar = x * st["vel"][sl + (d,)]
        cs = css * np.abs(x)
        total += max(0.0, float(np.max(ubar + cs)))
    return cfl / total


def tgv_state(im, jm, km, mach=0.1, x=None, y=None, z=None):
    """tgvini + updateq (src/initialisation.F90:621-691, src/fludyna.F90:
    254-300): halo-layout q, rho, vel, prs, tmp with interior nodes set."""
    c = refcal(mach, 1600.0)
    if x is None:
        L = 2.0 * PI
        x, y, z = gridcube(im, jm, km, L, L, L)
    X = x.reshape(-1, 1, 1)
    Y = y.reshape(1, -1, 1)
    Z = z.reshape(1, 1, -1)
    rho = np.ones((im + 1, jm + 1, km + 1))
    u = 1.0 * np.sin(X) * np.cos(Y) * np.cos(Z) * np.ones_like(rho)
    v = -(1.0 * np.cos(X) * np.sin(Y) * np.cos(Z)) * np.ones_like(rho)
    w = np.zeros_like(rho)
    p = c["pinf"] + rho / 16.0 * (1.0 * 1.0) * (np.cos(2.0 * X) + np.cos(2.0 * Y)) * (np.cos(2.0 * Z) + 2.0)
    T = p / rho * c["const2"]
    q5 = rho * (T * c["const1"] + 0.5 * (u * u + v * v + w * w))
    return _pack_state(im, jm, km, rho, u, v, w, p, T, q5)


def vortex_fields(x, y, t=0.0, beta=5.0, gamma=1.4, half=5.0, uinf=(1.0, 1.0), mach=None):
    """Isentropic vortex of strength beta (Shu, NASA/CR-97-206253 / ICASE
    97-65, 1997, sec. 4.3.5; Yee, Sandham & Djomehri, JCP 150, 1999): on the
    periodic box [-half, half)^2 with freestream (u, v) = uinf, rho = p = T =
    1 far away, the exact solution at time t is the initial vortex advected
    to centre uinf * t (nearest periodic image):
        du, dv = beta/(2 pi) exp((1 - r^2)/2) (-ybar, xbar)
        dT = -(gamma - 1) beta^2 / (8 gamma pi^2) exp(1 - r^2)
        rho = T^(1/(gamma-1)),  p = rho T.
    In ASTR's nondimensional variables with mach = 1/sqrt(gamma), p_inf =
    1/(gamma mach^2) = 1 and T = p/rho * gamma mach^2 = p/rho, so these are
    the solver's own rho, u, v, p, T.  For another reference Mach number M
    (same velocity scale, T_inf = 1, p_inf = 1/(gamma M^2)) the radial
    momentum balance of the isentropic vortex gives dT = -(gamma - 1) M^2
    beta^2 / (8 pi^2) exp(1 - r^2), rho = T^(1/(gamma-1)), p = rho T /
    (gamma M^2); M = 1/sqrt(gamma) is the form above."""
    L = 2.0 * half
    X = np.asarray(x).reshape(-1, 1)
    Y = np.asarray(y).reshape(1, -1)
    xb = np.mod(X - uinf[0] * t + half, L) - half
    yb = np.mod(Y - uinf[1] * t + half, L) - half
    r2 = xb * xb + yb * yb
    e = np.exp(0.5 * (1.0 - r2))
    u = uinf[0] - beta / (2.0 * PI) * e * yb
    v = uinf[1] + beta / (2.0 * PI) * e * xb
    if mach is None:
        T = 1.0 - (gamma - 1.0) * beta * beta / (8.0 * gamma * PI * PI) * e * e
        rho = T ** (1.0 / (gamma - 1.0))
        p = rho * T
    else:
        T = 1.0 - (gamma - 1.0) * mach * mach * beta * beta / (8.0 * PI * PI) * e * e
        rho = T ** (1.0 / (gamma - 1.0))
        p = rho * T / (gamma * mach * mach)
    return rho, u, v, p, T


def vortex_grid(n, half=5.0):
    """gridcube-style nodes of the 2-D periodic box [-half, half]: x(0:n),
    y(0:n), z = 0 (a 2-D case has km = 0)."""
    x, y, z = gridcube(n, n, 0, 2.0 * half, 2.0 * half, 0.0)
    return x - half, y - half, z


def vortex_state(n, t=0.0, beta=5.0, gamma=1.4, half=5.0, mach=None):
    """Halo-layout state (q, rho, vel, prs, tmp; km = 0) of the isentropic
    vortex on the n^2 grid at time t, with interior nodes set; mach None is
    the classic form (mach = 1/sqrt(gamma))."""
    x, y, _ = vortex_grid(n, half)
    rho, u, v, p, T = vortex_fields(x, y, t, beta, gamma, half, mach=mach)
    if mach is None:
        mach = 1.0 / np.sqrt(gamma)
    c = refcal(mach, 1.0, gamma=gamma)
    rho3, u3, v3 = (a[:, :, None] for a in (rho, u, v))
    p3, T3 = p[:, :, None], T[:, :, None]
    w3 = np.zeros_like(rho3)
    q5 = rho3 * (T3 * c["const1"] + 0.5 * (u3 * u3 + v3 * v3))
    return _pack_state(n, n, 0, rho3, u3, v3, w3, p3, T3, q5)


def channel_grid(ia, ja, ka, lx=2.0 * PI, ly=2.0, lz=PI, stretch=2.0, varc=None):
    """Channel nodes: x and z uniform (grichan, src/gridgeneration.F90:
    272-340, box 2 pi x 2 x pi with ref_len = 1), y on [0, ly] clustered at
    both walls.  Default: y = ly/2 (1 + tanh(s (2j/ja - 1)) / tanh s) with
    stretch s; varc given: grichan's own y = ly/2 (1 + varc tanh(atanh(1/varc)
    (2j/ja - 1)))."""
    x = np.array([lx / float(ia) * float(i) for i in range(ia + 1)])
    eta = np.array([2.0 * float(j) / float(ja) - 1.0 for j in range(ja + 1)])
    if varc is None:
        y = 0.5 * ly * (1.0 + np.tanh(stretch * eta) / np.tanh(stretch))
    else:
        y = 0.5 * ly * (1.0 + varc * np.tanh(np.arctanh(1.0 / varc) * eta))
    y[0], y[-1] = 0.0, ly
    z = np.array([0.0] if ka == 0 else [lz / float(ka) * float(k) for k in range(ka + 1)])
    return x, y, z


def splitmix64_uniform(seed, counter):
    """Counter-based uniform numbers in [0, 1): the splitmix64 output
    function (Steele, Lea & Flood, OOPSLA 2014) applied to seed + (counter
    + 1) * golden gamma; 53 high bits.  Vectorised over integer counters, so
    a node's numbers do not depend on the grid traversal order."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (np.asarray(counter, dtype=np.uint64) + np.uint64(1)) * \
            np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def channel_state(ia, ja, ka, y, mach=0.5, prandtl=0.72, gamma=1.4, seed=20261203, amp=0.05):
    """Channel initial state (after chanini, src/initialisation.F90:749-1001,
    ref_len = 1): laminar profile U = 1.5 (1 - (y-1)^2), T = 1 + (gamma-1)
    Pr M^2/3 * 1.5 (1 - (y-1)^4), rho = 1, p = rho T / (gamma M^2), plus a
    uniform random velocity perturbation of relative size amp on all three
    components, u' = amp U r, r in [-1, 1) from splitmix64 with the given
    seed and counter 3*(i + (ia+1)(j + (ja+1) k)) + component (the
    reference draws its perturbation from Fortran's random_number)."""
    c = refcal(mach, 1.0, prandtl, gamma)
    shape = (ia + 1, ja + 1, ka + 1)
    Y = np.asarray(y).reshape(1, -1, 1)
    U = 1.5 * (1.0 - (Y - 1.0) ** 2) * np.ones(shape)
    node = np.arange(int(np.prod(shape)), dtype=np.uint64).reshape(shape, order="F")
    r = [2.0 * splitmix64_uniform(seed, np.uint64(3) * node + np.uint64(m)) - 1.0 for m in range(3)]
    u = U * (1.0 + amp * r[0])
    v = amp * U * r[1]
    w = amp * U * r[2] if ka > 0 else np.zeros(shape)
    T = (1.0 + (gamma - 1.0) * prandtl * mach ** 2 / 3.0 * 1.5 * (1.0 - (Y - 1.0) ** 4)) * np.ones(shape)
    rho = np.ones(shape)
    p = rho * T / c["const2"]
    q5 = rho * (T * c["const1"] + 0.5 * (u * u + v * v + w * w))
    return _pack_state(ia, ja, ka, rho, u, v, w, p, T, q5)


def shock_box_state(n, mach=0.3, jump=0.5):
    """Periodic 3-D shock box for the compact MP scheme: the TGV fields of
    tgvini at the given Mach number with the pressure raised by the factor
    1 + jump in z < pi, so that two plane pressure jumps steepen into shocks
    and rarefactions inside the vortex field (T = p/rho gamma M^2)."""
    L = 2.0 * PI
    x, y, z = gridcube(n, n, n, L, L, L)
    st = tgv_state(n, n, n, mach=mach, x=x, y=y, z=z)
    c = refcal(mach, 1600.0)
    sl = (slice(HM, HM + n + 1),) * 3
    rho = st["rho"][sl]
    u, v, w = (st["vel"][sl + (m,)] for m in range(3))
    p = st["prs"][sl] * (1.0 + jump * (z.reshape(1, 1, -1) < PI))
    T = p / rho * c["const2"]
    q5 = rho * (T * c["const1"] + 0.5 * (u * u + v * v + w * w))
    return _pack_state(n, n, n, rho, u, v, w, p, T, q5)


def grid1d(ia, ja, xmin=-5.0, xmax=5.0):
    """grid1d (src/gridgeneration.F90:143-173) with a second direction:
    x = (xmax - xmin)/ia * i + xmin, y = j/ja, z = 0."""
    x = (xmax - xmin) / float(ia) * np.arange(ia + 1, dtype=np.float64) + xmin
    y = 1.0 / float(ja) * np.arange(ja + 1, dtype=np.float64)
    return x, y, np.zeros(1)


def shock_tube_fields(kind, x):
    """rho, u, p of sodini / shuosherini (src/initialisation.F90:283-331
    and the Sod set-up after it) on the nodes x."""
    x = np.asarray(x, dtype=np.float64)
    if kind == "sod":
        left = x < 0.0
        rho = np.where(left, 1.0, 0.125)
        p = np.where(left, 1.0, 0.1)
        u = np.zeros_like(x)
    elif kind == "shuosher":
        left = x < -4.0
        rho = np.where(left, 3.857143, 1.0 + 0.2 * np.sin(5.0 * x))
        u = np.where(left, 2.629369, 0.0)
        p = np.where(left, 10.33333, 1.0)
    else:
        raise ValueError(kind)
    return rho, u, p


def shock_tube_state(kind, im, jm, mach=3.0, amp=0.0, gamma=1.4):
    """Halo-layout 2-D state (km = 0) of the Sod or Shu-Osher tube along x
    on grid1d nodes, uniform in y unless amp > 0, which multiplies the
    density by 1 + amp sin(2 pi y) (pressure unchanged) so that the y
    fluxes do work.  T = p/rho * gamma M^2 (thermal), q5 = p/(gamma-1) +
    rho |u|^2 / 2."""
    x, y, _ = grid1d(im, jm)
    rho1, u1, p1 = shock_tube_fields(kind, x)
    Y = y.reshape(1, -1, 1)
    rho = rho1.reshape(-1, 1, 1) * (1.0 + amp * np.sin(2.0 * PI * Y))
    u = u1.reshape(-1, 1, 1) * np.ones_like(rho)
    p = p1.reshape(-1, 1, 1) * np.ones_like(rho)
    v = np.zeros_like(rho)
    w = np.zeros_like(rho)
    c = refcal(mach, 1.0, gamma=gamma)
    T = p / rho * c["const2"]
    q5 = rho * (T * c["const1"] + 0.5 * (u * u + v * v + w * w))
    return _pack_state(im, jm, 0, rho, u, v, w, p, T, q5)


def riemann_exact(left, right, x, t, x0=0.0, gamma=1.4):
    """Exact solution of the 1-D Riemann problem for the Euler equations
    (ideal gas), states (rho, u, p): star pressure by Newton iteration on
    the pressure function and sampling of the wave fan (Toro, Riemann
    Solvers and Numerical Methods for Fluid Dynamics, 3rd ed., ch. 4).
    Returns rho, u, p at x and time t > 0."""
    rl, ul, pl = left
    rr, ur, pr = right
    g = gamma
    cl, cr = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)

    def fk(p, rk, pk, ck):
        if p > pk:  # shock
            A, B = 2.0 / ((g + 1.0) * rk), (g - 1.0) / (g + 1.0) * pk
            s = np.sqrt(A / (p + B))
            return (p - pk) * s, s * (1.0 - 0.5 * (p - pk) / (B + p))
        r = p / pk  # rarefaction
        return (2.0 * ck / (g - 1.0) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0),
                1.0 / (rk * ck) * r ** (-(g + 1.0) / (2.0 * g)))

    p = max(1e-8, 0.5 * (pl + pr))
    for _ in range(100):
        f1, d1 = fk(p, rl, pl, cl)
        f2, d2 = fk(p, rr, pr, cr)
        dp = (f1 + f2 + ur - ul) / (d1 + d2)
        p_new = max(1e-12, p - dp)
        if abs(p_new - p) < 1e-14 * p:
            p = p_new
            break
        p = p_new
    f1, _ = fk(p, rl, pl, cl)
    f2, _ = fk(p, rr, pr, cr)
    us = 0.5 * (ul + ur) + 0.5 * (f2 - f1)
    S = (np.asarray(x, dtype=np.float64) - x0) / t
    rho = np.empty_like(S)
    uu = np.empty_like(S)
    pp = np.empty_like(S)
    gm = (g - 1.0) / (g + 1.0)
    for n, s in enumerate(S.ravel()):
        if s <= us:  # left of the contact
            if p > pl:
                sl = ul - cl * np.sqrt((g + 1.0) / (2.0 * g) * p / pl + (g - 1.0) / (2.0 * g))
                st = (rl * ((p / pl + gm) / (gm * p / pl + 1.0)), us, p) if s >= sl else (rl, ul, pl)
            else:
                shl = ul - cl
                cls = cl * (p / pl) ** ((g - 1.0) / (2.0 * g))
                stl = us - cls
                if s <= shl:
                    st = (rl, ul, pl)
                elif s >= stl:
                    st = (rl * (p / pl) ** (1.0 / g), us, p)
                else:
                    c = 2.0 / (g + 1.0) * (cl + (g - 1.0) / 2.0 * (ul - s))
                    uf = 2.0 / (g + 1.0) * (cl + (g - 1.0) / 2.0 * ul + s)
                    st = (rl * (c / cl) ** (2.0 / (g - 1.0)), uf, pl * (c / cl) ** (2.0 * g / (g - 1.0)))
        else:
            if p > pr:
                sr = ur + cr * np.sqrt((g + 1.0) / (2.0 * g) * p / pr + (g - 1.0) / (2.0 * g))
                st = (rr * ((p / pr + gm) / (gm * p / pr + 1.0)), us, p) if s <= sr else (rr, ur, pr)
            else:
                shr = ur + cr
                crs = cr * (p / pr) ** ((g - 1.0) / (2.0 * g))
                str_ = us + crs
                if s >= shr:
                    st = (rr, ur, pr)
                elif s <= str_:
                    st = (rr * (p / pr) ** (1.0 / g), us, p)
                else:
                    c = 2.0 / (g + 1.0) * (cr - (g - 1.0) / 2.0 * (ur - s))
                    uf = 2.0 / (g + 1.0) * (-cr + (g - 1.0) / 2.0 * ur + s)
                    st = (rr * (c / cr) ** (2.0 / (g - 1.0)), uf, pr * (c / cr) ** (2.0 * g / (g - 1.0)))
        rho.flat[n], uu.flat[n], pp.flat[n] = st
    return rho, uu, pp


def _pack_state(im, jm, km, rho, u, v, w, p, T, q5):
    full = (im + 2 * HM + 1, jm + 2 * HM + 1, km + 2 * HM + 1)
    sl = (slice(HM, HM + im + 1), slice(HM, HM + jm + 1), slice(HM, HM + km + 1))
    q = np.zeros(full + (5,), order="F")
    vel = np.zeros(full + (3,), order="F")
    out = {"q": q, "vel": vel}
    for name in ("rho", "prs", "tmp"):
        out[name] = np.zeros(full, order="F")
    out["rho"][sl] = rho
    out["prs"][sl] = p
    out["tmp"][sl] = T
    vel[sl + (0,)] = u
    vel[sl + (1,)] = v
    vel[sl + (2,)] = w
    q[sl + (0,)] = rho
    q[sl + (1,)] = rho * u
    q[sl + (2,)] = rho * v
    q[sl + (3,)] = rho * w
    q[sl + (4,)] = q5
    return out
