"""Compact MP convective scheme (conschm 543c) in the oracle, on CPU: the
known answers of its parts (MP5 limiter, Steger-Warming split, Roe
eigenvectors, compact upwind interface flux) and a Sod shock tube against
the exact Riemann solution."""
import numpy as np
import pytest

from astr_gb300 import cases

H = 5


def _line_oracle(n, npdc=3, bfac=0.3):
    from oracle import pyoracle as po
    return po.Oracle(n, 8, 0, npdc=(npdc, 3, 3), conschm="543c", bfacmpld=bfac, lfilter=False,
                     diffterm=False)


def test_mp5_known_answers():
    from oracle import pyoracle as po
    # smooth monotone data: the linear value passes unchanged
    u = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    ul = (2 * u[0] - 13 * u[1] + 47 * u[2] + 27 * u[3] - 3 * u[4]) / 60.0
    assert po.mp5(u, ul) == ul
    # no limiting when the shock flag is off, whatever the data
    step = np.array([0.0, 0.0, 0.0, 1.0, 1.0])
    assert po.mp5(step, 1.3, discont=False) == 1.3
    # an overshoot at a step is pulled back into the monotone range
    v = po.mp5(step, 1.3)
    assert 0.0 <= v <= 1.0
    v = po.mp5(step[::-1].copy(), -0.2)
    assert 0.0 <= v <= 1.0


def test_steger_warming_split_sums_to_the_flux():
    o = _line_oracle(16)
    rng = np.random.default_rng(7)
    mach = o.cfg.mach
    for trial in range(50):
        rho = rng.uniform(0.5, 2.0)
        vel = rng.uniform(-0.5, 0.5, 3)
        T = rng.uniform(0.5, 2.0)
        p = rho * T / (1.4 * mach * mach)
        q = np.array([rho, rho * vel[0], rho * vel[1], rho * vel[2],
                      p / 0.4 + 0.5 * rho * vel @ vel])
        x = rng.uniform(-2.0, 2.0, 3)
        J = rng.uniform(0.5, 2.0)
        fp, fm = o.steger_warming([rho, vel[0], vel[1], vel[2], p, T], q, x, J)
        U = x @ vel
        F = J * np.array([q[0] * U, q[1] * U + x[0] * p, q[2] * U + x[1] * p,
                          q[3] * U + x[2] * p, (q[4] + p) * U])
        scale = J * (abs(U) + np.sqrt(T) / mach * np.linalg.norm(x)) * (q[4] + p)
        assert np.max(np.abs(fp + fm - F)) <= 1e-13 * scale
    # supersonic along the metric direction: all of the flux goes one way
    rho, T = 1.0, 1.0
    p = rho * T / (1.4 * mach * mach)
    vel = np.array([2.0 / mach, 0.0, 0.0])
    q = np.array([rho, rho * vel[0], 0.0, 0.0, p / 0.4 + 0.5 * rho * vel @ vel])
    fp, fm = o.steger_warming([rho, vel[0], 0, 0, p, T], q, [1.0, 0, 0], 1.0)
    assert np.all(fm == 0.0) and fp[0] == rho * vel[0]
    fp, fm = o.steger_warming([rho, -vel[0], 0, 0, p, T], q * [1, -1, 1, 1, 1], [1.0, 0, 0], 1.0)
    assert np.all(fp == 0.0) and fm[0] == -rho * vel[0]


@pytest.mark.parametrize("row", [(1.0, 0.2, 0.1), (0.0, 1.0, 0.3), (0.0, 0.0, 2.0)])
def test_chardecomp_left_right_inverse(row):
    from oracle import pyoracle as po
    rng = np.random.default_rng(11)
    for trial in range(20):
        sts = []
        for side in range(2):
            rho = rng.uniform(0.5, 2.0)
            vel = rng.uniform(-1.0, 1.0, 3)
            p = rng.uniform(0.5, 2.0)
            E = p / 0.4 + 0.5 * rho * vel @ vel
            sts.append([p / rho, rho, p, E, vel[0], vel[1], vel[2]] + list(row))
        R, L = po.chardecomp(sts[0], sts[1])
        assert np.max(np.abs(L @ R - np.eye(5))) < 1e-12


@pytest.mark.parametrize("wind", [1, -1])
def test_compact_upwind_flux_order(wind):
    """(fh(i) - fh(i-1)) is the flux derivative to fifth order away from the
    ends of a periodic line, and to fourth order next to them, where the
    system's end rows are explicit sixth-order central interface values
    (ntype 3)."""
    inner, whole = [], []
    for n in (32, 64, 128):
        o = _line_oracle(n)
        h = 2.0 * np.pi / n
        xs = h * np.arange(-H, n + H + 1)
        fh = o.line_flux(0, wind, np.sin(xs))
        e = np.abs((fh[1:] - fh[:-1]) / h - np.cos(xs[H:H + n + 1]))  # nodes 0..n
        inner.append(e[n // 4:3 * n // 4].max())
        whole.append(e.max())
    r_in = np.log2(np.array(inner[:-1]) / np.array(inner[1:]))
    r_all = np.log2(np.array(whole[:-1]) / np.array(whole[1:]))
    assert np.all(r_in > 4.8) and np.all(r_all > 3.9) and whole[-1] < 1e-8, (r_in, r_all)


def test_compact_upwind_flux_walls():
    """ntype 4 (both ends physical): third-order closures; a linear flux is
    reproduced exactly up to rounding, a smooth one to the boundary order."""
    n = 64
    o = _line_oracle(n, npdc=4)
    xs = np.arange(-H, n + H + 1) / n
    for wind in (1, -1):
        fh = o.line_flux(0, wind, 2.0 * xs + 1.0)
        d = (fh[1:] - fh[:-1]) * n
        assert np.max(np.abs(d[1:] - 2.0)) < 1e-10
        fh = o.line_flux(0, wind, np.sin(3.0 * xs))
        d = (fh[1:] - fh[:-1]) * n
        assert np.max(np.abs(d[1:] - 3.0 * np.cos(3.0 * xs[H + 1:H + n + 1]))) < 5e-3


def sod_oracle(im, jm, dt, amp=0.0, **kw):
    from oracle import pyoracle as po
    st = cases.shock_tube_state("sod", im, jm, amp=amp)
    o = po.from_state(st, (im, jm, 0), grid=cases.grid1d(im, jm), npdc=(4, 3, 3), mach=3.0,
                      conschm="543c", lfilter=False, diffterm=False, deltat=dt, **kw)
    return o, st


def test_sod_tube_matches_the_exact_solution():
    im, jm, dt, t_end = 100, 8, 0.01, 1.5
    o, _ = sod_oracle(im, jm, dt)
    o.rk3_steps(int(round(t_end / dt)))
    x, _, _ = cases.grid1d(im, jm)
    rho = o.field("rho")[H:H + im + 1, H:H + jm + 1, H]
    # uniform in y
    assert np.max(np.abs(rho - rho[:, :1])) < 1e-12
    re, ue, pe = cases.riemann_exact((1.0, 0.0, 1.0), (0.125, 0.0, 0.1), x, t_end)
    l1 = np.mean(np.abs(rho[:, 0] - re))
    assert l1 < 0.02, l1
    # the shock sensor marks the shock and the contact, not the still gas
    # (it also marks the five nodes next to each end, where the sensor's
    # pressure stencil reads the unset halo: zero here)
    ls = o.lshock()[:, 0, 0]
    assert ls[np.argmin(np.abs(x - 1.75 * t_end))]
    assert not ls[np.argmin(np.abs(x + 3.0))] and not ls[np.argmin(np.abs(x - 3.5))]
    # no new extrema beyond a few per cent (monotonicity preservation)
    assert rho.min() > 0.125 * 0.97 and rho.max() < 1.0 * 1.03
