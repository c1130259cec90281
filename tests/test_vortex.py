"""2-D isentropic vortex transport (inviscid, periodic [-5,5]^2, beta = 5,
freestream (1, 1)): the analytic workload against the oracle's 2-D
inviscid path, on CPU."""
import numpy as np

from astr_gb300 import cases

GAMMA = 1.4
MACH = 1.0 / np.sqrt(GAMMA)


def _oracle_error(n, t_end=1.0):
    from oracle import pyoracle as po
    st = cases.vortex_state(n)
    x, y, z = cases.vortex_grid(n)
    (d11, d22, d33), _ = cases.rect_metrics(x, y, z, diag_only=True)
    dt = cases.cfl_deltat(st, (d11, d22, d33), MACH)
    nst = int(round(t_end / dt))
    o = po.from_state(st, (n, n, 0), lx=10.0, ly=10.0, lz=0.0, diffterm=False, mach=MACH,
                      reynolds=1e4, deltat=t_end / nst)
    o.rk3_steps(nst)
    ex = cases.vortex_state(n, t=t_end)
    h = 5
    sl = (slice(h, h + n + 1), slice(h, h + n + 1), h)
    e = o.field("rho")[sl] - ex["rho"][sl]
    return float(np.sqrt(np.mean(e * e))), float(np.abs(e).max())


def test_vortex_initial_state_is_isentropic():
    st = cases.vortex_state(64)
    h = 5
    sl = (slice(h, h + 65), slice(h, h + 65), h)
    rho, p, T = st["rho"][sl], st["prs"][sl], st["tmp"][sl]
    np.testing.assert_allclose(p, rho ** GAMMA, rtol=1e-14)
    np.testing.assert_allclose(T, p / rho, rtol=1e-14)
    # the exact solution after one period of the box (t = 10) is the start
    st10 = cases.vortex_state(64, t=10.0)
    np.testing.assert_allclose(st10["q"], st["q"], atol=1e-12)


def test_vortex_oracle_converges_to_analytic():
    e32, _ = _oracle_error(32)
    e64, m64 = _oracle_error(64)
    # 6th-order compact scheme: at least 2^5 from 32^2 to 64^2
    assert e32 / e64 > 32.0, (e32, e64)
    assert e64 < 2e-6 and m64 < 2e-5, (e64, m64)
