"""Compressible channel (noslip isothermal j-walls, src_chan body force,
mass-flux controller) in the oracle, and the channel workload, on CPU."""
import numpy as np

from astr_gb300 import cases

MACH, RE = 0.5, 3000.0
H = 5


def channel_oracle(im, jm, km, zero_offdiag=True, **kw):
    from oracle import pyoracle as po
    x, y, z = cases.channel_grid(im, jm, km)
    st = cases.channel_state(im, jm, km, y, mach=MACH)
    dxi, _ = cases.rect_metrics(x, y, z, npdc=(3, 4, 3))
    dt = cases.cfl_deltat(st, tuple(dxi[..., d, d] for d in range(3)), MACH)
    o = po.from_state(st, (im, jm, km), grid=(x, y, z), npdc=(3, 4, 3), channel=True, mach=MACH,
                      reynolds=RE, deltat=dt, twall=1.0, **kw)
    if zero_offdiag:
        D = o.field("dxi")
        for d in range(3):
            for m in range(3):
                if d != m:
                    D[..., d + 3 * m] = 0.0
    return o, (x, y, z), st, dt


def test_channel_workload():
    x, y, z = cases.channel_grid(32, 48, 16)
    assert y[0] == 0.0 and y[-1] == 2.0 and np.all(np.diff(y) > 0)
    dy = np.diff(y)
    assert dy[0] < dy[len(dy) // 2] / 3  # clustered at the walls
    st = cases.channel_state(32, 48, 16, y, mach=MACH)
    sl = (slice(H, H + 33), slice(H, H + 49), slice(H, H + 17))
    u = st["vel"][sl + (0,)]
    assert np.all(u[:, 0, :] == 0.0) and np.all(u[:, -1, :] == 0.0)
    # laminar bulk velocity 1 (trapezoid), perturbation bounded by 5 %
    U = 1.5 * (1.0 - (y - 1.0) ** 2)
    assert np.all(np.abs(u - U[None, :, None]) <= 0.05 * U[None, :, None] + 1e-15)
    # counter-based: the same numbers whatever the array is reused for
    r1 = cases.splitmix64_uniform(20261203, np.arange(10, dtype=np.uint64))
    r2 = cases.splitmix64_uniform(20261203, np.arange(5, 10, dtype=np.uint64))
    assert np.array_equal(r1[5:], r2) and np.all((r1 >= 0) & (r1 < 1))


def test_channel_oracle_walls_and_controller():
    o, (x, y, z), st, dt = channel_oracle(16, 32, 8)
    hist = []
    for _ in range(6):
        o.rk3_steps(1)
        hist.append(o.chan_state())
    im, jm, km = 16, 32, 8
    # boucon runs at the start of each stage: apply it to see the walls
    o.call("boucon")
    vel, tmp = o.field("vel"), o.field("tmp")
    for j in (0, jm):
        assert np.all(vel[H:H + im + 1, H + j, H:H + km + 1, :] == 0.0)
        assert np.all(tmp[H:H + im + 1, H + j, H:H + km + 1] == 1.0)
    hist = np.array(hist)
    # no statcal on the first step; the target is the mass flux at the first statcal
    assert hist[0, 0] == 0.0 and hist[0, 2] == 0.0
    assert hist[1, 2] != 0.0 and np.all(hist[2:, 2] == hist[1, 2])
    # the controller keeps the mass flux at its target
    assert np.all(np.abs(hist[1:, 1] - hist[1, 2]) / hist[1, 2] < 1e-3)
    assert np.all(np.isfinite(o.field("q")))
