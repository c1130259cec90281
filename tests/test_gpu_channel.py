"""Compressible channel on the GPU: noslip isothermal walls, src_chan body
force and the mass-flux controller against the oracle (FP64, 1e-12), and
the FP32-storage form against the FP64 form."""
import numpy as np
import pytest

from test_channel import H, MACH, RE, channel_oracle

pytestmark = pytest.mark.gpu


def gpu_channel(o, dxi, precision):
    """GPU channel context from the oracle's state; dxi with nonzero
    off-diagonals selects the general-metric kernels."""
    from astr_gb300.solver import GpuSolver
    c = o.cfg
    g = GpuSolver(o.im, o.jm, o.km, precision=precision, npdc=(3, 4, 3), mach=MACH,
                  reynolds=RE, deltat=c.deltat, channel=True, twall=1.0)
    g.set_metrics(dxi, o.field("jacob"))
    g.set_grid(o.field("x"))
    g.upload_state(o.field("q"), o.field("rho"), o.field("vel"), o.field("prs"), o.field("tmp"))
    return g


def _case(im, jm, km):
    """The oracle with gridgeom's off-diagonal rounding residue (about 1e-12
    of the diagonal) zeroed, and the same diagonal metrics for the GPU (the
    rectilinear kernels); the residue itself is covered by the general-metric
    test."""
    o, grid, st, dt = channel_oracle(im, jm, km, zero_offdiag=True)
    return o, o.field("dxi").copy(order="F")


@pytest.mark.parametrize("dims", [(32, 48, 16), (24, 40, 20)])
def test_channel_fp64_matches_oracle(gpu_lib, dims):
    from astr_gb300 import capi
    im, jm, km = dims
    o, dxi = _case(im, jm, km)
    g = gpu_channel(o, dxi, capi.FP64)
    steps = 6
    o.rk3_steps(steps)
    g.time_integration_rk(steps)
    s = g.download_state()
    cs = g.channel_state()
    g.close()
    sl = (slice(H, H + im + 1), slice(H, H + jm + 1), slice(H, H + km + 1))
    for m in range(5):
        ref = o.field("q")[sl + (m,)]
        err = np.abs(s["q"][sl + (m,)] - ref).max() / np.abs(ref).max()
        assert err <= 1e-12, (m, err)
    for name in ("prs", "tmp", "rho"):
        ref = o.field(name)[sl]
        err = np.abs(s[name][sl] - ref).max() / np.abs(ref).max()
        assert err <= 1e-12, (name, err)
    oc = o.chan_state()
    assert cs[4] == oc[4] == steps
    # mass flux, its target and the wall friction: relative
    for k in (1, 2, 3):
        assert abs(cs[k] - oc[k]) <= 1e-12 * abs(oc[k]), (k, cs[k], oc[k])
    # the force of chanfoce is a difference of mass fluxes that agree to
    # about 1e-5 (src/statistic.F90:1516-1519): scored against its operand
    # scale, mass flux / ly
    ly = 2.0
    assert abs(cs[0] - oc[0]) <= 1e-12 * abs(oc[2]) / ly, (cs[0], oc[0])


def test_channel_fp32_storage_error(gpu_lib):
    from astr_gb300 import capi
    im, jm, km = 48, 64, 32
    o, dxi = _case(im, jm, km)
    steps = 20
    out = {}
    for name, prec in (("fp64", capi.FP64), ("fp32", capi.FP32_STORAGE)):
        g = gpu_channel(o, dxi, prec)
        g.time_integration_rk(steps)
        out[name] = (g.download_state(), g.channel_state())
        g.close()
    sl = (slice(H, H + im + 1), slice(H, H + jm + 1), slice(H, H + km + 1))
    a, b = out["fp32"][0]["q"][sl], out["fp64"][0]["q"][sl]

    def l2(x, y):
        return float(np.linalg.norm(x - y) / np.linalg.norm(y))

    e = {"rho": l2(a[..., 0], b[..., 0]), "mom": l2(a[..., 1:4], b[..., 1:4]),
         "E": l2(a[..., 4], b[..., 4])}
    fe = abs(out["fp32"][1][0] - out["fp64"][1][0]) / abs(out["fp64"][1][0])
    print(f"channel {im}x{jm}x{km}, {steps} steps: FP32-storage vs FP64 " +
          " ".join(f"{k} {v:.2e}" for k, v in e.items()) + f"; force {fe:.2e}")
    assert max(e.values()) <= 1e-5
    assert fe <= 1e-4
