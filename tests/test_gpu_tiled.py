"""The tile-staged sweeps (sweeps2.cuh) against the oracle and against the
register-window sweeps.

The FP32-storage form runs the tiled sweeps by default; the FP64 form runs
them when ASTR_V2=2 is set at context creation, which is how these tests
hold them to the FP64 bar (1e-12 max-norm relative against the oracle):
periodic boxes with and without the variables spread over blocks (a grid
too small to fill the SMs spreads them), walls with a stretched grid and
uniform Thomas chunks (the channel), a box with a boundary routine on every
face, and the per-routine drop-ins.  The FP32-storage form's two sweep
families must agree to its own rounding.
"""
import numpy as np
import pytest

from conftest import relerr
from oracle import pyoracle as po
from test_gpu_parity import TOL, compare_state, gpu_from_oracle, interior

pytestmark = pytest.mark.gpu


@pytest.fixture
def tiled64(monkeypatch):
    monkeypatch.setenv("ASTR_V2", "2")


@pytest.mark.parametrize("n", [40, 64])
def test_tiled_fp64_tgv(gpu_lib, tiled64, n):
    """40^3 spreads the variables over blocks, 64^3 runs whole lines per block."""
    o = po.tgv_main(n)
    g = gpu_from_oracle(o)
    hist_g = g.time_integration_rk(3)
    hist_o = o.rk3_steps(3)
    compare_state(o, g.download_state(), full=True)
    assert relerr(hist_g, hist_o) <= TOL
    g.close()


def test_tiled_fp64_anisotropic(gpu_lib, tiled64):
    o = po.Oracle(72, 40, 56, mode=po.MODE_MAIN)
    L = 2 * np.pi
    o.gridcube(L, L, L)
    o.call("gridgeom")
    o.call("init_tgv")
    g = gpu_from_oracle(o)
    g.time_integration_rk(2)
    o.rk3_steps(2)
    compare_state(o, g.download_state(), full=True)
    g.close()


def test_tiled_fp64_channel(gpu_lib, tiled64):
    """Walls in y with the one-sided closures, a tanh-stretched grid, the
    body force and controller; lines long enough for uniform chunks."""
    from astr_gb300 import capi
    from test_gpu_channel import _case, gpu_channel
    im, jm, km = 32, 96, 16
    o, dxi = _case(im, jm, km)
    g = gpu_channel(o, dxi, capi.FP64)
    o.rk3_steps(4)
    g.time_integration_rk(4)
    s = g.download_state()
    g.close()
    h = po.HM
    sl = (slice(h, h + im + 1), slice(h, h + jm + 1), slice(h, h + km + 1))
    for m in range(5):
        ref = o.field("q")[sl + (m,)]
        err = np.abs(s["q"][sl + (m,)] - ref).max() / np.abs(ref).max()
        assert err <= TOL, (m, err)


def test_tiled_fp64_boundary_routines(gpu_lib, tiled64):
    from test_gpu_bc import _cmp, _gpu_from, _mixed_box
    o = _mixed_box()
    g = _gpu_from(o)
    o.rk3_steps(4)
    g.time_integration_rk(4)
    s = g.download_state()
    g.close()
    _cmp(o, s)


def test_tiled_fp64_routines(gpu_lib, tiled64):
    """filterq, gradcal and rhscal one at a time (the drop-in entry points)."""
    from test_gpu_parity import flux_scale
    o = po.tgv_main(48)
    o.rk3_steps(1)
    g = gpu_from_oracle(o)
    o.call("filterq")
    g.filterq()
    assert relerr(interior(g.download_state()["q"], o), interior(o.field("q"), o)) <= TOL
    o.call("qswap")
    g.qswap()
    o.call("gradcal")
    g.gradcal()
    r = g.download_rhs()
    dvel_ref = o.field("dvel")
    dvel = r["dvel"].reshape(dvel_ref.shape, order="F")
    vel = interior(o.field("vel"), o)
    dxi_max = float(np.max(np.abs(o.field("dxi"))))
    assert np.max(np.abs(dvel - dvel_ref)) / (np.max(np.abs(vel)) * dxi_max) <= TOL
    o.field("qrhs")[...] = 0.0
    o.call("rhscal")
    g.rhscal()
    r = g.download_rhs()
    scale = flux_scale(o)
    for n in range(5):
        e = float(np.max(np.abs(r["qrhs"][..., n] - o.field("qrhs")[..., n]))) / scale[n]
        assert e <= TOL, (n, e)
    g.close()


def _fp32_tgv(n, steps, v2):
    import os
    from astr_gb300 import capi
    from test_gpu_fp32 import _case
    old = os.environ.get("ASTR_V2")
    os.environ["ASTR_V2"] = v2
    try:
        return _case(n, capi.FP32_STORAGE, steps=steps)
    finally:
        if old is None:
            del os.environ["ASTR_V2"]
        else:
            os.environ["ASTR_V2"] = old


def test_tiled_fp32_matches_register_window(gpu_lib):
    """Both FP32-storage sweep families from the same state: the same
    arithmetic up to FP32 rounding order."""
    a, ha = _fp32_tgv(64, 10, "1")
    b, hb = _fp32_tgv(64, 10, "0")
    h = po.HM
    sl = (slice(h, h + 65),) * 3
    qa, qb = a["q"][sl], b["q"][sl]
    err = float(np.linalg.norm((qa - qb).ravel()) / np.linalg.norm(qb.ravel()))
    print(f"FP32 storage, tiled vs register-window sweeps: rel L2 {err:.2e}")
    assert err <= 1e-6
    assert relerr(ha, hb) <= 1e-6
