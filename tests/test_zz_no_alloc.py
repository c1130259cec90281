"""The allocation-free statistics entry point against the context's own.

astr_gpu_stats_noalloc exists for callers that cannot call cudaMalloc (a
host whose HBM is all owned by its own pool, or a time loop that must not
synchronise the device through an allocation).  It keeps its partial sums
in a fixed device array instead of context memory; this checks, through the
C ABI, that two calls in a row (and a second block size after them) return
what astr_gpu_reduce_stats returns, to the parity tolerance of the suite.
This file is collected last so a stop-at-first-failure run has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _device_copy(torch, a):
    flat = np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))
    return torch.from_numpy(flat).to("cuda")


def _case(n, steps):
    from astr_gb300 import capi, cases
    from astr_gb300.solver import GpuSolver
    L = 2 * np.pi
    x, y, z = cases.gridcube(n, n, n, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.tgv_state(n, n, n, x=x, y=y, z=z)
    g = GpuSolver(n, n, n, order=capi.ORDER_MAIN)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    g.time_integration_rk(steps)
    ref = g.reduce_stats()
    state = g.download_state()
    rhs = g.download_rhs()
    return g, ref, state, rhs


def _noalloc(gpu_lib, torch, g, state, rhs, l0=1.0, stream=None):
    from astr_gb300 import capi
    rho = _device_copy(torch, state["rho"])
    vel = _device_copy(torch, state["vel"])
    dvel = _device_copy(torch, rhs["dvel"])
    torch.cuda.synchronize()
    ke, en = ctypes.c_double(), ctypes.c_double()
    handle = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
    rc = gpu_lib.astr_gpu_stats_noalloc(rho.data_ptr(), vel.data_ptr(), dvel.data_ptr(),
                                        ctypes.byref(g.dims), l0, handle,
                                        ctypes.byref(ke), ctypes.byref(en))
    assert rc == capi.ASTR_OK
    return ke.value, en.value


def _vortex2d(n, steps):
    """A 2-D block (ka = 0): only the k = 0 plane is summed and the
    enstrophy comes from the z vorticity alone."""
    from astr_gb300 import cases
    from astr_gb300.solver import GpuSolver
    mach = 1.0 / np.sqrt(1.4)
    st = cases.vortex_state(n)
    x, y, z = cases.vortex_grid(n)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    dt = cases.cfl_deltat(st, (d11, d22, d33), mach)
    g = GpuSolver(n, n, 0, diffterm=False, mach=mach, reynolds=1e4, deltat=dt)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    g.time_integration_rk(steps)
    return g, g.reduce_stats(), g.download_state(), g.download_rhs()


def test_stats_noalloc_matches_reduce_stats(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g, ref, state, rhs = _case(40, 2)
    first = _noalloc(gpu_lib, torch, g, state, rhs)
    second = _noalloc(gpu_lib, torch, g, state, rhs)
    for got in (first, second):
        assert abs(got[0] - ref[0]) <= TOL * abs(ref[0])
        assert abs(got[1] - ref[1]) <= TOL * abs(ref[1])
    g.close()
    # a smaller block right after: the shared scratch keeps the previous
    # call's partials, none of which may leak into this result
    g2, ref2, state2, rhs2 = _case(24, 1)
    third = _noalloc(gpu_lib, torch, g2, state2, rhs2)
    assert abs(third[0] - ref2[0]) <= TOL * abs(ref2[0])
    assert abs(third[1] - ref2[1]) <= TOL * abs(ref2[1])
    g2.close()


def test_stats_noalloc_2d_and_caller_stream(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g, ref, state, rhs = _vortex2d(24, 1)
    for _ in range(2):
        got = _noalloc(gpu_lib, torch, g, state, rhs)
        assert abs(got[0] - ref[0]) <= TOL * abs(ref[0])
        assert abs(got[1] - ref[1]) <= TOL * abs(ref[1])
    # on a stream of the caller's, with an enstrophy length scale l0 = 2:
    # the enstrophy is normalised by (uinf / l0)^2, so it scales by l0^2
    s = torch.cuda.Stream()
    got = _noalloc(gpu_lib, torch, g, state, rhs, l0=2.0, stream=s)
    assert abs(got[0] - ref[0]) <= TOL * abs(ref[0])
    assert abs(got[1] - 4.0 * ref[1]) <= TOL * abs(4.0 * ref[1])
    g.close()


def test_stats_noalloc_rejects_oversize(gpu_lib):
    from astr_gb300 import capi
    d = capi.AstrDims(700, 700, 700, 700, 700, 700, 3, 3, 3)
    ke, en = ctypes.c_double(), ctypes.c_double()
    one = ctypes.c_double(0.0)
    p = ctypes.addressof(one)
    rc = gpu_lib.astr_gpu_stats_noalloc(p, p, p, ctypes.byref(d), 1.0, None,
                                        ctypes.byref(ke), ctypes.byref(en))
    assert rc == capi.ASTR_ERR_UNSUPPORTED


def test_stats_noalloc_rejects_dims_create_rejects(gpu_lib):
    """The block sizes astr_gpu_create refuses are refused here too: a 2-D
    block (ka = 0) with km != 0, and lines shorter than 8 intervals."""
    from astr_gb300 import capi
    ke, en = ctypes.c_double(), ctypes.c_double()
    one = ctypes.c_double(0.0)
    p = ctypes.addressof(one)
    for dims in ((16, 16, 4, 16, 16, 0), (4, 16, 16, 4, 16, 16), (16, 16, 6, 16, 16, 6)):
        d = capi.AstrDims(*dims, 3, 3, 3)
        rc = gpu_lib.astr_gpu_stats_noalloc(p, p, p, ctypes.byref(d), 1.0, None,
                                            ctypes.byref(ke), ctypes.byref(en))
        assert rc == capi.ASTR_ERR_ARG, dims
