"""Serving on the GPU: every case's result is the same alone and in the mix
(bit for bit: each case keeps its own context and stream, and its kernels
and reductions do not depend on what else runs), and the graph-launched
steps equal the ordinary stepping path."""
import numpy as np
import pytest

from astr_gb300 import capi, serve

pytestmark = pytest.mark.gpu

MIX = [
    serve.Request(0, "tgv3d", 24, 1600.0, 0.1, 12, 0.0),
    serve.Request(1, "vortex2d", 64, 500.0, 0.2, 30, 0.0),
    serve.Request(2, "tgv3d", 40, 300.0, 0.25, 8, 0.01),
    serve.Request(3, "vortex2d", 96, 2000.0, 0.05, 20, 0.02),
    serve.Request(4, "tgv3d", 32, 3000.0, 0.15, 15, 0.02),
    serve.Request(5, "vortex2d", 80, 100.0, 0.3, 25, 0.03),
]


def _alone(req, precision):
    be = serve.GpuBackend(precision)
    h = be.start(req)
    be.enqueue(h, req.steps)
    while not be.done(h):
        pass
    out, _ = be.finish(h)
    return out


def test_results_same_alone_and_in_mix(gpu_lib):
    be = serve.GpuBackend(capi.FP32_STORAGE)
    srv = serve.Server(be, hbm_budget=8 << 30, max_active=4)
    recs = serve.serve(MIX, srv)
    assert srv.peak_active >= 2  # cases overlapped
    for req, rec in zip(MIX, recs):
        ref = _alone(req, capi.FP32_STORAGE)
        for k in ("q", "rho", "vel", "prs", "tmp"):
            assert np.array_equal(rec.result[k], ref[k]), (req.rid, k)


def test_graph_steps_equal_plain_steps(gpu_lib):
    from astr_gb300.solver import GpuSolver
    for req in (MIX[0], MIX[1]):
        dims, kw, diag, J, st = serve.case_inputs(req)
        outs = []
        for mode in ("graph", "plain"):
            g = GpuSolver(*dims, precision=capi.FP32_STORAGE, **kw)
            g.set_metrics_diag(diag[0], diag[1], diag[2], J)
            g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
            if mode == "graph":
                g.step_async(req.steps)
                g.synchronize()
            else:
                g.timed_steps(req.steps)
            outs.append(g.download_state())
            g.close()
        for k in ("q", "prs"):
            assert np.array_equal(outs[0][k], outs[1][k])
