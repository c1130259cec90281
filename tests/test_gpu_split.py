"""Both sweep organisations against the oracle: the variables of a line in
one block with the stress, RK3 update and statistics fused into the sweeps
(large grids), and the variables spread over blocks with those as point
kernels (grids with fewer y-line blocks than SMs); and the statistics entry
point in every mode."""
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from test_gpu_parity import compare_state, gpu_from_oracle

pytestmark = pytest.mark.gpu


def _with_split(split, fn):
    old = os.environ.get("ASTR_VAR_SPLIT")
    os.environ["ASTR_VAR_SPLIT"] = "1" if split else "0"
    try:
        return fn()
    finally:
        if old is None:
            del os.environ["ASTR_VAR_SPLIT"]
        else:
            os.environ["ASTR_VAR_SPLIT"] = old


@pytest.mark.parametrize("split", [False, True])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_tgv_steps_both_organisations(gpu_lib, split, prec):
    from astr_gb300 import capi
    o = po.tgv_main(24)
    precision = capi.FP64 if prec == "fp64" else capi.FP32_STORAGE
    g = _with_split(split, lambda: gpu_from_oracle(o, precision=precision))
    hist_g = g.time_integration_rk(3)
    st = g.download_state()
    g.close()
    hist_o = o.rk3_steps(3)
    if prec == "fp64":
        compare_state(o, st, full=False)
        np.testing.assert_allclose(hist_g, hist_o, rtol=1e-12)
    else:
        compare_state(o, st, full=False, tol=1e-6)
        np.testing.assert_allclose(hist_g, hist_o, rtol=1e-6)


@pytest.mark.parametrize("split", [False, True])
@pytest.mark.parametrize("general", [False, True])
def test_reduce_stats(gpu_lib, split, general):
    """astr_gpu_reduce_stats after qswap + gradcal equals the oracle's
    kenergycal / enstophycal on the same state."""
    from test_gpu_general_metrics import _wavy_case
    o = _wavy_case(16, deltat=2e-3) if general else po.tgv_main(24)
    g = _with_split(split, lambda: gpu_from_oracle(o))
    o.call("qswap")
    o.call("gradcal")
    g.qswap()
    g.gradcal()
    ke, en = g.reduce_stats()
    g.close()
    np.testing.assert_allclose([ke, en], [o.kenergy(), o.enstrophy()], rtol=1e-12)
