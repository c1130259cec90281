"""Crash control (lcracon, src/mainloop.F90:709-1198) on the GPU.

Failures are made on the host, never by a device fault: a state poisoned
with a negative density is uploaded, and the context must roll back to its
older snapshot (databakup's 'recovery') and carry on exactly as an
unpoisoned run from that step; crashfix is checked against a restatement of
the reference loop on the host; repeated rollbacks to one snapshot expand
the critical-node mask; a crash before any backup is an error.
"""
import numpy as np
import pytest

from astr_gb300 import capi

pytestmark = pytest.mark.gpu

H = 5


def _tgv(n, precision=capi.FP64):
    from astr_gb300 import cases
    from astr_gb300.solver import GpuSolver
    L = 2 * np.pi
    x, y, z = cases.gridcube(n, n, n, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.tgv_state(n, n, n, x=x, y=y, z=z)
    g = GpuSolver(n, n, n, order=capi.ORDER_MAIN, precision=precision, deltat=2e-3)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(st["q"], st["rho"], st["vel"], st["prs"], st["tmp"])
    return g


def _poison(g, node=(7, 9, 11)):
    q = g.download_state()["q"]
    i, j, k = node
    q[H + i, H + j, H + k, 0] = -1.0
    g.upload_q(q)


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32_STORAGE])
def test_rollback_matches_unpoisoned_run(gpu_lib, precision):
    g = _tgv(24, precision)
    g.set_crash_control(True)
    for _ in range(12):
        g.time_integration_rk(1)
    rep = g.crash_report()
    # backups at nstep 5 and 10 (interval 5, then doubled), next at 20
    assert rep["backups"] == 2 and rep["next_backup"] == 20 and rep["rollbacks"] == 0
    _poison(g)
    st = capi.AstrStatus()
    import ctypes
    g._c(g.L.astr_gpu_rk3_step(g.h, 1, None, ctypes.byref(st)))
    assert st.crash == 1
    rep = g.crash_report()
    # rolled back to the older snapshot (nstep 5), then stepped once
    assert rep["rollbacks"] == 1 and rep["nstep"] == 6 and rep["critical_nodes"] == 1
    got = g.download_state()
    g.close()
    ref = _tgv(24, precision)
    ref.time_integration_rk(6)
    want = ref.download_state()
    ref.close()
    sl = (slice(H, H + 25),) * 3
    assert np.array_equal(got["q"][sl], want["q"][sl])
    assert np.array_equal(got["prs"][sl], want["prs"][sl])


def test_channel_rollback_restores_controller(gpu_lib):
    from test_gpu_channel import _case, gpu_channel
    o, dxi = _case(16, 24, 8)
    g = gpu_channel(o, dxi, capi.FP64)
    g.set_crash_control(True)
    g.time_integration_rk(7)       # backup at nstep 5
    _poison(g, (3, 4, 5))
    g.time_integration_rk(2)       # rollback to 5, then 6 and 7
    got, cs = g.download_state(), g.channel_state()
    g.close()
    r = gpu_channel(o, dxi, capi.FP64)
    r.time_integration_rk(7)
    want, cw = r.download_state(), r.channel_state()
    r.close()
    sl = (slice(H, H + 17), slice(H, H + 25), slice(H, H + 9))
    assert np.array_equal(got["q"][sl], want["q"][sl])
    assert np.array_equal(np.asarray(cs[:4]), np.asarray(cw[:4]))


def test_repeated_rollbacks_expand_critical_nodes(gpu_lib):
    g = _tgv(20)
    g.set_crash_control(True)
    g.time_integration_rk(11)      # snapshots at 5 (a) and 10 (b)
    node = (6, 7, 8)
    for expect_nstep in (6, 11, 6):  # from a, then b, then a a second time
        _poison(g, node)
        g.time_integration_rk(1)
        assert g.crash_report()["nstep"] == expect_nstep
    rep = g.crash_report()
    assert rep["rollbacks"] == 3
    # the second rollback to snapshot a expanded the mask around the node
    assert rep["critical_nodes"] == 27
    g.close()


def test_crash_without_backup_is_an_error(gpu_lib):
    g = _tgv(16)
    g.set_crash_control(True)
    _poison(g)
    with pytest.raises(capi.AstrError, match="no backup"):
        g.time_integration_rk(1)
    g.close()


def _crashfix_host(q, rho, vel, prs, tmp, im, jm, km, const2):
    """crashfix (src/mainloop.F90:1045-1198) as the reference loops: i
    fastest, each replaced node's primitives recovered before the next."""
    eps = 1e-5
    eps_p = eps * eps / const2
    wiped = 0
    for k in range(km + 1):
        for j in range(jm + 1):
            for i in range(im + 1):
                p = (H + i, H + j, H + k)
                if rho[p] >= eps and prs[p] >= eps_p and tmp[p] >= eps:
                    continue
                qa = np.zeros(5)
                norm = 0
                for kk in (-1, 0, 1):
                    for jj in (-1, 0, 1):
                        for ii in (-1, 0, 1):
                            if ii == 0 and jj == 0 and kk == 0:
                                continue
                            a, b = i + ii, j + jj
                            if a < 0 or a > im or b < 0 or b > jm:
                                continue
                            nb = (H + a, H + b, H + k + kk)
                            if rho[nb] >= 0 and prs[nb] >= 0 and tmp[nb] >= 0:
                                qa += q[nb]
                                norm += 1
                if norm >= 1:
                    q[p] = qa / norm
                    ro = q[p][0]
                    rr = 1.0 / ro
                    u, v, w = q[p][1] * rr, q[p][2] * rr, q[p][3] * rr
                    pp = (q[p][4] - 0.5 * ro * (u * u + v * v + w * w)) * 0.4
                    rho[p], prs[p], tmp[p] = ro, pp, pp * rr * const2
                    vel[p] = (u, v, w)
                    wiped += 1
    return wiped


def test_crashfix_matches_reference_loop(gpu_lib):
    from astr_gb300 import cases
    from astr_gb300.solver import GpuSolver
    n, mach = 12, 0.1
    L = 2 * np.pi
    x, y, z = cases.gridcube(n, n, n, L, L, L)
    (d11, d22, d33), J = cases.rect_metrics(x, y, z, diag_only=True)
    st = cases.tgv_state(n, n, n, x=x, y=y, z=z)
    q, rho, vel, prs, tmp = (np.array(st[k], order="F") for k in ("q", "rho", "vel", "prs", "tmp"))
    const2 = 1.4 * (mach * mach)
    # three bad nodes, two of them neighbours (the second sees the first's fix),
    # one on the i = 0 face (neighbours below i = 0 skipped), and a neighbour
    # with a negative temperature left out of the means
    for (i, j, k) in ((4, 5, 6), (5, 5, 6), (0, 3, 3)):
        rho[H + i, H + j, H + k] = 1e-7
        q[H + i, H + j, H + k, 0] = 1e-7
    tmp[H + 6, H + 6, H + 7] = -0.5
    g = GpuSolver(n, n, n, order=capi.ORDER_MAIN, mach=mach)
    g.set_metrics_diag(d11, d22, d33, J)
    g.upload_state(q, rho, vel, prs, tmp)
    g.set_crash_control(True)
    wiped = g.crashfix()
    got = g.download_state()
    g.close()
    want = _crashfix_host(q, rho, vel, prs, tmp, n, n, n, const2)
    assert wiped == want >= 3
    sl = (slice(H, H + n + 1),) * 3
    for name, ref in (("q", q), ("rho", rho), ("prs", prs), ("tmp", tmp)):
        err = np.abs(got[name][sl] - ref[sl]).max() / np.abs(ref[sl]).max()
        assert err <= 1e-14, (name, err)
