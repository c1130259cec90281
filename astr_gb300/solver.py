"""Host-side mirror of the ASTR module interface for the RHS hot path.

ASTR's time loop calls argument-less module routines on module arrays
(``filterq``, ``qswap``, ``gradcal``, ``rhscal``, ``updatefvar``; the stage
loop ``time_integration_rk``, src/mainloop.F90:301-601).  ``GpuSolver`` keeps
the same routine names, with the module state resident in HBM behind the C
ABI of ``include/astr_gpu.h``.  Host arrays use the reference's Fortran
layout: halo arrays ``(im+11, jm+11, km+11[, n])`` in Fortran order.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi

HM = 5


def halo_shape(im, jm, km, n=None):
    s = (im + 2 * HM + 1, jm + 2 * HM + 1, km + 2 * HM + 1)
    return s + (n,) if n else s


def interior_shape(im, jm, km, n=None):
    s = (im + 1, jm + 1, km + 1)
    return s + (n,) if n else s


def _f(a, shape):
    a = np.asarray(a, dtype=np.float64)
    if a.shape != shape and a.size == int(np.prod(shape)) and a.shape[:3] == shape[:3]:
        # trailing component axes given flattened, e.g. dxi(...,9) for dxi(...,3,3)
        a = np.asfortranarray(a).reshape(shape, order="F")
    if a.shape != shape:
        raise ValueError(f"array shape {a.shape}, expected {shape}")
    return np.asfortranarray(a)


class GpuSolver:
    """One single-rank block of the ASTR solver resident on one GPU."""

    def __init__(self, im, jm, km, *, order=capi.ORDER_MAIN, precision=capi.FP64,
                 npdc=(3, 3, 3), lfilter=True, diffterm=True, alfa_filter=0.49,
                 beter_halo=1.11, beter_bound=0.98, mach=0.1, reynolds=1600.0, prandtl=0.72,
                 ref_tem=273.15, suth_const=None, deltat=1e-3, ia=None, ja=None, ka=None,
                 channel=False, twall=1.0, conschm="643c", lchardecomp=True, bfacmpld=0.3,
                 shkcrt=0.01, bctype=(0, 0, 0, 0, 0, 0), twall_face=(0.0,) * 6, xslip=0.0):
        """The keywords are the fields of ``astr_params`` under the reference's
        names: npdc = (npdci, npdcj, npdck), 3 periodic, 4 both ends physical;
        conschm "643c" (central) or "543c" (compact MP, with lchardecomp,
        bfacmpld, shkcrt); bctype, the routine of each face (xmin, xmax, ymin,
        ymax, zmin, zmax; 21, 41, 42, 411, 421, 50, 51, 60, 0/1 none) with
        twall_face (0: twall) for the isothermal faces and xslip for 411,
        whose slip region needs set_grid; channel for the channel flow."""
        L = capi.load()
        if conschm not in ("643c", "543c"):
            raise ValueError(f"conschm {conschm!r}: 643c (central) or 543c (compact MP)")
        if suth_const is None:
            suth_const = 110.4 if order == capi.ORDER_MINIAPP else 110.3
        self.im, self.jm, self.km = im, jm, km
        self.dims = capi.AstrDims(im, jm, km, im if ia is None else ia, jm if ja is None else ja,
                                  km if ka is None else ka, *npdc)
        self.params = capi.AstrParams(order, precision, int(lfilter), int(diffterm), alfa_filter,
                                      beter_halo, beter_bound, mach, reynolds, prandtl, ref_tem,
                                      suth_const, deltat, int(channel), twall,
                                      capi.CONSCHM_MP if conschm == "543c" else capi.CONSCHM_CENTRAL,
                                      int(lchardecomp), bfacmpld, shkcrt,
                                      (ctypes.c_int * 6)(*bctype),
                                      (ctypes.c_double * 6)(*twall_face), xslip)
        h = ctypes.c_void_p()
        rc = L.astr_gpu_create(ctypes.byref(self.dims), ctypes.byref(self.params), ctypes.byref(h))
        if rc != capi.ASTR_OK:
            raise capi.AstrError(rc, capi.last_error(None))
        self.h = h
        self.L = L

    # -- lifecycle --------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.L.astr_gpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        return capi.check(self.h, rc)

    # -- data movement ----------------------------------------------------
    def set_metrics(self, dxi, jacob):
        im, jm, km = self.im, self.jm, self.km
        dxi = _f(dxi, halo_shape(im, jm, km) + (3, 3))
        jacob = _f(jacob, halo_shape(im, jm, km))
        self._c(self.L.astr_gpu_set_metrics(self.h, capi.dptr(dxi), capi.dptr(jacob)))

    def set_metrics_diag(self, dxi11, dxi22, dxi33, jacob):
        shp = halo_shape(self.im, self.jm, self.km)
        arrs = [_f(a, shp) for a in (dxi11, dxi22, dxi33, jacob)]
        self._c(self.L.astr_gpu_set_metrics_diag(self.h, *(capi.dptr(a) for a in arrs)))

    def set_grid(self, x):
        """Node coordinates x(-hm:..,1:3) (halo layout, Fortran order), or
        the rectilinear node vectors (x, y, z) of the interior, which are
        laid out with gridgeom's single-rank halo extension."""
        if isinstance(x, (tuple, list)):
            from .cases import grid_halo
            x = grid_halo(*x)
        x = _f(x, halo_shape(self.im, self.jm, self.km, 3))
        self._c(self.L.astr_gpu_set_grid(self.h, capi.dptr(x)))

    def set_inflow(self, vel_in=None, tmp_in=None, tmp_prof=None, prs_in=None):
        """Inflow arrays of bctypes 11 and 12 on xmin: vel_in (jm+1, km+1,
        3), tmp_in (jm+1, km+1), tmp_prof (jm+1), prs_in (jm+1, km+1);
        None takes the freestream values."""
        nj, nk = self.jm + 1, self.km + 1
        args = []
        for a, shape in ((vel_in, (nj, nk, 3)), (tmp_in, (nj, nk)), (tmp_prof, (nj,)),
                         (prs_in, (nj, nk))):
            if a is None:
                args.append(None)
                continue
            a = np.asarray(a, dtype=np.float64)
            if a.shape != shape:
                raise ValueError(f"inflow array of shape {a.shape}, want {shape}")
            args.append(np.asfortranarray(a))
        self._c(self.L.astr_gpu_set_inflow(self.h, *(capi.dptr(a) for a in args)))

    def channel_state(self):
        """(force(1), mass flux, target mass flux, wall friction, steps)."""
        out = np.zeros(5)
        self._c(self.L.astr_gpu_channel_state(self.h, capi.dptr(out)))
        return out

    def upload_state(self, q, rho, vel, prs, tmp):
        im, jm, km = self.im, self.jm, self.km
        q = _f(q, halo_shape(im, jm, km, 5))
        rho = _f(rho, halo_shape(im, jm, km))
        vel = _f(vel, halo_shape(im, jm, km, 3))
        prs = _f(prs, halo_shape(im, jm, km))
        tmp = _f(tmp, halo_shape(im, jm, km))
        self._c(self.L.astr_gpu_upload_state(self.h, capi.dptr(q), capi.dptr(rho), capi.dptr(vel),
                                             capi.dptr(prs), capi.dptr(tmp)))

    def upload_q(self, q):
        """Upload q alone; the interior primitives are recomputed on the
        device (updatefvar)."""
        q = _f(q, halo_shape(self.im, self.jm, self.km, 5))
        self._c(self.L.astr_gpu_upload_q(self.h, capi.dptr(q)))

    def download_state(self):
        im, jm, km = self.im, self.jm, self.km
        out = {
            "q": np.zeros(halo_shape(im, jm, km, 5), order="F"),
            "rho": np.zeros(halo_shape(im, jm, km), order="F"),
            "vel": np.zeros(halo_shape(im, jm, km, 3), order="F"),
            "prs": np.zeros(halo_shape(im, jm, km), order="F"),
            "tmp": np.zeros(halo_shape(im, jm, km), order="F"),
        }
        self._c(self.L.astr_gpu_download_state(self.h, *(capi.dptr(out[k]) for k in
                                                          ("q", "rho", "vel", "prs", "tmp"))))
        return out

    def download_rhs(self):
        im, jm, km = self.im, self.jm, self.km
        out = {
            "qrhs": np.zeros(interior_shape(im, jm, km, 5), order="F"),
            "dvel": np.zeros(interior_shape(im, jm, km) + (3, 3), order="F"),
            "dtmp": np.zeros(interior_shape(im, jm, km, 3), order="F"),
        }
        self._c(self.L.astr_gpu_download_rhs(self.h, capi.dptr(out["qrhs"]), capi.dptr(out["dvel"]),
                                             capi.dptr(out["dtmp"])))
        return out

    # -- reference routines -------------------------------------------------
    def time_integration_rk(self, nsteps: int = 1, stats: bool = True):
        """nsteps RK3 steps; returns the (nsteps, 2) kinetic-energy /
        enstrophy history sampled at stage 1 of each step."""
        hist = np.zeros(2 * max(nsteps, 1))
        st = capi.AstrStatus()
        self._c(self.L.astr_gpu_rk3_step(self.h, int(nsteps), capi.dptr(hist) if stats else None,
                                         ctypes.byref(st)))
        return hist[: 2 * nsteps].reshape(nsteps, 2)

    def filterq(self):
        self._c(self.L.astr_gpu_filterq(self.h))

    def qswap(self):
        self._c(self.L.astr_gpu_qswap(self.h))

    def gradcal(self):
        self._c(self.L.astr_gpu_gradcal(self.h))

    def rhscal(self):
        self._c(self.L.astr_gpu_rhscal(self.h))

    def crashcheck(self):
        """(number of interior nodes with rho < 0 or NaN, first such (i, j, k)
        or None) — crashcheck, src/mainloop.F90:709-812."""
        n = ctypes.c_longlong()
        ijk = (ctypes.c_int * 3)()
        self._c(self.L.astr_gpu_crashcheck(self.h, ctypes.byref(n), ijk))
        return n.value, (tuple(ijk) if n.value else None)

    def set_crash_control(self, on: bool = True):
        """lcracon: crashcheck / databakup before every step and crashfix
        after every stage of time_integration_rk (src/mainloop.F90:709-1198)."""
        self._c(self.L.astr_gpu_set_crash_control(self.h, 1 if on else 0))

    def databakup(self, mode: str) -> int:
        """databakup('backup' or 'recovery'); returns nstep after the call."""
        n = ctypes.c_longlong()
        self._c(self.L.astr_gpu_databakup(self.h, {"backup": 0, "recovery": 1}[mode], ctypes.byref(n)))
        return n.value

    def crashfix(self) -> int:
        """One crashfix pass; returns the number of nodes it replaced."""
        n = ctypes.c_longlong()
        self._c(self.L.astr_gpu_crashfix(self.h, ctypes.byref(n)))
        return n.value

    def crash_report(self) -> dict:
        out = (ctypes.c_longlong * 6)()
        self._c(self.L.astr_gpu_crash_report(self.h, out))
        keys = ("rollbacks", "backups", "wiped", "critical_nodes", "nstep", "next_backup")
        return dict(zip(keys, (int(v) for v in out)))

    def cflcal(self, deltat: float):
        """(CFL number of the resident state at this time step, (Di, Dj, Dk))
        — cflcal, src/commcal.F90:27-87."""
        cfl = ctypes.c_double()
        d3 = np.zeros(3)
        self._c(self.L.astr_gpu_cflcal(self.h, float(deltat), ctypes.byref(cfl), capi.dptr(d3)))
        return cfl.value, d3

    def boucon(self):
        self._c(self.L.astr_gpu_boucon(self.h))

    def updatefvar(self):
        self._c(self.L.astr_gpu_updatefvar(self.h))

    def reduce_stats(self):
        ke, en = ctypes.c_double(), ctypes.c_double()
        self._c(self.L.astr_gpu_reduce_stats(self.h, ctypes.byref(ke), ctypes.byref(en)))
        return ke.value, en.value

    def timed_steps(self, nsteps: int) -> float:
        """Device milliseconds of nsteps RK3 steps (CUDA events on the
        context's stream, no statistics)."""
        ms = ctypes.c_double()
        self._c(self.L.astr_gpu_timed_steps(self.h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def step_async(self, nsteps: int):
        """Enqueue nsteps RK3 steps (one CUDA graph launch each) and return
        without waiting."""
        self._c(self.L.astr_gpu_step_async(self.h, int(nsteps)))

    def poll(self) -> bool:
        """True when every enqueued step has finished."""
        rc = self.L.astr_gpu_poll(self.h)
        if rc < 0:
            self._c(rc)
        return rc == 1

    def set_profiling(self, on: bool):
        self._c(self.L.astr_gpu_set_profiling(self.h, int(on)))

    def kernel_times(self):
        n = len(capi.KERNEL_CLASSES)
        ms = np.zeros(n)
        cnt = (ctypes.c_longlong * n)()
        rc = self.L.astr_gpu_kernel_times(self.h, capi.dptr(ms), cnt, n)
        if rc < 0:
            capi.check(self.h, rc)
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(capi.KERNEL_CLASSES)}

    def synchronize(self):
        self._c(self.L.astr_gpu_synchronize(self.h))

    @property
    def launches(self) -> int:
        return int(self.L.astr_gpu_launch_count(self.h))
