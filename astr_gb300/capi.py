"""ctypes binding of the C ABI in ``include/astr_gpu.h``.

This is the same binding a Python or Fortran (ISO_C_BINDING) host makes: plain
pointers to host arrays in the reference's Fortran layout.  The library is
the in-tree sm_103a build (``astr_gb300/_build/libastr_gb300.so``); there is
no CPU fallback, and loading fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libastr_gb300.so")

ASTR_OK = 0
ASTR_ERR_ARG = -1
ASTR_ERR_OOM = -2
ASTR_ERR_CUDA = -3
ASTR_ERR_UNSUPPORTED = -4
ASTR_ERR_NONFINITE = -5
ASTR_ERR_STATE = -6
ASTR_ERR_TIMEOUT = -7
ASTR_ERR_CANCELLED = -8

ORDER_MAIN = 0
ORDER_MINIAPP = 1
FP64 = 0
FP32_STORAGE = 1
CONSCHM_CENTRAL = 0
CONSCHM_MP = 1

# Every symbol the header declares (checked by the CPU test suite).
EXPORTS = [
    "astr_gpu_create", "astr_gpu_destroy", "astr_gpu_set_metrics", "astr_gpu_upload_state",
    "astr_gpu_download_state", "astr_gpu_download_rhs", "astr_gpu_rk3_step", "astr_gpu_filterq",
    "astr_gpu_qswap", "astr_gpu_gradcal", "astr_gpu_rhscal", "astr_gpu_updatefvar",
    "astr_gpu_reduce_stats", "astr_gpu_synchronize", "astr_gpu_last_error",
    "astr_gpu_footprint", "astr_gpu_launch_count", "astr_gpu_set_metrics_diag",
    "astr_gpu_host_alloc", "astr_gpu_host_free", "astr_gpu_timed_steps",
    "astr_gpu_set_profiling", "astr_gpu_kernel_times", "astr_gpu_measure_fp64_peak",
    "astr_gpu_stats_noalloc", "astr_gpu_set_grid", "astr_gpu_channel_state",
    "astr_gpu_boucon", "astr_gpu_step_async", "astr_gpu_poll", "astr_gpu_crashcheck",
    "astr_gpu_cflcal", "astr_gpu_upload_q", "astr_gpu_set_crash_control", "astr_gpu_databakup",
    "astr_gpu_crashfix", "astr_gpu_crash_report",
    "astr_batch_create", "astr_batch_destroy", "astr_batch_add", "astr_batch_remove",
    "astr_batch_size", "astr_batch_step_async", "astr_batch_poll", "astr_batch_wait",
    "astr_batch_cancel", "astr_batch_step", "astr_batch_last_error", "astr_batch_launch_count",
    "astr_batch_set_share", "astr_gpu_set_inflow",
]
NOALLOC_STATS_MAX_BLOCKS = 65536
KERNEL_CLASSES = ["filter", "halo", "convgrad", "visc", "pointwise", "stats", "mp"]


class AstrDims(ctypes.Structure):
    _fields_ = [("im", ctypes.c_int), ("jm", ctypes.c_int), ("km", ctypes.c_int),
                ("ia", ctypes.c_int), ("ja", ctypes.c_int), ("ka", ctypes.c_int),
                ("npdci", ctypes.c_int), ("npdcj", ctypes.c_int), ("npdck", ctypes.c_int)]


class AstrParams(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("precision", ctypes.c_int),
                ("lfilter", ctypes.c_int), ("diffterm", ctypes.c_int),
                ("alfa_filter", ctypes.c_double), ("beter_halo", ctypes.c_double),
                ("beter_bound", ctypes.c_double), ("mach", ctypes.c_double),
                ("reynolds", ctypes.c_double), ("prandtl", ctypes.c_double),
                ("ref_tem", ctypes.c_double), ("suth_const", ctypes.c_double),
                ("deltat", ctypes.c_double), ("channel", ctypes.c_int),
                ("twall", ctypes.c_double), ("conschm", ctypes.c_int),
                ("lchardecomp", ctypes.c_int), ("bfacmpld", ctypes.c_double),
                ("shkcrt", ctypes.c_double), ("bctype", ctypes.c_int * 6),
                ("twall_face", ctypes.c_double * 6), ("xslip", ctypes.c_double)]


class AstrStatus(ctypes.Structure):
    _fields_ = [("kenergy", ctypes.c_double), ("enstrophy", ctypes.c_double),
                ("crash", ctypes.c_int)]


class AstrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"astr_gpu error {code}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load the C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"astr_gb300 CUDA library not built: {path} "
                           "(run python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(path)
    vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
    L.astr_gpu_create.argtypes = [ctypes.POINTER(AstrDims), ctypes.POINTER(AstrParams),
                                  ctypes.POINTER(vp)]
    L.astr_gpu_create.restype = ip
    L.astr_gpu_destroy.argtypes = [vp]
    L.astr_gpu_destroy.restype = None
    L.astr_gpu_set_metrics.argtypes = [vp, dp, dp]
    L.astr_gpu_upload_state.argtypes = [vp, dp, dp, dp, dp, dp]
    L.astr_gpu_upload_q.argtypes = [vp, dp]
    L.astr_gpu_upload_q.restype = ip
    L.astr_gpu_download_state.argtypes = [vp, dp, dp, dp, dp, dp]
    L.astr_gpu_download_rhs.argtypes = [vp, dp, dp, dp]
    L.astr_gpu_rk3_step.argtypes = [vp, ip, dp, ctypes.POINTER(AstrStatus)]
    for n in ("astr_gpu_filterq", "astr_gpu_qswap", "astr_gpu_gradcal", "astr_gpu_rhscal",
              "astr_gpu_updatefvar", "astr_gpu_synchronize", "astr_gpu_boucon"):
        getattr(L, n).argtypes = [vp]
        getattr(L, n).restype = ip
    L.astr_gpu_reduce_stats.argtypes = [vp, dp, dp]
    L.astr_gpu_last_error.argtypes = [vp, ctypes.c_char_p, ip]
    L.astr_gpu_footprint.argtypes = [ctypes.POINTER(AstrDims), ctypes.POINTER(AstrParams)]
    L.astr_gpu_footprint.restype = ctypes.c_size_t
    L.astr_gpu_launch_count.argtypes = [vp]
    L.astr_gpu_launch_count.restype = ctypes.c_longlong
    L.astr_gpu_set_metrics_diag.argtypes = [vp, dp, dp, dp, dp]
    L.astr_gpu_set_metrics_diag.restype = ip
    L.astr_gpu_host_alloc.argtypes = [ctypes.c_size_t]
    L.astr_gpu_host_alloc.restype = vp
    L.astr_gpu_host_free.argtypes = [vp]
    L.astr_gpu_host_free.restype = None
    L.astr_gpu_timed_steps.argtypes = [vp, ip, dp]
    L.astr_gpu_timed_steps.restype = ip
    L.astr_gpu_set_profiling.argtypes = [vp, ip]
    L.astr_gpu_set_profiling.restype = ip
    L.astr_gpu_kernel_times.argtypes = [vp, dp, ctypes.POINTER(ctypes.c_longlong), ip]
    L.astr_gpu_kernel_times.restype = ip
    L.astr_gpu_measure_fp64_peak.argtypes = [dp]
    L.astr_gpu_measure_fp64_peak.restype = ip
    L.astr_gpu_stats_noalloc.argtypes = [vp, vp, vp, ctypes.POINTER(AstrDims), ctypes.c_double,
                                         vp, dp, dp]
    L.astr_gpu_stats_noalloc.restype = ip
    L.astr_gpu_crashcheck.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ip)]
    L.astr_gpu_set_crash_control.argtypes = [vp, ip]
    L.astr_gpu_set_crash_control.restype = ip
    L.astr_gpu_databakup.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_longlong)]
    L.astr_gpu_databakup.restype = ip
    L.astr_gpu_crashfix.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    L.astr_gpu_crashfix.restype = ip
    L.astr_gpu_crash_report.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    L.astr_gpu_crash_report.restype = ip
    L.astr_gpu_crashcheck.restype = ip
    L.astr_gpu_cflcal.argtypes = [vp, ctypes.c_double, dp, dp]
    L.astr_gpu_cflcal.restype = ip
    L.astr_gpu_step_async.argtypes = [vp, ip]
    L.astr_gpu_step_async.restype = ip
    L.astr_gpu_poll.argtypes = [vp]
    L.astr_gpu_poll.restype = ip
    L.astr_gpu_set_grid.argtypes = [vp, dp]
    L.astr_gpu_set_grid.restype = ip
    L.astr_gpu_set_inflow.argtypes = [vp, dp, dp, dp, dp]
    L.astr_gpu_set_inflow.restype = ip
    L.astr_gpu_channel_state.argtypes = [vp, dp]
    L.astr_gpu_channel_state.restype = ip
    L.astr_batch_create.argtypes = [ip, ctypes.POINTER(vp)]
    L.astr_batch_create.restype = ip
    L.astr_batch_destroy.argtypes = [vp]
    L.astr_batch_destroy.restype = None
    for n in ("astr_batch_add", "astr_batch_remove"):
        getattr(L, n).argtypes = [vp, vp]
        getattr(L, n).restype = ip
    for n in ("astr_batch_size", "astr_batch_poll", "astr_batch_cancel"):
        getattr(L, n).argtypes = [vp]
        getattr(L, n).restype = ip
    L.astr_batch_set_share.argtypes = [vp, ctypes.c_double]
    L.astr_batch_set_share.restype = ip
    L.astr_batch_step_async.argtypes = [vp, ip, ctypes.c_double]
    L.astr_batch_step_async.restype = ip
    L.astr_batch_wait.argtypes = [vp, ctypes.POINTER(ip)]
    L.astr_batch_wait.restype = ip
    L.astr_batch_step.argtypes = [vp, ip, ctypes.c_double, ctypes.POINTER(ip)]
    L.astr_batch_step.restype = ip
    L.astr_batch_last_error.argtypes = [vp, ctypes.c_char_p, ip]
    L.astr_batch_last_error.restype = ip
    L.astr_batch_launch_count.argtypes = [vp]
    L.astr_batch_launch_count.restype = ctypes.c_longlong
    for n in ("astr_gpu_set_metrics", "astr_gpu_upload_state", "astr_gpu_download_state",
              "astr_gpu_download_rhs", "astr_gpu_rk3_step", "astr_gpu_reduce_stats"):
        getattr(L, n).restype = ip
    _lib = L
    return L


def dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64
    assert a.flags.f_contiguous or a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class PinnedArray:
    """A numpy array over page-locked host memory (astr_gpu_host_alloc)."""

    def __init__(self, shape, dtype=np.float64, order="F"):
        L = load()
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = L.astr_gpu_host_alloc(self.nbytes)
        if not self.ptr:
            raise MemoryError(f"astr_gpu_host_alloc({self.nbytes}) failed")
        buf = (ctypes.c_char * self.nbytes).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape, order=order)

    def free(self):
        if self.ptr:
            self.array = None
            load().astr_gpu_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def last_error(h) -> str:
    L = load()
    buf = ctypes.create_string_buffer(1024)
    L.astr_gpu_last_error(h, buf, 1024)
    return buf.value.decode(errors="replace")


def check(h, rc: int):
    if rc != ASTR_OK:
        raise AstrError(rc, last_error(h))
    return rc


def batch_error(b) -> str:
    L = load()
    buf = ctypes.create_string_buffer(1024)
    L.astr_batch_last_error(b, buf, 1024)
    return buf.value.decode(errors="replace")


class Batch:
    """A batch of cases stepped together (astr_batch_*): one launch per phase
    of an RK3 stage covers every case; each case advances as it would alone.

    Cases are GpuSolver objects (or anything with a context handle ``h``)."""

    def __init__(self, precision: int = FP32_STORAGE):
        L = load()
        self.L = L
        h = ctypes.c_void_p()
        rc = L.astr_batch_create(precision, ctypes.byref(h))
        if rc != ASTR_OK:
            raise AstrError(rc, last_error(None))
        self.h = h
        self.members = []

    def _c(self, rc: int):
        if rc != ASTR_OK:
            raise AstrError(rc, batch_error(self.h))
        return rc

    def add(self, case):
        self._c(self.L.astr_batch_add(self.h, case.h))
        self.members.append(case)

    def remove(self, case):
        self._c(self.L.astr_batch_remove(self.h, case.h))
        self.members.remove(case)

    def __len__(self):
        return self.L.astr_batch_size(self.h)

    def set_share(self, share: float):
        """Fraction (0, 1] of the GPU's resident blocks a launch takes."""
        self._c(self.L.astr_batch_set_share(self.h, float(share)))

    def step_async(self, nsteps: int, budget_ms: float = 0.0):
        self._c(self.L.astr_batch_step_async(self.h, nsteps, budget_ms))

    def poll(self) -> bool:
        rc = self.L.astr_batch_poll(self.h)
        if rc < 0:
            self._c(rc)
        return rc == 1

    def wait(self):
        """(code, steps_done): code is ASTR_OK, ASTR_ERR_TIMEOUT or
        ASTR_ERR_CANCELLED; other errors raise."""
        n = ctypes.c_int(0)
        rc = self.L.astr_batch_wait(self.h, ctypes.byref(n))
        if rc not in (ASTR_OK, ASTR_ERR_TIMEOUT, ASTR_ERR_CANCELLED):
            self._c(rc)
        return rc, n.value

    def step(self, nsteps: int, budget_ms: float = 0.0):
        self.step_async(nsteps, budget_ms)
        return self.wait()

    def cancel(self):
        self._c(self.L.astr_batch_cancel(self.h))

    @property
    def launches(self) -> int:
        return self.L.astr_batch_launch_count(self.h)

    def close(self):
        if self.h:
            self.L.astr_batch_destroy(self.h)
            self.h = None
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
