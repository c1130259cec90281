"""ORACLE — test infrastructure only.

ctypes binding of the C++ restatement of the ASTR right-hand-side hot path
(``astr_oracle.cpp``).  Only the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module; the GPU product never
does.

Arrays are exposed as numpy views in the reference's Fortran layout:
halo arrays have shape ``(im+11, jm+11, km+11[, n])`` with ``order='F'`` and
index ``i+5`` for Fortran index ``i``; interior arrays have shape
``(im+1, jm+1, km+1[, n])``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liborc.so")
HM = 5

MODE_MAIN = 0
MODE_MINIAPP = 1


def build(force: bool = False) -> str:
    """Compile the oracle library (strict FP64: no FMA contraction)."""
    src = os.path.join(HERE, "astr_oracle.cpp")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(src)
            and os.path.getmtime(LIB) >= os.path.getmtime(os.path.join(HERE, "astr_oracle.h"))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-std=c++17", "-o", LIB + ".tmp", src]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class OrcConfig(ctypes.Structure):
    _fields_ = [
        ("im", ctypes.c_int), ("jm", ctypes.c_int), ("km", ctypes.c_int),
        ("ia", ctypes.c_int), ("ja", ctypes.c_int), ("ka", ctypes.c_int),
        ("npdci", ctypes.c_int), ("npdcj", ctypes.c_int), ("npdck", ctypes.c_int),
        ("mode", ctypes.c_int), ("lfilter", ctypes.c_int), ("diffterm", ctypes.c_int),
        ("channel", ctypes.c_int),
        ("alfa_filter", ctypes.c_double), ("beter_halo", ctypes.c_double),
        ("beter_bound", ctypes.c_double),
        ("mach", ctypes.c_double), ("reynolds", ctypes.c_double),
        ("prandtl", ctypes.c_double), ("ref_tem", ctypes.c_double),
        ("suth_const", ctypes.c_double), ("deltat", ctypes.c_double),
        ("twall", ctypes.c_double),
        ("conschm_mp", ctypes.c_int), ("lchardecomp", ctypes.c_int),
        ("bfacmpld", ctypes.c_double), ("shkcrt", ctypes.c_double),
        ("bctype", ctypes.c_int * 6), ("twall6", ctypes.c_double * 6),
        ("xslip", ctypes.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.POINTER(OrcConfig)]
        L.orc_destroy.argtypes = [vp]
        L.orc_field.restype = dp
        L.orc_field.argtypes = [vp, ctypes.c_char_p]
        L.orc_scheme.restype = ctypes.c_int
        L.orc_scheme.argtypes = [vp, ctypes.c_int, ctypes.c_int, ip, dp, ctypes.c_int]
        L.orc_filter_tables.argtypes = [vp, dp, dp, dp, dp, dp]
        L.orc_constants.argtypes = [vp, dp]
        L.orc_gridcube.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        for name in ("orc_gridgeom", "orc_init_tgv", "orc_updateq", "orc_filterq", "orc_qswap",
                     "orc_boucon", "orc_gradcal", "orc_convrsdcal6", "orc_diffrsdcal6",
                     "orc_rhscal", "orc_updatefvar", "orc_bchomo"):
            getattr(L, name).argtypes = [vp]
        L.orc_chan_state.argtypes = [vp, dp]
        L.orc_rk3_step.argtypes = [vp, dp]
        L.orc_rk3_steps.argtypes = [vp, ctypes.c_int, dp]
        L.orc_line_derivative.argtypes = [vp, ctypes.c_int, dp, dp]
        L.orc_line_filter.argtypes = [vp, ctypes.c_int, dp, dp]
        L.orc_kenergy.restype = ctypes.c_double
        L.orc_kenergy.argtypes = [vp]
        L.orc_enstrophy.restype = ctypes.c_double
        L.orc_enstrophy.argtypes = [vp]
        for name in ("orc_ducrossensor", "orc_convrsdcmp"):
            getattr(L, name).argtypes = [vp]
        L.orc_lshock.argtypes = [vp, ctypes.c_void_p]
        L.orc_lshock.restype = ctypes.c_int
        L.orc_line_flux.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, dp]
        L.orc_mp5.argtypes = [dp, ctypes.c_double, ctypes.c_int]
        L.orc_mp5.restype = ctypes.c_double
        L.orc_steger_warming.argtypes = [vp, dp, dp, dp, ctypes.c_double, dp, dp]
        L.orc_chardecomp.argtypes = [dp, dp, dp, dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.flags.c_contiguous)
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


HALO_FIELDS = {"q": 5, "rho": 0, "vel": 3, "prs": 0, "tmp": 0, "x": 3, "dxi": 9,
               "jacob": 0, "sigma": 6, "qflux": 3, "ssf": 0}
INTERIOR_FIELDS = {"qrhs": 5, "qsave": 5, "dvel": 9, "dtmp": 3}


class Oracle:
    """One reference-restatement context (module state of one ASTR rank)."""

    def __init__(self, im, jm, km, *, mode=MODE_MAIN, npdc=(3, 3, 3), lfilter=True,
                 diffterm=True, alfa_filter=0.49, beter_halo=1.11, beter_bound=0.98,
                 mach=0.1, reynolds=1600.0, prandtl=0.72, ref_tem=273.15,
                 suth_const=None, deltat=1e-3, ia=None, ja=None, ka=None, channel=False,
                 twall=1.0, conschm="643c", lchardecomp=True, bfacmpld=0.3, shkcrt=0.01,
                 bctype=(0, 0, 0, 0, 0, 0), twall6=(0.0,) * 6, xslip=0.0):
        if suth_const is None:
            suth_const = 110.4 if mode == MODE_MINIAPP else 110.3
        self.cfg = OrcConfig(im, jm, km, im if ia is None else ia, jm if ja is None else ja,
                             km if ka is None else ka, npdc[0], npdc[1], npdc[2], mode,
                             int(lfilter), int(diffterm), int(channel), alfa_filter,
                             beter_halo, beter_bound, mach, reynolds, prandtl, ref_tem,
                             suth_const, deltat, twall, int(conschm == "543c"),
                             int(lchardecomp), bfacmpld, shkcrt,
                             (ctypes.c_int * 6)(*bctype), (ctypes.c_double * 6)(*twall6),
                             xslip)
        if conschm not in ("643c", "543c"):
            raise ValueError(f"conschm {conschm!r}: 643c (central) or 543c (compact MP)")
        self.L = lib()
        self.h = self.L.orc_create(ctypes.byref(self.cfg))
        self.im, self.jm, self.km = im, jm, km
        self.mode = mode

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- array views ------------------------------------------------------
    def field(self, name: str) -> np.ndarray:
        p = self.L.orc_field(self.h, name.encode())
        if name in HALO_FIELDS:
            n = HALO_FIELDS[name]
            shape = (self.im + 2 * HM + 1, self.jm + 2 * HM + 1, self.km + 2 * HM + 1)
        else:
            n = INTERIOR_FIELDS[name]
            shape = (self.im + 1, self.jm + 1, self.km + 1)
        if n:
            shape = shape + (n,)
        count = int(np.prod(shape))
        buf = np.ctypeslib.as_array(p, shape=(count,))
        return buf.reshape(shape, order="F")

    def inflow(self):
        """Views of the inflow arrays of bctypes 11 and 12 (freestream values
        until set): vel_in (jm+1, km+1, 3), tmp_in (jm+1, km+1), tmp_prof
        (jm+1), prs_in (jm+1, km+1)."""
        nj, nk = self.jm + 1, self.km + 1
        out = {}
        for name, shape in (("vel_in", (nj, nk, 3)), ("tmp_in", (nj, nk)), ("tmp_prof", (nj,)),
                            ("prs_in", (nj, nk))):
            p = self.L.orc_field(self.h, name.encode())
            buf = np.ctypeslib.as_array(p, shape=(int(np.prod(shape)),))
            out[name] = buf.reshape(shape, order="F")
        return out

    def scheme(self, d: int, kind: int):
        first = ctypes.c_int()
        out = np.zeros(5 * 4200)
        n = self.L.orc_scheme(self.h, d, kind, ctypes.byref(first), _dptr(out), out.size)
        a = out[: 5 * n].reshape(5, n)
        return first.value, a

    def filter_tables(self):
        c10, c8, c6 = np.zeros(6), np.zeros(5), np.zeros(4)
        cb, ch = np.zeros(45), np.zeros(55)
        self.L.orc_filter_tables(self.h, _dptr(c10), _dptr(c8), _dptr(c6), _dptr(cb), _dptr(ch))
        return c10, c8, c6, cb.reshape(5, 9, order="F"), ch.reshape(5, 11, order="F")

    def constants(self):
        o = np.zeros(9)
        self.L.orc_constants(self.h, _dptr(o))
        return o

    # -- reference routines -------------------------------------------------
    def gridcube(self, lx, ly, lz):
        self.L.orc_gridcube(self.h, lx, ly, lz)

    def set_grid(self, x, y, z):
        """Rectilinear node coordinates x(0:im), y(0:jm), z(0:km) into the
        interior of the coordinate array (gridgeom fills the halos)."""
        X = self.field("x")
        h = HM
        sl = (slice(h, h + self.im + 1), slice(h, h + self.jm + 1), slice(h, h + self.km + 1))
        X[sl + (0,)] = np.asarray(x).reshape(-1, 1, 1)
        X[sl + (1,)] = np.asarray(y).reshape(1, -1, 1)
        X[sl + (2,)] = np.asarray(z).reshape(1, 1, -1)

    def chan_state(self):
        """(force(1), mass flux, target mass flux, wall friction, steps)."""
        out = np.zeros(5)
        self.L.orc_chan_state(self.h, _dptr(out))
        return out

    def call(self, name: str):
        getattr(self.L, "orc_" + name)(self.h)

    def rk3_steps(self, n: int) -> np.ndarray:
        st = np.zeros(2 * n)
        self.L.orc_rk3_steps(self.h, n, _dptr(st))
        return st.reshape(n, 2)

    def kenergy(self):
        return self.L.orc_kenergy(self.h)

    def enstrophy(self):
        return self.L.orc_enstrophy(self.h)

    def line_derivative(self, d: int, f: np.ndarray) -> np.ndarray:
        dim = (self.im, self.jm, self.km)[d]
        f = np.ascontiguousarray(f, dtype=np.float64)
        assert f.size == dim + 2 * HM + 1
        out = np.zeros(dim + 1)
        self.L.orc_line_derivative(self.h, d, _dptr(f), _dptr(out))
        return out

    def line_filter(self, d: int, f: np.ndarray) -> np.ndarray:
        dim = (self.im, self.jm, self.km)[d]
        f = np.ascontiguousarray(f, dtype=np.float64)
        assert f.size == dim + 2 * HM + 1
        out = np.zeros(dim + 1)
        self.L.orc_line_filter(self.h, d, _dptr(f), _dptr(out))
        return out

    # -- compact MP path ----------------------------------------------------
    def lshock(self):
        """lshock(0:im,0:jm,0:km) as a bool array, None before the sensor ran."""
        out = np.zeros((self.im + 1) * (self.jm + 1) * (self.km + 1), dtype=np.uint8)
        ok = self.L.orc_lshock(self.h, out.ctypes.data_as(ctypes.c_void_p))
        if not ok:
            return None
        return out.reshape((self.im + 1, self.jm + 1, self.km + 1), order="F").astype(bool)

    def line_flux(self, d: int, wind: int, f: np.ndarray) -> np.ndarray:
        """Compact upwind (wind=+1) / downwind (-1) interface flux fh(-1..dim)."""
        dim = (self.im, self.jm, self.km)[d]
        f = np.ascontiguousarray(f, dtype=np.float64)
        assert f.size == dim + 2 * HM + 1
        out = np.zeros(dim + 2)
        self.L.orc_line_flux(self.h, d, int(wind), _dptr(f), _dptr(out))
        return out

    def steger_warming(self, prim, q5, dxi3, jac):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        q5 = np.ascontiguousarray(q5, dtype=np.float64)
        dxi3 = np.ascontiguousarray(dxi3, dtype=np.float64)
        fp, fm = np.zeros(5), np.zeros(5)
        self.L.orc_steger_warming(self.h, _dptr(prim), _dptr(q5), _dptr(dxi3), float(jac),
                                  _dptr(fp), _dptr(fm))
        return fp, fm


def mp5(u5, ul, discont=True) -> float:
    u5 = np.ascontiguousarray(u5, dtype=np.float64)
    return lib().orc_mp5(_dptr(u5), float(ul), int(bool(discont)))


def chardecomp(stl, str_):
    """REV, LEV (5x5) between two node states {T,rho,p,E,u,v,w,dxi1..3}."""
    a = np.ascontiguousarray(stl, dtype=np.float64)
    b = np.ascontiguousarray(str_, dtype=np.float64)
    R, L = np.zeros(25), np.zeros(25)
    lib().orc_chardecomp(_dptr(a), _dptr(b), _dptr(R), _dptr(L))
    return R.reshape(5, 5, order="F"), L.reshape(5, 5, order="F")


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return lib().orc_get_threads()


def tgv_main(n: int, **kw) -> Oracle:
    """Main-solver TGV case: gridcube(2*pi)^3, gridgeom, tgvini + updateq."""
    o = Oracle(n, n, n, mode=MODE_MAIN, **kw)
    L = 2.0 * np.pi
    o.gridcube(L, L, L)
    o.call("gridgeom")
    o.call("init_tgv")
    return o


def tgv_miniapp(n: int, **kw) -> Oracle:
    """Mini-app TGV case (miniapps/tgv_solver_3d/tgvsolver.F90)."""
    kw.setdefault("beter_bound", 1.09)
    o = Oracle(n, n, n, mode=MODE_MINIAPP, **kw)
    o.call("init_tgv")
    return o


def from_state(st, dims, *, lx=None, ly=None, lz=None, grid=None, **kw) -> Oracle:
    """An oracle case on a gridcube box (lx, ly, lz), or on the rectilinear
    grid = (x, y, z), with metrics from gridgeom and the given halo-layout
    state (q, rho, vel, prs, tmp) written into its interior nodes (the
    filter's own halo swaps fill the halos)."""
    im, jm, km = dims
    o = Oracle(im, jm, km, mode=MODE_MAIN, **kw)
    if grid is not None:
        o.set_grid(*grid)
    else:
        o.gridcube(lx, ly, lz)
    o.call("gridgeom")
    for name in ("q", "rho", "vel", "prs", "tmp"):
        o.field(name)[...] = st[name]
    return o
