"""The C-ABI library: it builds for sm_103a, loads, and exports every entry
point include/astr_gpu.h declares.  No compute call needs a GPU here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "astr_gpu.h")).read()
    return sorted(set(re.findall(r"\b(astr_(?:gpu|batch)_\w+)\s*\(", src)))


def test_exports_every_declared_symbol(gpu_lib):
    from astr_gb300 import capi
    syms = header_symbols()
    assert syms, "no declarations found"
    missing = [s for s in syms if not hasattr(gpu_lib, s)]
    assert not missing, missing
    assert sorted(capi.EXPORTS) == syms


def test_footprint_without_gpu(gpu_lib):
    from astr_gb300 import capi
    d = capi.AstrDims(512, 512, 512, 512, 512, 512, 3, 3, 3)
    p = capi.AstrParams()
    nbytes = gpu_lib.astr_gpu_footprint(ctypes.byref(d), ctypes.byref(p))
    assert 40e9 < nbytes < 80e9


def test_create_rejects_bad_dims(gpu_lib):
    from astr_gb300 import capi
    d = capi.AstrDims(4, 4, 4, 4, 4, 4, 3, 3, 3)
    p = capi.AstrParams(0, 0, 1, 1, 0.49, 1.11, 0.98, 0.1, 1600.0, 0.72, 273.15, 110.3, 1e-3)
    h = ctypes.c_void_p()
    rc = gpu_lib.astr_gpu_create(ctypes.byref(d), ctypes.byref(p), ctypes.byref(h))
    assert rc == capi.ASTR_ERR_ARG
    assert "too small" in capi.last_error(None)


def _params(**kw):
    from astr_gb300 import capi
    p = capi.AstrParams(0, 0, 1, 1, 0.49, 1.11, 0.98, 0.1, 1600.0, 0.72, 273.15, 110.3, 1e-3)
    for k, v in kw.items():
        if k == "bctype":
            p.bctype = (ctypes.c_int * 6)(*v)
        else:
            setattr(p, k, v)
    return p


@pytest.mark.parametrize("npdc, kw, code, text", [
    ((3, 3, 3), dict(bctype=(41, 0, 0, 0, 0, 0), twall=1.0), "ARG", "npdc = 4"),
    ((3, 3, 4), dict(bctype=(0, 0, 0, 0, 42, 0)), "UNSUPPORTED", "x and y faces"),
    ((4, 3, 3), dict(bctype=(22, 21, 0, 0, 0, 0)), "UNSUPPORTED", "bctype"),
    ((4, 4, 3), dict(bctype=(12, 21, 0, 0, 0, 0)), "UNSUPPORTED", "periodic y and z"),
    ((4, 4, 3), dict(bctype=(0, 0, 11, 0, 0, 0)), "UNSUPPORTED", "xmin"),
    ((4, 3, 3), dict(bctype=(421, 0, 0, 0, 0, 0)), "UNSUPPORTED", "y faces"),
    ((4, 3, 3), dict(bctype=(0, 411, 0, 0, 0, 0), twall=1.0), "UNSUPPORTED", "y faces"),
    ((3, 4, 3), dict(bctype=(0, 0, 411, 0, 0, 0), twall=0.0), "ARG", "wall temperature"),
    ((4, 3, 3), dict(bctype=(21, 0, 0, 0, 0, 0)), "UNSUPPORTED", "xmax and ymax"),
    ((4, 3, 3), dict(bctype=(0, 51, 0, 0, 0, 0)), "UNSUPPORTED", "y and z faces"),
    ((4, 3, 3), dict(bctype=(41, 0, 0, 0, 0, 0), twall=0.0), "ARG", "wall temperature"),
    ((3, 3, 3), dict(conschm=1, precision=1), "UNSUPPORTED", "FP64"),
    ((3, 3, 3), dict(conschm=7), "ARG", "conschm"),
])
def test_create_checks_without_gpu(gpu_lib, npdc, kw, code, text):
    """Boundary routines and the convective scheme are checked before any
    device call: the context is refused on a machine without a GPU too."""
    from astr_gb300 import capi
    d = capi.AstrDims(16, 16, 16, 16, 16, 16, *npdc)
    p = _params(**kw)
    h = ctypes.c_void_p()
    rc = gpu_lib.astr_gpu_create(ctypes.byref(d), ctypes.byref(p), ctypes.byref(h))
    assert rc == getattr(capi, "ASTR_ERR_" + code), (rc, capi.last_error(None))
    assert text in capi.last_error(None)


C_HOST = r"""
#include "astr_gpu.h"
#include <stdio.h>
int main(void) {
  astr_dims d = {512, 512, 512, 512, 512, 512, 3, 3, 3};
  astr_params p = {0};
  astr_dims bad = {4, 4, 4, 4, 4, 4, 3, 3, 3};
  astr_ctx* c = NULL;
  char buf[256];
  int rc;
  printf("footprint %zu\n", astr_gpu_footprint(&d, &p));
  p.mach = 0.1; p.reynolds = 1600.0; p.deltat = 1e-3; p.alfa_filter = 0.49;
  rc = astr_gpu_create(&bad, &p, &c);
  astr_gpu_last_error(NULL, buf, (int)sizeof buf);
  printf("create %d %s\n", rc, buf);
  return c == NULL ? 0 : 1;
}
"""


def test_plain_c_host(gpu_lib, tmp_path):
    """The header is strict C99 (a C or Fortran host includes or mirrors
    it) and a C program links the library and calls it without a GPU."""
    import shutil
    import subprocess
    from astr_gb300 import capi
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    src = tmp_path / "host.c"
    src.write_text(C_HOST)
    exe = tmp_path / "host"
    libdir = os.path.dirname(capi.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    "-I", os.path.join(ROOT, "include"), str(src), "-L", libdir, "-lastr_gb300",
                    "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    lines = out.splitlines()
    assert 40e9 < int(lines[0].split()[1]) < 80e9
    assert lines[1].startswith(f"create {capi.ASTR_ERR_ARG} grid too small")


C_HOST_NULLS = r"""
#include "astr_gpu.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
/* Every nullable argument of the state, residual and step entry points
   passed as NULL, one at a time and all together, on a uniform 16^3 box. */
#define CHECK(x) do { int rc_ = (x); if (rc_ != ASTR_OK) { printf("FAIL %s -> %d\n", #x, rc_); return 1; } } while (0)
int main(void) {
  const int n = 16;
  const size_t nh = (size_t)(n + 11) * (n + 11) * (n + 11), n0 = (size_t)(n + 1) * (n + 1) * (n + 1);
  astr_dims d = {n, n, n, n, n, n, 3, 3, 3};
  astr_params p = {0};
  astr_ctx* c = NULL;
  astr_status st;
  double hist[4], dx = 6.283185307179586 / n, pinf = 1.0 / (1.4 * 0.01);
  double *q = malloc(5 * nh * sizeof(double)), *rho = malloc(nh * sizeof(double));
  double *vel = calloc(3 * nh, sizeof(double)), *prs = malloc(nh * sizeof(double));
  double *tmp = malloc(nh * sizeof(double)), *x1 = malloc(nh * sizeof(double));
  double *jac = malloc(nh * sizeof(double)), *qrhs = malloc(5 * n0 * sizeof(double));
  double *dvel = malloc(9 * n0 * sizeof(double)), *dtmp = malloc(3 * n0 * sizeof(double));
  size_t i;
  p.order = ASTR_ORDER_MAIN; p.precision = ASTR_FP64; p.lfilter = 1; p.diffterm = 1;
  p.alfa_filter = 0.49; p.beter_halo = 1.11; p.beter_bound = 0.98; p.mach = 0.1;
  p.reynolds = 1600.0; p.prandtl = 0.72; p.ref_tem = 273.15; p.suth_const = 110.3;
  p.deltat = 1e-3;
  for (i = 0; i < nh; ++i) {
    rho[i] = 1.0; prs[i] = pinf; tmp[i] = 1.0; x1[i] = 1.0 / dx; jac[i] = dx * dx * dx;
    q[i] = 1.0; q[nh + i] = q[2 * nh + i] = q[3 * nh + i] = 0.0; q[4 * nh + i] = pinf / 0.4;
  }
  CHECK(astr_gpu_create(&d, &p, &c));
  CHECK(astr_gpu_set_metrics_diag(c, x1, x1, x1, jac));
  CHECK(astr_gpu_upload_state(c, q, rho, vel, prs, tmp));
  CHECK(astr_gpu_rk3_step(c, 1, NULL, NULL));
  CHECK(astr_gpu_rk3_step(c, 2, hist, NULL));
  CHECK(astr_gpu_rk3_step(c, 1, NULL, &st));
  CHECK(astr_gpu_download_state(c, NULL, NULL, NULL, NULL, NULL));
  for (i = 0; i < nh; ++i) rho[i] = prs[i] = -1.0;
  CHECK(astr_gpu_download_state(c, NULL, rho, NULL, NULL, NULL));
  CHECK(astr_gpu_download_state(c, NULL, NULL, NULL, prs, NULL));
  CHECK(astr_gpu_download_state(c, q, NULL, vel, NULL, tmp));
  CHECK(astr_gpu_download_rhs(c, NULL, NULL, NULL));
  CHECK(astr_gpu_download_rhs(c, qrhs, NULL, NULL));
  CHECK(astr_gpu_download_rhs(c, NULL, dvel, NULL));
  CHECK(astr_gpu_download_rhs(c, NULL, NULL, dtmp));
  astr_gpu_destroy(c);
  /* a uniform state stays uniform */
  printf("rho %.15g prs %.15g ke %.3g crash %d\n", rho[nh / 2], prs[nh / 2] / pinf, hist[2], st.crash);
  return fabs(rho[nh / 2] - 1.0) < 1e-12 && fabs(prs[nh / 2] / pinf - 1.0) < 1e-12 ? 0 : 2;
}
"""


@pytest.mark.gpu
def test_plain_c_host_null_arguments(gpu_lib, tmp_path):
    """A C host passes NULL for each array the state, residual and step
    entry points may skip (the contract the Fortran binding's c_null_ptr
    arguments rely on)."""
    import shutil
    import subprocess
    from astr_gb300 import capi
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    src = tmp_path / "nulls.c"
    src.write_text(C_HOST_NULLS)
    exe = tmp_path / "nulls"
    libdir = os.path.dirname(capi.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    "-I", os.path.join(ROOT, "include"), str(src), "-L", libdir, "-lastr_gb300",
                    "-Wl,-rpath," + libdir, "-lm", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr


# Faces on which each routine of boucon exists (src/bc.F90: noslip 6306-6712
# all faces; noslip_adibatic 6728-7036 x and y; slipisotwall 7038-7229 and
# slipadibwall 7231-7430 y; outflow 3404-3617 xmax and ymax; farfield
# 3008-3392 y and z; zeroextrap 2356-2652 and symmetry 2664-2996 all faces;
# inflow 1366-1562 and inflow_nscbc 2114-2344 xmin; gcnscbc 8024-8254 xmax
# and ymax).
FACES = {41: range(6), 42: range(4), 411: (2, 3), 421: (2, 3), 21: (1, 3), 51: range(2, 6),
         50: range(6), 60: range(6), 11: (0,), 12: (0,), 23: (1, 3)}


@pytest.mark.parametrize("btype", sorted(FACES) + [22, 31, 52])
def test_routine_face_table(gpu_lib, btype):
    """create accepts a routine exactly on the faces where the reference
    has it and refuses the routines that are not built.  Accepted contexts
    get past validation (ASTR_OK with a GPU, ASTR_ERR_CUDA without one)."""
    from astr_gb300 import capi
    for n in range(6):
        npdc = [3, 3, 3]
        npdc[n // 2] = 4
        d = capi.AstrDims(16, 16, 16, 16, 16, 16, *npdc)
        bct = [0] * 6
        bct[n] = btype
        p = _params(bctype=tuple(bct), twall=1.0, xslip=1.0)
        h = ctypes.c_void_p()
        rc = gpu_lib.astr_gpu_create(ctypes.byref(d), ctypes.byref(p), ctypes.byref(h))
        if rc == capi.ASTR_OK:
            gpu_lib.astr_gpu_destroy(h)
        accepted = rc in (capi.ASTR_OK, capi.ASTR_ERR_CUDA)
        assert accepted == (n in FACES.get(btype, ())), (btype, n, rc, capi.last_error(None))
        if not accepted:
            assert rc == capi.ASTR_ERR_UNSUPPORTED
