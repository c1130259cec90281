"""The C-ABI library: it builds for sm_103a, loads, and exports every entry
point include/astr_gpu.h declares.  No compute call needs a GPU here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "astr_gpu.h")).read()
    return sorted(set(re.findall(r"\b(astr_gpu_\w+)\s*\(", src)))


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
