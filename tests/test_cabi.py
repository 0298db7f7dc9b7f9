"""The C-ABI library builds, loads and exports every function include/*.h declares; argument
checks that need no GPU behave like the reference's (errors are codes, never exceptions)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from samaya_gb300 import _native


def _lib():
    return _native.load(build_if_missing=True)


def test_every_declared_symbol_is_exported():
    lib = _lib()
    names = _native.declared_symbols()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_error_strings_and_defaults():
    lib = _lib()
    assert lib.sg_pdlp_error_string(0) == b"ok"
    assert lib.sg_pdlp_error_string(-1) == b"invalid argument"
    assert lib.sg_pdlp_error_string(-5).startswith(b"problem too large")
    o = _native.Opts()
    lib.sg_pdlp_default_opts(ctypes.byref(o))
    assert o.tol == 1e-8 and o.max_iterations == -1 and o.precision == 0


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def test_invalid_problems_are_rejected_before_any_device_work():
    lib = _lib()
    h = ctypes.c_void_p()
    colptr = np.array([0, 2, 3], dtype=np.int64)
    rowidx = np.array([0, 5, 1], dtype=np.int32)  # row 5 out of range for m = 2
    vals = np.array([1.0, 2.0, 3.0])
    v = np.zeros(4)
    rc = lib.sg_pdlp_create(ctypes.byref(h), 2, 2, _p(colptr, ctypes.c_int64),
                            _p(rowidx, ctypes.c_int32), _p(vals, ctypes.c_double),
                            _p(v, ctypes.c_double), _p(v, ctypes.c_double),
                            _p(v, ctypes.c_double), None)
    assert rc == -1 and not h.value
    assert b"row index" in lib.sg_pdlp_last_error()
    rowidx[1] = 1
    vals[0] = np.nan
    rc = lib.sg_pdlp_create(ctypes.byref(h), 2, 2, _p(colptr, ctypes.c_int64),
                            _p(rowidx, ctypes.c_int32), _p(vals, ctypes.c_double),
                            _p(v, ctypes.c_double), _p(v, ctypes.c_double),
                            _p(v, ctypes.c_double), None)
    assert rc == -1
    bad = np.array([0, 2, 1], dtype=np.int64)  # decreasing column starts
    vals[0] = 1.0
    rc = lib.sg_pdlp_create(ctypes.byref(h), 2, 2, _p(bad, ctypes.c_int64),
                            _p(rowidx, ctypes.c_int32), _p(vals, ctypes.c_double),
                            _p(v, ctypes.c_double), _p(v, ctypes.c_double),
                            _p(v, ctypes.c_double), None)
    assert rc == -1
    assert lib.sg_pdlp_solve(None, None, None, None, None, None) == -1
    lib.sg_pdlp_destroy(None)


def test_no_device_is_reported_as_an_error_code():
    lib = _lib()
    if os.environ.get("CUDA_VISIBLE_DEVICES") is None and _has_gpu():
        return
    major, minor = ctypes.c_int(0), ctypes.c_int(0)
    buf = ctypes.create_string_buffer(64)
    assert lib.sg_pdlp_available(ctypes.byref(major), ctypes.byref(minor), buf, 64) == -2


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
