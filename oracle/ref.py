"""Test infrastructure only: ctypes binding of ``oracle/_ref/libsamaya_ref.so``, the reference
solver's own CPU code compiled from the reference checkout by ``oracle/Makefile.ref``.

It exists only where the reference checkout exists (it is never shipped); tests that need it
skip when it is absent.  Used to pin the oracle restatement and to make ``tests/golden/``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_ref", "libsamaya_ref.so")
# The reference checkout: SAMAYA_REFERENCE_ROOT, else a sibling directory `reference` of this
# repository's root.
REFERENCE_ROOT = os.path.abspath(os.environ.get(
    "SAMAYA_REFERENCE_ROOT", os.path.join(_HERE, "..", "..", "reference")))

D = ctypes.c_double
I64 = ctypes.c_int64
I32 = ctypes.c_int32


def available() -> bool:
    return os.path.exists(_LIB) or os.path.isdir(os.path.join(REFERENCE_ROOT, "src"))


def build() -> str | None:
    """Builds the reference's CPU sources in place (only where the checkout exists; make
    rebuilds what changed, ref_driver.cpp included)."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "src")):
        return _LIB if os.path.exists(_LIB) else None
    subprocess.check_call(["make", "-s", "-f", "Makefile.ref", f"REF={REFERENCE_ROOT}",
                           f"-j{os.cpu_count() or 4}"], cwd=_HERE)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        if path is None:
            raise RuntimeError("the reference checkout is not available")
        _lib = ctypes.CDLL(path)
    return _lib


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _model_args(model):
    arrs = [np.ascontiguousarray(v, dtype=t) for v, t in (
        (model.colptr, np.int64), (model.rowidx, np.int32), (model.vals, np.float64),
        (model.obj, np.float64), (model.col_lower, np.float64), (model.col_upper, np.float64),
        (model.row_lower, np.float64), (model.row_upper, np.float64))]
    return arrs, [ctypes.c_int(model.m), ctypes.c_int(model.n), _p(arrs[0], I64),
                  _p(arrs[1], I32)] + [_p(a, D) for a in arrs[2:]] + [
        ctypes.c_int(1 if model.maximize else 0)]


def pdlp_solve(m, n, colptr, rowidx, vals, cost, lower, upper, tol=1e-8, max_iter=-1,
               time_limit=0.0):
    arrs = [np.ascontiguousarray(a, dtype=t) for a, t in (
        (colptr, np.int64), (rowidx, np.int32), (vals, np.float64), (cost, np.float64),
        (lower, np.float64), (upper, np.float64))]
    x = np.zeros(n + m)
    y = np.zeros(max(m, 1))
    dr = np.zeros(max(m, 1))
    pr = np.zeros(max(n, 1))
    flags = np.zeros(2, dtype=np.int32)
    res = np.zeros(3)
    iters = ctypes.c_longlong(0)
    f = lib().ref_pdlp_solve
    f.restype = ctypes.c_int
    status = f(ctypes.c_int(m), ctypes.c_int(n), _p(arrs[0], I64), _p(arrs[1], I32),
               *[_p(a, D) for a in arrs[2:]], D(tol), ctypes.c_longlong(max_iter), D(time_limit),
               ctypes.byref(iters), _p(res, D), _p(x, D), _p(y, D), _p(dr, D), _p(pr, D),
               _p(flags, I32))
    return dict(status=status, iterations=iters.value, primal_residual=res[0],
                dual_residual=res[1], gap=res[2], x=x, y=y[:m],
                dual_ray=dr[:m] if flags[0] else None, primal_ray=pr[:n] if flags[1] else None)


def scale_model(model):
    m, n = model.m, model.n
    nnz = int(model.colptr[-1])
    oc = np.zeros(n + 1, dtype=np.int64)
    orow = np.zeros(max(nnz, 1), dtype=np.int32)
    ov = np.zeros(max(nnz, 1))
    cost, lower, upper = np.zeros(n + m), np.zeros(n + m), np.zeros(n + m)
    cs, rs = np.zeros(max(n, 1)), np.zeros(max(m, 1))
    nnz_out = ctypes.c_int64(0)
    keep, args = _model_args(model)
    lib().ref_scale_model(*args, _p(oc, I64), _p(orow, I32), _p(ov, D), _p(cost, D),
                          _p(lower, D), _p(upper, D), _p(cs, D), _p(rs, D),
                          ctypes.byref(nnz_out))
    k = nnz_out.value
    return dict(colptr=oc, rowidx=orow[:k].copy(), vals=ov[:k].copy(), cost=cost, lower=lower,
                upper=upper, col_scale=cs[:n], row_scale=rs[:m])


def dual_simplex(model, time_limit=0.0):
    x = np.zeros(max(model.n, 1))
    y = np.zeros(max(model.m, 1))
    obj = ctypes.c_double(0)
    iters = ctypes.c_longlong(0)
    keep, args = _model_args(model)
    f = lib().ref_dual_simplex
    f.restype = ctypes.c_int
    status = f(*args, D(time_limit), ctypes.byref(obj), _p(x, D), _p(y, D), ctypes.byref(iters))
    return dict(status=status, objective=obj.value, x=x[:model.n], y=y[:model.m],
                iterations=iters.value)


def verify_optimal(model, x, y, tol=1e-6):
    obj = ctypes.c_double(0)
    keep, args = _model_args(model)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    f = lib().ref_verify_optimal
    f.restype = ctypes.c_int
    ok = f(*args, _p(x, D), _p(y, D), D(tol), ctypes.byref(obj))
    return bool(ok), obj.value


def random_lp(family, max_rows, max_cols, seed, index, prefix_family=0, prefix_count=0):
    """The reference test generator's model number ``index`` from std::mt19937(seed), after
    ``prefix_count`` draws of ``prefix_family`` from the same generator."""
    dims = np.zeros(3, dtype=np.int32)
    f = lib().ref_random_lp
    null = ctypes.POINTER(ctypes.c_double)()
    f(ctypes.c_int(family), ctypes.c_int(max_rows), ctypes.c_int(max_cols), ctypes.c_uint(seed),
      ctypes.c_int(index), ctypes.c_int(prefix_family), ctypes.c_int(prefix_count), _p(dims, I32),
      ctypes.POINTER(I64)(), ctypes.POINTER(I32)(), null,
      null, null, null, null, null, ctypes.POINTER(ctypes.c_int)(), null)
    m, n, nnz = (int(d) for d in dims)
    colptr = np.zeros(n + 1, dtype=np.int64)
    rowidx = np.zeros(max(nnz, 1), dtype=np.int32)
    vals = np.zeros(max(nnz, 1))
    obj, cl, cu = np.zeros(n), np.zeros(n), np.zeros(n)
    rl, ru = np.zeros(max(m, 1)), np.zeros(max(m, 1))
    mx = ctypes.c_int(0)
    off = ctypes.c_double(0)
    f(ctypes.c_int(family), ctypes.c_int(max_rows), ctypes.c_int(max_cols), ctypes.c_uint(seed),
      ctypes.c_int(index), ctypes.c_int(prefix_family), ctypes.c_int(prefix_count), _p(dims, I32),
      _p(colptr, I64), _p(rowidx, I32), _p(vals, D),
      _p(obj, D), _p(cl, D), _p(cu, D), _p(rl, D), _p(ru, D), ctypes.byref(mx), ctypes.byref(off))
    return dict(m=m, n=n, colptr=colptr, rowidx=rowidx[:nnz], vals=vals[:nnz], obj=obj,
                col_lower=cl, col_upper=cu, row_lower=rl[:m], row_upper=ru[:m],
                maximize=bool(mx.value), obj_offset=off.value)


def reference_lp(model):
    """The reference tests' dense long-double tableau simplex: (status, objective) with status
    0 optimal, 1 infeasible, 2 unbounded."""
    obj = ctypes.c_double(0)
    keep, args = _model_args(model)
    f = lib().ref_reference_lp
    f.restype = ctypes.c_int
    status = f(*args, D(model.obj_offset), ctypes.byref(obj))
    return status, obj.value


def solver_pdlp(model):
    obj = ctypes.c_double(0)
    ver = ctypes.c_int(0)
    si = ctypes.c_longlong(0)
    pi = ctypes.c_longlong(0)
    keep, args = _model_args(model)
    f = lib().ref_solver_pdlp
    f.restype = ctypes.c_int
    status = f(*args, D(model.obj_offset), ctypes.byref(obj), ctypes.byref(ver), ctypes.byref(si),
               ctypes.byref(pi))
    return dict(status=status, objective=obj.value, verified=bool(ver.value),
                simplex_iterations=si.value, pdlp_iterations=pi.value)


class RefMpsError(RuntimeError):
    """samaya's reader raised: ``parse`` is True for a samaya::ParseError."""

    def __init__(self, parse: bool, message: str):
        super().__init__(message)
        self.parse = parse


def _mps_take(h):
    L = lib()
    info = np.zeros(10, dtype=np.int64)
    off = ctypes.c_double(0)
    secs = ctypes.c_double(0)
    L.ref_mps_info(h, _p(info, I64), ctypes.byref(off), ctypes.byref(secs))
    m, n, nnz = int(info[0]), int(info[1]), int(info[2])
    colptr = np.zeros(n + 1, dtype=np.int64)
    rowidx = np.zeros(max(nnz, 1), dtype=np.int32)
    vals = np.zeros(max(nnz, 1))
    obj, cl, cu = np.zeros(max(n, 1)), np.zeros(max(n, 1)), np.zeros(max(n, 1))
    integer = np.zeros(max(n, 1), dtype=np.uint8)
    rl, ru = np.zeros(max(m, 1)), np.zeros(max(m, 1))
    L.ref_mps_get(h, _p(colptr, I64), _p(rowidx, I32), _p(vals, D), _p(obj, D), _p(cl, D),
                  _p(cu, D), integer.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _p(rl, D),
                  _p(ru, D))
    name = ctypes.create_string_buffer(int(info[5]) + 1)
    rn = ctypes.create_string_buffer(int(info[6]) + 1)
    cn = ctypes.create_string_buffer(int(info[7]) + 1)
    rs = np.zeros(m + 1, dtype=np.int64)
    cs = np.zeros(n + 1, dtype=np.int64)
    L.ref_mps_names(h, name, rn, _p(rs, I64), cn, _p(cs, I64))
    return dict(m=m, n=n, colptr=colptr, rowidx=rowidx[:nnz], vals=vals[:nnz], obj=obj[:n],
                col_lower=cl[:n], col_upper=cu[:n], col_integer=integer[:n], row_lower=rl[:m],
                row_upper=ru[:m], maximize=bool(info[3]), obj_offset=off.value,
                name=name.raw[:int(info[5])], row_names=rn.raw[:int(info[6])], row_starts=rs,
                col_names=cn.raw[:int(info[7])], col_starts=cs, q_nnz=int(info[8]),
                quadratic_rows=int(info[9]), seconds=secs.value)


def _mps_call(fn, *args):
    L = lib()
    f = getattr(L, fn)
    f.restype = ctypes.c_int
    L.ref_mps_free.argtypes = [ctypes.c_void_p]
    h = ctypes.c_void_p()
    err = ctypes.create_string_buffer(4096)
    rc = f(*args, ctypes.byref(h), err, ctypes.c_size_t(len(err)))
    if rc != 0:
        raise RefMpsError(rc == 1, err.value.decode(errors="replace"))
    try:
        return _mps_take(h)
    finally:
        L.ref_mps_free(h)


def mps_read_text(text):
    """samaya::read_mps_from_string (src/io/mps_reader.cpp:517): the Model as arrays, names as
    bytes with starts; raises RefMpsError where samaya raises."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    return _mps_call("ref_mps_read", ctypes.c_char_p(data), ctypes.c_size_t(len(data)))


def mps_read_file(path):
    """samaya::read_mps (src/io/mps_reader.cpp:530); ``seconds`` is its wall time."""
    return _mps_call("ref_mps_read_file", ctypes.c_char_p(os.fsencode(path)))
