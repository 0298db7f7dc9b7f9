"""ORACLE — test infrastructure only.

ctypes binding of ``oracle/pdlp_oracle.c``, the plain-C restatement of the reference solver's
CPU PDLP path (``src/lp/pdlp.cpp`` of the reference).  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this module, as the
result the GPU engine is compared with or as the timed CPU baseline; the product package
``samaya_gb300`` never does.

Pinned bit-for-bit against the reference's own compiled code through the fixtures in
``tests/golden/`` (``tests/test_oracle_pin.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")
_SRC = os.path.join(_HERE, "pdlp_oracle.c")

# SimplexStatus values of the reference (src/lp/simplex.hpp:28-35).
OPTIMAL, INFEASIBLE, UNBOUNDED, ITERATION_LIMIT, TIME_LIMIT, NUMERICAL_ERROR = range(6)
STATUS_NAMES = ["optimal", "infeasible", "unbounded", "iteration_limit", "time_limit",
                "numerical_error"]


def build(force: bool = False) -> str:
    """Compiles the oracle with gcc (no FMA contraction, as the reference is built)."""
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC)):
        os.makedirs(_BUILD, exist_ok=True)
        tmp = _LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC",
                               "-shared", "-o", tmp, _SRC, "-lm"])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class _Stats(ctypes.Structure):
    _fields_ = [("restarts", ctypes.c_longlong), ("evaluations", ctypes.c_longlong),
                ("omega", ctypes.c_double), ("step_size", ctypes.c_double),
                ("operator_norm", ctypes.c_double), ("last", ctypes.c_double * 3)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    return _lib


def _p(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


D = ctypes.c_double
I64 = ctypes.c_int64
I32 = ctypes.c_int32


@dataclass
class OracleResult:
    status: int
    iterations: int
    primal_residual: float
    dual_residual: float
    gap: float
    x: np.ndarray
    y: np.ndarray
    dual_ray: np.ndarray | None
    primal_ray: np.ndarray | None
    stats: dict = field(default_factory=dict)


def pdlp_solve(m, n, colptr, rowidx, vals, cost, lower, upper, tol=1e-8, max_iter=-1,
               time_limit=0.0) -> OracleResult:
    """The reference's CPU ``solve_pdlp`` on an LpProblem (computational form, A as CSC)."""
    colptr = np.ascontiguousarray(colptr, dtype=np.int64)
    rowidx = np.ascontiguousarray(rowidx, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    cost = np.ascontiguousarray(cost, dtype=np.float64)
    lower = np.ascontiguousarray(lower, dtype=np.float64)
    upper = np.ascontiguousarray(upper, dtype=np.float64)
    x = np.zeros(n + m)
    y = np.zeros(max(m, 1))
    dr = np.zeros(max(m, 1))
    pr = np.zeros(max(n, 1))
    flags = np.zeros(2, dtype=np.int32)
    res = np.zeros(3)
    iters = ctypes.c_longlong(0)
    st = _Stats()
    f = lib().orc_pdlp_solve
    f.restype = ctypes.c_int
    status = f(ctypes.c_int(m), ctypes.c_int(n), _p(colptr, I64), _p(rowidx, I32), _p(vals, D),
               _p(cost, D), _p(lower, D), _p(upper, D), D(tol), ctypes.c_longlong(max_iter),
               D(time_limit), ctypes.byref(iters), _p(res, D), _p(x, D), _p(y, D), _p(dr, D),
               _p(pr, D), _p(flags, I32), ctypes.byref(st))
    return OracleResult(status, iters.value, res[0], res[1], res[2], x, y[:m],
                        dr[:m] if flags[0] else None, pr[:n] if flags[1] else None,
                        dict(restarts=st.restarts, evaluations=st.evaluations, omega=st.omega,
                             step_size=st.step_size, operator_norm=st.operator_norm,
                             last=tuple(st.last)))


def compute_scaling(m, n, colptr, rowidx, vals):
    """Power-of-two scaling factors (col, row) of ``compute_scaling``."""
    col = np.zeros(max(n, 1))
    row = np.zeros(max(m, 1))
    colptr = np.ascontiguousarray(colptr, dtype=np.int64)
    rowidx = np.ascontiguousarray(rowidx, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    lib().orc_compute_scaling(ctypes.c_int(m), ctypes.c_int(n), _p(colptr, I64), _p(rowidx, I32),
                              _p(vals, D), _p(col, D), _p(row, D))
    return col[:n], row[:m]


def make_problem(model, col, row):
    """``make_problem``: the scaled computational form of a model (dict-like with the fields of
    ``samaya_gb300.Model``).  Returns (colptr, rowidx, vals, cost, lower, upper)."""
    m, n = model.m, model.n
    nnz = int(model.colptr[-1])
    oc = np.zeros(n + 1, dtype=np.int64)
    orow = np.zeros(max(nnz, 1), dtype=np.int32)
    ov = np.zeros(max(nnz, 1))
    cost = np.zeros(n + m)
    lower = np.zeros(n + m)
    upper = np.zeros(n + m)
    nnz_out = ctypes.c_int64(0)
    a = [np.ascontiguousarray(v, dtype=t) for v, t in (
        (model.colptr, np.int64), (model.rowidx, np.int32), (model.vals, np.float64),
        (model.obj, np.float64), (model.col_lower, np.float64), (model.col_upper, np.float64),
        (model.row_lower, np.float64), (model.row_upper, np.float64))]
    col = np.ascontiguousarray(col, dtype=np.float64)
    row = np.ascontiguousarray(row, dtype=np.float64)
    lib().orc_make_problem(ctypes.c_int(m), ctypes.c_int(n), _p(a[0], I64), _p(a[1], I32),
                           _p(a[2], D), _p(a[3], D), _p(a[4], D), _p(a[5], D), _p(a[6], D),
                           _p(a[7], D), ctypes.c_int(1 if model.maximize else 0), _p(col, D),
                           _p(row, D), _p(oc, I64), _p(orow, I32), _p(ov, D), _p(cost, D),
                           _p(lower, D), _p(upper, D), ctypes.byref(nnz_out))
    k = nnz_out.value
    return oc, orow[:k].copy(), ov[:k].copy(), cost, lower, upper


def setup(m, n, colptr, rowidx, vals):
    """Ruiz factors, A_eq values (CSC order), A_eq^T values (CSR order of A) and L."""
    nnz = int(colptr[-1])
    rs = np.zeros(max(m, 1))
    cs = np.zeros(max(n, 1))
    aeq = np.zeros(max(nnz, 1))
    ateq = np.zeros(max(nnz, 1))
    L = ctypes.c_double(0)
    colptr = np.ascontiguousarray(colptr, dtype=np.int64)
    rowidx = np.ascontiguousarray(rowidx, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    lib().orc_setup(ctypes.c_int(m), ctypes.c_int(n), _p(colptr, I64), _p(rowidx, I32),
                    _p(vals, D), _p(rs, D), _p(cs, D), _p(aeq, D), _p(ateq, D), ctypes.byref(L))
    return rs[:m], cs[:n], aeq[:nnz], ateq[:nnz], L.value


def power_start(m):
    u = np.zeros(max(m, 1))
    lib().orc_power_start(ctypes.c_int(m), _p(u, D))
    return u[:m]


def pdhg_steps(m, n, colptr, rowidx, vals, cost, lower, upper, tau, sigma, steps, k, state):
    """Fixed-step PDHG on an equilibrated problem; ``state`` = dict(v, v_prev, y, v_erg, y_erg)
    (updated in place)."""
    st = {key: np.ascontiguousarray(state[key], dtype=np.float64) for key in
          ("v", "v_prev", "y", "v_erg", "y_erg")}
    arrs = [np.ascontiguousarray(a, dtype=t) for a, t in (
        (colptr, np.int64), (rowidx, np.int32), (vals, np.float64), (cost, np.float64),
        (lower, np.float64), (upper, np.float64))]
    lib().orc_pdhg_steps(ctypes.c_int(m), ctypes.c_int(n), _p(arrs[0], I64), _p(arrs[1], I32),
                         _p(arrs[2], D), _p(arrs[3], D), _p(arrs[4], D), _p(arrs[5], D), D(tau),
                         D(sigma), ctypes.c_int(steps), ctypes.c_longlong(k), _p(st["v"], D),
                         _p(st["v_prev"], D), _p(st["y"], D), _p(st["v_erg"], D),
                         _p(st["y_erg"], D))
    return st


def halpern_steps(m, n, colptr, rowidx, vals, cost, lower, upper, tau, sigma, steps, k, v, y,
                  v0, y0):
    """Reflected Halpern PDHG iterations on an equilibrated problem (the engine's Halpern
    variant; no reference counterpart): returns dict(v, y, v_hat, y_hat) after ``steps``
    iterations from z = (v, y) with anchor (v0, y0), k iterations since the anchor."""
    out = {"v": np.ascontiguousarray(v, dtype=np.float64).copy(),
           "y": np.ascontiguousarray(y if m else np.zeros(1), dtype=np.float64).copy(),
           "v_hat": np.zeros(n + m), "y_hat": np.zeros(max(m, 1))}
    anchors = [np.ascontiguousarray(a, dtype=np.float64) for a in
               (v0, y0 if m else np.zeros(1))]
    arrs = [np.ascontiguousarray(a, dtype=t) for a, t in (
        (colptr, np.int64), (rowidx, np.int32), (vals, np.float64), (cost, np.float64),
        (lower, np.float64), (upper, np.float64))]
    lib().orc_halpern_steps(ctypes.c_int(m), ctypes.c_int(n), _p(arrs[0], I64),
                            _p(arrs[1], I32), _p(arrs[2], D), _p(arrs[3], D), _p(arrs[4], D),
                            _p(arrs[5], D), D(tau), D(sigma), ctypes.c_int(steps),
                            ctypes.c_longlong(k), _p(out["v"], D), _p(out["y"], D),
                            _p(anchors[0], D), _p(anchors[1], D), _p(out["v_hat"], D),
                            _p(out["y_hat"], D))
    out["y"] = out["y"][:m]
    out["y_hat"] = out["y_hat"][:m]
    return out


def eval_sums(m, n, colptr, rowidx, vals, cost, lower, upper, cs, rs, v, y):
    """The seven evaluation sums (primal_sq, dual_sq, primal_obj, dual_obj, x_sq, r_sq, y_sq)."""
    out = np.zeros(7)
    arrs = [np.ascontiguousarray(a, dtype=t) for a, t in (
        (colptr, np.int64), (rowidx, np.int32), (vals, np.float64), (cost, np.float64),
        (lower, np.float64), (upper, np.float64), (cs, np.float64), (rs, np.float64),
        (v, np.float64), (y, np.float64))]
    lib().orc_eval_sums(ctypes.c_int(m), ctypes.c_int(n), _p(arrs[0], I64), _p(arrs[1], I32),
                        *[_p(a, D) for a in arrs[2:]], _p(out, D))
    return out


def verify_lp(model, x, y, tol_primal=1e-6, tol_dual=1e-6):
    """The reference's verify_lp_optimality (src/verify/verify.cpp) for an LP model and its
    column values x and row duals y (the reference's convention, d = c - A'y): (ok, dict of the
    largest bound / row / dual violations and the objective)."""
    out = np.zeros(4)
    a = [np.ascontiguousarray(v, dtype=t) for v, t in (
        (model.colptr, np.int64), (model.rowidx, np.int32), (model.vals, np.float64),
        (model.obj, np.float64), (model.col_lower, np.float64), (model.col_upper, np.float64),
        (model.row_lower, np.float64), (model.row_upper, np.float64), (x, np.float64),
        (y, np.float64))]
    f = lib().orc_verify_lp
    f.restype = ctypes.c_int
    ok = f(ctypes.c_int(model.m), ctypes.c_int(model.n), _p(a[0], I64), _p(a[1], I32),
           _p(a[2], D), _p(a[3], D), D(model.obj_offset), _p(a[4], D), _p(a[5], D),
           _p(a[6], D), _p(a[7], D), ctypes.c_int(int(model.maximize)), _p(a[8], D),
           _p(a[9], D), D(tol_primal), D(tol_dual), _p(out, D))
    return bool(ok), {"bound": out[0], "row": out[1], "dual": out[2], "objective": out[3]}
