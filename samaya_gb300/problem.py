"""Model <-> LpProblem through the engine library's host code (C++, no GPU needed).

``make_problem(model)`` is samaya's ``compute_scaling`` + ``make_problem`` (reference
src/linalg/scaling.cpp:130-200, src/lp/lp_solver.cpp:28-51): the power-of-two scaled
computational form that ``solve_pdlp`` receives.  ``model_solution`` maps a PDLP answer back as
samaya's ``solve_pdlp_lp`` does (src/core/solver.cpp:415-432).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native
from .model import LpProblem, Model


@dataclass
class Scaling:
    col: np.ndarray
    row: np.ndarray


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def make_problem(model: Model, device: bool = False):
    """Returns (LpProblem, Scaling); ``device=True`` computes it on the GPU
    (sg_scale_model_device, the same bits)."""
    lib = _native.load()
    m, n = model.m, model.n
    nnz = model.nnz
    colptr = np.zeros(n + 1, dtype=np.int64)
    rowidx = np.zeros(max(nnz, 1), dtype=np.int32)
    vals = np.zeros(max(nnz, 1))
    cost, lower, upper = np.zeros(n + m), np.zeros(n + m), np.zeros(n + m)
    col = np.zeros(max(n, 1))
    row = np.zeros(max(m, 1))
    out_nnz = ctypes.c_int64(0)
    D, I64, I32 = ctypes.c_double, ctypes.c_int64, ctypes.c_int32
    fn = lib.sg_scale_model_device if device else lib.sg_scale_model
    rc = fn(m, n, _p(model.colptr, I64), _p(model.rowidx, I32),
                            _p(model.vals, D), _p(model.obj, D), _p(model.col_lower, D),
                            _p(model.col_upper, D), _p(model.row_lower, D),
                            _p(model.row_upper, D), 1 if model.maximize else 0, _p(colptr, I64),
                            _p(rowidx, I32), _p(vals, D), _p(cost, D), _p(lower, D),
                            _p(upper, D), _p(col, D), _p(row, D), ctypes.byref(out_nnz))
    _native.check(rc, "sg_scale_model_device" if device else "sg_scale_model")
    k = out_nnz.value
    lp = LpProblem(m=m, n=n, colptr=colptr, rowidx=rowidx[:k].copy(), vals=vals[:k].copy(),
                   cost=cost, lower=lower, upper=upper)
    return lp, Scaling(col=col[:n].copy(), row=row[:m].copy())


def model_solution(model: Model, scaling: Scaling, x_lp, y_lp):
    """(x, row_activity, row_dual, objective) in the model's space."""
    lib = _native.load()
    m, n = model.m, model.n
    x = np.zeros(max(n, 1))
    act = np.zeros(max(m, 1))
    dual = np.zeros(max(m, 1))
    D = ctypes.c_double
    xl = np.ascontiguousarray(x_lp, dtype=np.float64)
    yl = np.ascontiguousarray(y_lp if len(y_lp) else np.zeros(1), dtype=np.float64)
    col = np.ascontiguousarray(scaling.col, dtype=np.float64)
    row = np.ascontiguousarray(scaling.row if m else np.ones(1), dtype=np.float64)
    _native.check(lib.sg_unscale_solution(m, n, _p(col, D), _p(row, D),
                                           1 if model.maximize else 0, _p(xl, D), _p(yl, D),
                                           _p(x, D), _p(act, D), _p(dual, D)),
                  "sg_unscale_solution")
    x = x[:n]
    return x, act[:m], dual[:m], model.obj_offset + float(np.dot(model.obj, x))
