"""Batched PDLP over the C ABI (``sg_batch_*``): many LpProblems solved in one persistent GPU
launch, each with its own restarts and termination. Instances may share one matrix (node
relaxations of one LP with different bounds) through ``BatchSolver.shared``."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native
from .model import LpProblem
from .pdlp import PdlpOptions, STATUS_NAMES


class _BatchResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("pad", ctypes.c_int),
                ("iterations", ctypes.c_longlong), ("primal_residual", ctypes.c_double),
                ("dual_residual", ctypes.c_double), ("gap", ctypes.c_double),
                ("primal_objective", ctypes.c_double), ("dual_objective", ctypes.c_double),
                ("restarts", ctypes.c_longlong)]


@dataclass
class BatchItem:
    status: int
    iterations: int
    primal_residual: float
    dual_residual: float
    gap: float
    primal_objective: float
    dual_objective: float
    restarts: int
    x: np.ndarray
    y: np.ndarray

    @property
    def status_name(self):
        return STATUS_NAMES[self.status]


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


class BatchSolver:
    """``matrices``: list of (m, n, colptr, rowidx, vals); ``instances``: list of
    (matrix index, cost, lower, upper)."""

    def __init__(self, matrices, instances, options: PdlpOptions | None = None):
        lib = _native.load()
        f = lib.sg_batch_create
        f.restype = ctypes.c_int
        self._lib = lib
        self.options = options or PdlpOptions()
        self.dims = [(int(m), int(n)) for (m, n, *_r) in matrices]
        mm = np.array([d[0] for d in self.dims], dtype=np.int32)
        nn = np.array([d[1] for d in self.dims], dtype=np.int32)
        colptr = np.concatenate([np.asarray(c, dtype=np.int64) for (_, _, c, _, _) in matrices])
        rowidx = np.concatenate([np.asarray(r, dtype=np.int32) for (_, _, _, r, _) in matrices] +
                                [np.zeros(0, np.int32)])
        vals = np.concatenate([np.asarray(v, dtype=np.float64) for (*_, v) in matrices] +
                              [np.zeros(0)])
        self.inst_mat = np.array([i[0] for i in instances], dtype=np.int32)
        cost = np.concatenate([np.asarray(i[1], dtype=np.float64) for i in instances])
        lower = np.concatenate([np.asarray(i[2], dtype=np.float64) for i in instances])
        upper = np.concatenate([np.asarray(i[3], dtype=np.float64) for i in instances])
        self._keep = (mm, nn, colptr, rowidx, vals, cost, lower, upper)
        self._h = ctypes.c_void_p()
        o = self.options.to_c()
        rc = f(ctypes.byref(self._h), len(matrices), _p(mm, ctypes.c_int), _p(nn, ctypes.c_int),
               _p(colptr, ctypes.c_int64), _p(rowidx, ctypes.c_int32),
               _p(vals, ctypes.c_double), len(instances), _p(self.inst_mat, ctypes.c_int),
               _p(cost, ctypes.c_double), _p(lower, ctypes.c_double),
               _p(upper, ctypes.c_double), ctypes.byref(o))
        if rc != 0:
            lib.sg_batch_last_error.restype = ctypes.c_char_p
            raise _native.EngineError(rc, "sg_batch_create: " +
                                      lib.sg_batch_last_error().decode())
        self.count = len(instances)
        self.nt = [self.dims[g][0] + self.dims[g][1] for g in self.inst_mat]
        self.ms = [self.dims[g][0] for g in self.inst_mat]

    @classmethod
    def from_problems(cls, problems, options=None):
        mats = [(p.m, p.n, p.colptr, p.rowidx, p.vals) for p in problems]
        inst = [(k, p.cost, p.lower, p.upper) for k, p in enumerate(problems)]
        return cls(mats, inst, options)

    @classmethod
    def shared(cls, lp: LpProblem, bounds, options=None):
        """One matrix, one instance per (lower, upper) pair (cost shared)."""
        inst = [(0, lp.cost, lo, up) for (lo, up) in bounds]
        return cls([(lp.m, lp.n, lp.colptr, lp.rowidx, lp.vals)], inst, options)

    def solve(self, download: bool = True):
        res = (_BatchResult * self.count)()
        x = np.zeros(sum(self.nt)) if download else None
        y = np.zeros(max(sum(self.ms), 1)) if download else None
        ms = ctypes.c_double(0)
        f = self._lib.sg_batch_solve
        f.restype = ctypes.c_int
        rc = f(self._h, res, _p(x, ctypes.c_double) if download else None,
               _p(y, ctypes.c_double) if download else None, ctypes.byref(ms))
        if rc != 0:
            self._lib.sg_batch_last_error.restype = ctypes.c_char_p
            raise _native.EngineError(rc, "sg_batch_solve: " +
                                      self._lib.sg_batch_last_error().decode())
        out = []
        xo = yo = 0
        for k in range(self.count):
            r = res[k]
            nt, m = self.nt[k], self.ms[k]
            out.append(BatchItem(r.status, r.iterations, r.primal_residual, r.dual_residual,
                                 r.gap, r.primal_objective, r.dual_objective, r.restarts,
                                 x[xo:xo + nt].copy() if download else None,
                                 y[yo:yo + m].copy() if download else None))
            xo += nt
            yo += m
        self.device_ms = ms.value
        return out

    def close(self):
        if self._h:
            self._lib.sg_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
