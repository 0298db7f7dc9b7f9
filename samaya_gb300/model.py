"""Problem containers of the PDLP path.

``Model`` mirrors the linear part of ``samaya::Model`` (include/samaya/model.hpp:36-60 of the
reference): min/max c'x + offset s.t. row_lower <= A x <= row_upper, col_lower <= x <= col_upper,
with A stored column-wise (CSC: int64 column starts, int32 row indices, float64 values).

``LpProblem`` mirrors ``samaya::LpProblem`` (src/lp/simplex.hpp:18-26): the computational form
min cost'v s.t. [A -I] v = 0, lower <= v <= upper, v = (x, r) with n structurals followed by m
row activities; cost/lower/upper have n + m entries.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


@dataclass
class Model:
    m: int
    n: int
    colptr: np.ndarray
    rowidx: np.ndarray
    vals: np.ndarray
    obj: np.ndarray
    col_lower: np.ndarray
    col_upper: np.ndarray
    row_lower: np.ndarray
    row_upper: np.ndarray
    maximize: bool = False
    obj_offset: float = 0.0

    def __post_init__(self):
        self.m = int(self.m)
        self.n = int(self.n)
        self.colptr = np.ascontiguousarray(self.colptr, dtype=np.int64)
        self.rowidx = np.ascontiguousarray(self.rowidx, dtype=np.int32)
        self.vals = _f64(self.vals)
        self.obj = _f64(self.obj)
        self.col_lower = _f64(self.col_lower)
        self.col_upper = _f64(self.col_upper)
        self.row_lower = _f64(self.row_lower)
        self.row_upper = _f64(self.row_upper)
        self.maximize = bool(self.maximize)
        self.obj_offset = float(self.obj_offset)

    @property
    def nnz(self) -> int:
        return int(self.colptr[-1])

    @classmethod
    def from_dict(cls, d) -> "Model":
        keys = ("m", "n", "colptr", "rowidx", "vals", "obj", "col_lower", "col_upper",
                "row_lower", "row_upper", "maximize", "obj_offset")
        return cls(**{k: d[k] for k in keys if k in d})


@dataclass
class LpProblem:
    m: int
    n: int
    colptr: np.ndarray
    rowidx: np.ndarray
    vals: np.ndarray
    cost: np.ndarray
    lower: np.ndarray
    upper: np.ndarray

    def __post_init__(self):
        self.m = int(self.m)
        self.n = int(self.n)
        self.colptr = np.ascontiguousarray(self.colptr, dtype=np.int64)
        self.rowidx = np.ascontiguousarray(self.rowidx, dtype=np.int32)
        self.vals = _f64(self.vals)
        self.cost = _f64(self.cost)
        self.lower = _f64(self.lower)
        self.upper = _f64(self.upper)

    @property
    def nnz(self) -> int:
        return int(self.colptr[-1])

    def arrays(self):
        return (self.m, self.n, self.colptr, self.rowidx, self.vals, self.cost, self.lower,
                self.upper)
