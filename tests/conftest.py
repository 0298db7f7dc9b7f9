"""Shared fixtures. Tests marked ``gpu`` need a GB300; everything else runs on the CPU."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def engine():
    """The engine library, built in-tree if missing (GPU tests)."""
    import samaya_gb300
    from samaya_gb300 import _native
    _native.load(build_if_missing=True)
    return samaya_gb300


class Case:
    """One LP of a golden group."""

    def __init__(self, data, k):
        p = f"k{k}_"
        self.k = k
        self.opts = data[p + "opts"]
        self.tol = float(self.opts[0])
        self.max_iter = int(self.opts[1])
        self.ref_status = int(data[p + "ref_status"][0])
        self.ref_iterations = int(data[p + "ref_iterations"][0])
        self.ref_res = data[p + "ref_res"]
        self.ref_x = data[p + "ref_x"]
        self.ref_y = data[p + "ref_y"]
        self.ref_dual_ray = data.get(p + "ref_dual_ray")
        self.ref_primal_ray = data.get(p + "ref_primal_ray")
        self.refnlp = data.get(p + "refnlp")
        self.simplex = data.get(p + "simplex")
        if p + "model_dims" in data:
            from samaya_gb300.model import LpProblem, Model
            dims = data[p + "model_dims"]
            self.model = Model(m=int(dims[0]), n=int(dims[1]), maximize=bool(dims[2]),
                               obj_offset=float(data[p + "model_offset"][0]),
                               **{k: data[p + "model_" + k] for k in
                                  ("colptr", "rowidx", "vals", "obj", "col_lower", "col_upper",
                                   "row_lower", "row_upper")})
            self.lp = LpProblem(m=self.model.m, n=self.model.n,
                                **{k: data[p + "lp_" + k] for k in
                                   ("colptr", "rowidx", "vals", "cost", "lower", "upper")})
            self.col_scale = data[p + "lp_col_scale"]
            self.row_scale = data[p + "lp_row_scale"]


def load_group(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        data = {k: z[k] for k in z.files}
    return [Case(data, k) for k in range(int(data["count"][0]))]


GROUPS = ["basic", "feasible8", "vs_simplex10", "infeasible8", "loose8", "gpu_vs_cpu6",
          "repeatable30", "config0_small"]


def highs_objective(model):
    """(status, objective) of a Model from scipy's HiGHS (scipy.optimize.linprog), an optimum
    independent of the reference and of the engine; status 0 is optimal."""
    import scipy.sparse as sp
    from scipy.optimize import linprog
    A = sp.csc_matrix((model.vals, model.rowidx, model.colptr), shape=(model.m, model.n)).tocsr()
    eq = model.row_lower == model.row_upper
    ub = ~eq & np.isfinite(model.row_upper)
    lb = ~eq & np.isfinite(model.row_lower)
    A_ub = sp.vstack([A[ub], -A[lb]]) if (ub.any() or lb.any()) else None
    b_ub = np.concatenate([model.row_upper[ub], -model.row_lower[lb]]) if A_ub is not None \
        else None
    sign = -1.0 if model.maximize else 1.0
    r = linprog(sign * model.obj, A_ub=A_ub, b_ub=b_ub, A_eq=A[eq] if eq.any() else None,
                b_eq=model.row_upper[eq] if eq.any() else None,
                bounds=np.column_stack([model.col_lower, model.col_upper]), method="highs",
                options={"primal_feasibility_tolerance": 1e-10,
                         "dual_feasibility_tolerance": 1e-10})
    if r.status != 0:
        return int(r.status), None
    return 0, sign * float(r.fun) + model.obj_offset
