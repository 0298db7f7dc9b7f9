"""Independent optima of the full-size synthetic LPs, for the GPU tests' objective checks.

Solves each LP once with scipy's HiGHS (``scipy.optimize.linprog(method="highs")``: a solver
independent of both the reference and this engine) and writes ``tests/golden/optima.json``
with the objective value, the solver status and the scipy version. Run from the repository
root:

    python tests/golden/make_optima.py [transport] [config0]
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.join(ROOT, "tests", "golden", "optima.json")


def highs_objective(model):
    import scipy
    import scipy.sparse as sp
    from scipy.optimize import linprog
    A = sp.csc_matrix((model.vals, model.rowidx, model.colptr), shape=(model.m, model.n))
    eq = model.row_lower == model.row_upper
    A = A.tocsr()
    A_eq, b_eq = A[eq], model.row_upper[eq]
    ub_rows = ~eq & np.isfinite(model.row_upper)
    lb_rows = ~eq & np.isfinite(model.row_lower)
    A_ub = sp.vstack([A[ub_rows], -A[lb_rows]]) if (ub_rows.any() or lb_rows.any()) else None
    b_ub = np.concatenate([model.row_upper[ub_rows], -model.row_lower[lb_rows]]) \
        if A_ub is not None else None
    bounds = np.column_stack([np.where(np.isfinite(model.col_lower), model.col_lower, -np.inf),
                              np.where(np.isfinite(model.col_upper), model.col_upper, np.inf)])
    t0 = time.time()
    r = linprog(model.obj, A_ub=A_ub, b_ub=b_ub, A_eq=A_eq if eq.any() else None,
                b_eq=b_eq if eq.any() else None, bounds=bounds, method="highs",
                options={"primal_feasibility_tolerance": 1e-10,
                         "dual_feasibility_tolerance": 1e-10})
    return {"objective": float(r.fun) + model.obj_offset, "status": int(r.status),
            "message": r.message, "seconds": time.time() - t0, "scipy": scipy.__version__}


def main(names):
    from samaya_gb300 import generators as g
    makers = {
        "transport": ("transportation LP 1000 supplies x 2000 demands, seed 0",
                      lambda: g.transportation_lp(1000, 2000, seed=0)),
        "config0": ("random sparse LP 2000 x 5000, seed 0",
                    lambda: g.random_sparse_lp(2000, 5000, seed=0)),
    }
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data = json.load(f)
    for name in names or list(makers):
        desc, make = makers[name]
        res = highs_objective(make())
        res["lp"] = desc
        data[name] = res
        print(name, res, flush=True)
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1:])
