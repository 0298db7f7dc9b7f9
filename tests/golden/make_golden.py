"""Generates the golden fixtures of the PDLP path from the reference solver's own code.

Run in a checkout that has the reference (it builds ``oracle/_ref`` from the reference sources
with ``oracle/Makefile.ref``):

    python tests/golden/make_golden.py

Each group mirrors one of the reference's own PDLP tests (same generator, seed, sizes,
tolerances and iteration limits):

    basic          tests/test_pdlp.cpp:54-83     row-less box LP, tol 1e-4
    feasible8      tests/test_pdlp.cpp:85-232    50 kFeasible <= 8x8 LPs, seed 42, tol 1e-8
    vs_simplex10   tests/test_pdlp.cpp:234-400   30 kFeasible <= 10x10, seed 123, tol 1e-4
    infeasible8    tests/test_pdlp.cpp:402-443   30 kRandom <= 8x8, seed 4242, tol 1e-4
    loose8         tests/test_pdlp.cpp:445-478   30 kLoose <= 8x8 after the kRandom draws
    gpu_vs_cpu6    tests/test_gpu.cpp:407-477    20 kFeasible <= 6x6, seed 42, tol 1e-6
    repeatable30   tests/test_gpu.cpp:675-697    5 kFeasible <= 30x30, seed 613, tol 1e-6
    config0        the 2000 x 5000 random sparse LP (seed 0) and a 200 x 500 one (seeds 0-2)

For every LP the fixture holds the model, the scaled LpProblem (compute_scaling +
make_problem), and the reference CPU solve_pdlp outputs (status, iterations, x, y, residuals,
rays); plus ReferenceLp (dense long-double simplex) or the reference dual simplex objective.
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from samaya_gb300.generators import random_sparse_lp  # noqa: E402
from samaya_gb300.model import Model  # noqa: E402

FEASIBLE, RANDOM, DEGENERATE, LOOSE, BOXED = range(5)

MODEL_KEYS = ("colptr", "rowidx", "vals", "obj", "col_lower", "col_upper", "row_lower",
              "row_upper")


def model_digest(model: Model) -> str:
    h = hashlib.sha256()
    for k in MODEL_KEYS:
        h.update(np.ascontiguousarray(getattr(model, k)).tobytes())
    h.update(str((model.m, model.n, model.maximize, model.obj_offset)).encode())
    return h.hexdigest()


def add_case(out, prefix, model: Model, tol, max_iter, with_refnlp=True, with_simplex=False,
             store_model=True):
    sc = ref.scale_model(model)
    r = ref.pdlp_solve(model.m, model.n, sc["colptr"], sc["rowidx"], sc["vals"], sc["cost"],
                       sc["lower"], sc["upper"], tol, max_iter)
    if store_model:
        for k in MODEL_KEYS:
            out[f"{prefix}model_{k}"] = getattr(model, k)
        out[f"{prefix}model_dims"] = np.array([model.m, model.n, int(model.maximize)])
        out[f"{prefix}model_offset"] = np.array([model.obj_offset])
        for k in ("colptr", "rowidx", "vals", "cost", "lower", "upper", "col_scale",
                  "row_scale"):
            out[f"{prefix}lp_{k}"] = sc[k]
    out[f"{prefix}digest"] = np.frombuffer(bytes.fromhex(model_digest(model)), dtype=np.uint8)
    out[f"{prefix}opts"] = np.array([tol, max_iter], dtype=np.float64)
    out[f"{prefix}ref_status"] = np.array([r["status"]])
    out[f"{prefix}ref_iterations"] = np.array([r["iterations"]])
    out[f"{prefix}ref_res"] = np.array([r["primal_residual"], r["dual_residual"], r["gap"]])
    out[f"{prefix}ref_x"] = r["x"]
    out[f"{prefix}ref_y"] = r["y"]
    if r["dual_ray"] is not None:
        out[f"{prefix}ref_dual_ray"] = r["dual_ray"]
    if r["primal_ray"] is not None:
        out[f"{prefix}ref_primal_ray"] = r["primal_ray"]
    if with_refnlp:
        st, obj = ref.reference_lp(model)
        out[f"{prefix}refnlp"] = np.array([st, obj])
    if with_simplex:
        t0 = time.time()
        ds = ref.dual_simplex(model)
        out[f"{prefix}simplex"] = np.array([ds["status"], ds["objective"], ds["iterations"],
                                            time.time() - t0])
        if ds["status"] == 0:
            ok, vobj = ref.verify_optimal(model, ds["x"], ds["y"])
            out[f"{prefix}simplex_verified"] = np.array([int(ok), vobj])
    return r


def family_group(name, family, size, seed, count, tol, max_iter, prefix_family=0,
                 prefix_count=0, with_simplex=False):
    out = {}
    for k in range(count):
        d = ref.random_lp(family, size, size, seed, k, prefix_family, prefix_count)
        model = Model.from_dict(d)
        add_case(out, f"k{k}_", model, tol, max_iter, with_refnlp=True,
                 with_simplex=with_simplex)
    out["count"] = np.array([count])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, "written", count)


def main():
    ref.build()
    # basic: min x, 1 <= x <= 2, no rows.
    basic = Model(m=0, n=1, colptr=np.array([0, 0]), rowidx=np.zeros(0, np.int32),
                  vals=np.zeros(0), obj=np.array([1.0]), col_lower=np.array([1.0]),
                  col_upper=np.array([2.0]), row_lower=np.zeros(0), row_upper=np.zeros(0))
    out = {}
    add_case(out, "k0_", basic, 1e-4, 10000, with_refnlp=False)
    out["count"] = np.array([1])
    np.savez_compressed(os.path.join(HERE, "basic.npz"), **out)
    family_group("feasible8", FEASIBLE, 8, 42, 50, 1e-8, 100000)
    family_group("vs_simplex10", FEASIBLE, 10, 123, 30, 1e-4, 100000, with_simplex=True)
    family_group("infeasible8", RANDOM, 8, 4242, 30, 1e-4, 50000)
    family_group("loose8", LOOSE, 8, 4242, 30, 1e-4, 50000, prefix_family=RANDOM,
                 prefix_count=30)
    family_group("gpu_vs_cpu6", FEASIBLE, 6, 42, 20, 1e-6, 10000)
    family_group("repeatable30", FEASIBLE, 30, 613, 5, 1e-6, 20000)
    # The random sparse LP: 200 x 500 (seeds 0-2) with the whole problem stored, and the
    # 2000 x 5000 CPU-runnable case (seed 0) by digest and results.
    out = {}
    for s in range(3):
        model = random_sparse_lp(m=200, n=500, seed=s)
        add_case(out, f"k{s}_", model, 1e-4, -1, with_refnlp=False, with_simplex=True)
    out["count"] = np.array([3])
    np.savez_compressed(os.path.join(HERE, "config0_small.npz"), **out)
    print("config0_small written")
    out = {}
    model = random_sparse_lp(m=2000, n=5000, seed=0)
    add_case(out, "k0_", model, 1e-4, -1, with_refnlp=False, with_simplex=True,
             store_model=False)
    r8 = ref.pdlp_solve(*(lambda sc: (model.m, model.n, sc["colptr"], sc["rowidx"], sc["vals"],
                                      sc["cost"], sc["lower"], sc["upper"]))(
        ref.scale_model(model)), 1e-8, -1)
    out["k0_ref8_status"] = np.array([r8["status"]])
    out["k0_ref8_iterations"] = np.array([r8["iterations"]])
    out["k0_ref8_x"] = r8["x"]
    out["k0_ref8_y"] = r8["y"]
    out["count"] = np.array([1])
    np.savez_compressed(os.path.join(HERE, "config0.npz"), **out)
    print("config0 written")
    config4()


def config4():
    """The differentiable layer's LPs (500 x 1200 random sparse, seeds 0-7): the reference dual
    simplex's objective, x and row duals (model space), with the model digest."""
    out = {}
    for k in range(8):
        model = random_sparse_lp(m=500, n=1200, seed=k)
        ds = ref.dual_simplex(model)
        ok, _ = ref.verify_optimal(model, ds["x"], ds["y"])
        out[f"k{k}_digest"] = np.frombuffer(bytes.fromhex(model_digest(model)), dtype=np.uint8)
        out[f"k{k}_simplex"] = np.array([ds["status"], ds["objective"], ds["iterations"], int(ok)])
        out[f"k{k}_x"] = ds["x"]
        out[f"k{k}_y"] = ds["y"]
    out["count"] = np.array([8])
    np.savez_compressed(os.path.join(HERE, "config4.npz"), **out)
    print("config4 written")


if __name__ == "__main__":
    main()
