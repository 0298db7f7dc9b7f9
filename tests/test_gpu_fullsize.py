"""Full-size solves checked against answers the engine did not produce: the reference's own
PDLP and dual simplex (golden fixtures of the 2000 x 5000 random sparse LP), an independent
optimum (scipy HiGHS, ``tests/golden/make_optima.py``) of the 3000 x 2,000,000 transportation
LP, and the oracle's restatement of the reference's verifier (``verify_lp_optimality``,
src/verify/verify.cpp:251, default tolerances 1e-6) on every answer."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _optima():
    with open(os.path.join(GOLDEN, "optima.json")) as f:
        return json.load(f)


def _config0():
    with np.load(os.path.join(GOLDEN, "config0.npz")) as z:
        return {k: z[k] for k in z.files}


def _solve_verified(engine, oracle, model, opts):
    """Solves the model's LpProblem, maps the answer back to the model (the reference's
    solve_pdlp_lp mapping) and runs the verifier restatement on it."""
    from samaya_gb300.problem import make_problem, model_solution
    lp, sc = make_problem(model)
    r = engine.solve_pdlp(lp, opts)
    x, _, dual, obj = model_solution(model, sc, r.x, r.y)
    ok, rep = oracle.verify_lp(model, x, dual)
    return r, obj, ok, rep


def test_config0_full_size_reference_algorithm_matches_the_reference_pdlp(engine, oracle):
    """2000 x 5000 random sparse LP (seed 0), plain FP64 with the reference algorithm at 1e-4:
    the reference's iteration count (6,720), its answer to round-off, the objective within
    1e-4 relative of the reference PDLP's, and the verifier's bound and row checks."""
    from samaya_gb300.generators import random_sparse_lp
    from samaya_gb300.problem import make_problem
    d = _config0()
    model = random_sparse_lp(2000, 5000, seed=0)
    lp, _ = make_problem(model)
    r = engine.solve_pdlp(lp, engine.PdlpOptions(tol=1e-4, algorithm=engine.REFERENCE))
    assert r.status == engine.OPTIMAL == int(d["k0_ref_status"][0])
    assert r.iterations == int(d["k0_ref_iterations"][0])
    ref_obj = float(lp.cost @ d["k0_ref_x"])
    obj = float(lp.cost @ r.x)
    assert abs(obj - ref_obj) <= 1e-4 * (1 + abs(ref_obj))
    assert np.max(np.abs(r.x - d["k0_ref_x"])) <= 1e-6 * (1 + np.max(np.abs(d["k0_ref_x"])))


@pytest.mark.parametrize("name,precision,algorithm", [
    ("fp64_reference", 0, 0), ("fp64_halpern", 0, 2), ("mixed_halpern", 2, 2),
    ("refined_halpern", 1, 2)])
def test_config0_full_size_at_1e8_matches_the_dual_simplex(engine, oracle, name, precision,
                                                           algorithm):
    """The same LP to 1e-8 relative KKT in each precision mode: the model objective within
    1e-8 relative of the reference dual simplex's (the fixture's k0_simplex), bound and row
    violations within 1e-5 in every mode, and the whole verifier restatement passing for the
    reference algorithm (as the reference's own CPU PDLP answers do). The verifier checks each
    row and column at 1e-6 on its own, which a 1e-8 relative KKT answer need not meet on every
    one (a column a few 1e-6 off its bound with a reduced cost: measured once in the refined
    mode, dual violation 0.07 with the objective still within 1e-8)."""
    from samaya_gb300.generators import random_sparse_lp
    d = _config0()
    simplex = float(d["k0_simplex"][1])
    model = random_sparse_lp(2000, 5000, seed=0)
    opts = engine.PdlpOptions(tol=1e-8, precision=precision, algorithm=algorithm,
                              inner_tol=1e-6 if precision == 2 else 1e-4)
    r, obj, ok, rep = _solve_verified(engine, oracle, model, opts)
    assert r.status == engine.OPTIMAL, (name, r.status_name)
    assert abs(obj - simplex) <= 1e-8 * (1 + abs(simplex)), (name, obj, simplex)
    assert rep["bound"] <= 1e-5 and rep["row"] <= 1e-5, (name, rep)
    if name == "fp64_reference":
        assert ok, (name, rep)


@pytest.mark.parametrize("name,precision,algorithm", [
    ("mixed_halpern", 2, 2), ("fp64_halpern", 0, 2), ("refined_halpern", 1, 2)])
def test_transport_full_size_verified_against_an_independent_optimum(engine, oracle, name,
                                                                     precision, algorithm):
    """The bench's transportation LP (1000 supplies x 2000 demands: 3000 rows, 2,000,000
    columns, 4,000,000 nonzeros, seed 0) to 1e-8 in the bench's mode and the others: the
    objective is within 1e-8 relative of the HiGHS optimum, and the verifier restatement finds
    bound and row violations within 1e-5. (The relative KKT test bounds 2-norms over all rows
    and columns and the total complementarity x'd; the verifier checks each of the 3,000 rows
    and 2,000,000 columns on its own at 1e-6: at 1e-8 a row may be off by ~1e-6 of its scale,
    and a column whose x_j is a few 1e-6 above 0 may keep a large reduced cost. A 1e-9 solve
    passes at the verifier's defaults, below.)"""
    from samaya_gb300.generators import transportation_lp
    opt = _optima()["transport"]
    assert opt["status"] == 0
    model = transportation_lp(1000, 2000, seed=0)
    opts = engine.PdlpOptions(tol=1e-8, precision=precision, algorithm=algorithm,
                              inner_tol=1e-6 if precision == 2 else 1e-4)
    r, obj, ok, rep = _solve_verified(engine, oracle, model, opts)
    assert r.status == engine.OPTIMAL, (name, r.status_name)
    assert abs(obj - opt["objective"]) <= 1e-8 * (1 + abs(opt["objective"])), (
        name, obj, opt["objective"])
    assert rep["bound"] <= 1e-5 and rep["row"] <= 1e-5, (name, rep)


def test_transport_full_size_at_1e9_passes_the_verifier(engine, oracle):
    """The bench's mode (FP32 then FP64, Halpern) to 1e-9 on the full transportation LP: the
    answer passes the verifier restatement at its default tolerances (1e-6)."""
    from samaya_gb300.generators import transportation_lp
    model = transportation_lp(1000, 2000, seed=0)
    opts = engine.PdlpOptions(tol=1e-9, precision=engine.FP32_THEN_FP64,
                              algorithm=engine.HALPERN, inner_tol=1e-6)
    r, obj, ok, rep = _solve_verified(engine, oracle, model, opts)
    assert r.status == engine.OPTIMAL, r.status_name
    assert ok, rep
