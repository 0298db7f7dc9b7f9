"""Batched PDLP (one persistent launch over many LPs) against the single-LP engine, the
reference's CPU PDLP fixtures and its simplex oracles."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_group

pytestmark = pytest.mark.gpu


def _node_problems(lp, scaling, model, bounds):
    """LpProblem bounds of branch-and-bound nodes: model column bounds / column scale, rows
    unchanged."""
    out = []
    for lo, up in bounds:
        lower = lp.lower.copy()
        upper = lp.upper.copy()
        lower[:lp.n] = lo / scaling.col
        upper[:lp.n] = up / scaling.col
        out.append((lower, upper))
    return out


def test_batch_matches_reference_families(engine):
    """The 50 random LPs of pdlp_random_feasible in one launch: where the reference's CPU PDLP
    finds an optimum so does the batch, with the objective within 1e-6 (1 + |ref|) of the dense
    reference simplex (tests/test_pdlp.cpp:85-232); the batch runs no infeasibility or
    unboundedness checks, so on the reference's unbounded LPs it must stop without claiming an
    optimum."""
    from samaya_gb300.batch import BatchSolver
    cases = load_group("feasible8")
    s = BatchSolver.from_problems([c.lp for c in cases],
                                  engine.PdlpOptions(tol=1e-8, max_iterations=20000))
    res = s.solve()
    bad = []
    for c, r in zip(cases, res):
        if c.ref_status != engine.OPTIMAL:
            if r.status == engine.OPTIMAL:
                bad.append(("claims optimum", c.k, c.ref_status))
            continue
        if r.status != c.ref_status:
            bad.append(("status", c.k, r.status, c.ref_status))
            continue
        if r.status == engine.OPTIMAL:
            xm = r.x[:c.lp.n] * c.col_scale
            obj = c.model.obj_offset + float(np.dot(c.model.obj, xm))
            ref = float(c.refnlp[1])
            if abs(obj - ref) > 1e-6 * (1 + abs(ref)):
                bad.append(("objective", c.k, obj, ref))
    assert not bad, bad
    again = s.solve()
    assert all(np.array_equal(a.x, b.x) and a.iterations == b.iterations
               for a, b in zip(res, again))
    s.close()


def _oracle_objective(lp, tol):
    """The reference's CPU PDLP (the oracle) on an LpProblem: (status, objective c'v)."""
    from oracle import oracle as o
    r = o.pdlp_solve(*lp.arrays(), tol=tol)
    return r.status, float(np.dot(lp.cost, r.x))


def test_batch_uneven_sizes_match_the_oracle(engine, oracle):
    """Random sparse LPs of uneven sizes (m from 60 to 400) in one launch, FP64 at 1e-7 and
    FP32 storage at 1e-4: every batched answer is optimal with the objective of the
    reference's CPU PDLP (the oracle, 1e-8) within 1e-5 relative (FP64) and 1e-3 (FP32)."""
    from samaya_gb300.batch import BatchSolver
    from samaya_gb300.generators import random_sparse_lp
    from samaya_gb300.problem import make_problem
    rng = np.random.default_rng(5)
    probs = []
    for k in range(8):
        m = int(rng.integers(60, 400))
        n = int(np.ceil(m * rng.uniform(2, 3)))
        lp, _ = make_problem(random_sparse_lp(m, n, seed=100 + k))
        probs.append(lp)
    refs = [_oracle_objective(lp, 1e-8) for lp in probs]
    assert all(st == oracle.OPTIMAL for st, _ in refs)
    for prec, tol, bar in ((engine.FP64, 1e-7, 1e-5), (engine.FP32_REFINED, 1e-4, 1e-3)):
        res = BatchSolver.from_problems(probs, engine.PdlpOptions(
            tol=tol, algorithm=engine.ENHANCED, precision=prec)).solve()
        for lp, r, (_, ref) in zip(probs, res, refs):
            assert r.status == engine.OPTIMAL
            a = float(np.dot(lp.cost, r.x))
            assert abs(a - ref) <= bar * (1 + abs(ref)), (prec, a, ref)


def test_batch_shared_matrix_node_relaxations(engine, oracle):
    """Facility-location node relaxations sharing one matrix (20 facilities x 60 customers, 8
    nodes with 5% of the open variables fixed) in one launch at 1e-8: every node's batched
    answer is optimal with the node's independent optimum (scipy HiGHS) to 1e-6 relative, and,
    mapped back to the node's model, at least 80% pass the verifier restatement (the
    reference's acceptance bar for PDLP answers, tests/test_pdlp.cpp:497-540). (The
    reference's CPU PDLP stops at its iteration limit on three of these nodes, so it cannot
    serve as their optimum.)"""
    import dataclasses

    from conftest import highs_objective
    from samaya_gb300.batch import BatchSolver
    from samaya_gb300.generators import facility_location_lp, facility_node_bounds
    from samaya_gb300.problem import make_problem, model_solution
    model = facility_location_lp(20, 60, seed=3)
    lp, sc = make_problem(model)
    node_bounds = facility_node_bounds(model, 20, 8, seed=4)
    bounds = _node_problems(lp, sc, model, node_bounds)
    opts = engine.PdlpOptions(tol=1e-8, algorithm=engine.ENHANCED)
    res = BatchSolver.shared(lp, bounds, opts).solve()
    verified, reports = 0, []
    for (mlo, mup), r in zip(node_bounds, res):
        node_model = dataclasses.replace(model, col_lower=mlo, col_upper=mup)
        st, ref = highs_objective(node_model)
        assert st == 0 and r.status == engine.OPTIMAL, (st, r.status)
        x, _, dual, obj = model_solution(node_model, sc, r.x, r.y)
        assert abs(obj - ref) <= 1e-6 * (1 + abs(ref)), (obj, ref)
        ok, rep = oracle.verify_lp(node_model, x, dual)
        verified += int(ok)
        reports.append(rep)
    assert verified >= 0.8 * len(res), reports


def test_batch_halpern_matches_the_oracle_and_the_node_optima(engine, oracle):
    """The reflected Halpern iteration in the batched engine (T(z) measured, restarted to and
    returned): uneven random LPs at 1e-7 against the oracle's objectives (1e-5 relative, FP64;
    1e-3 in FP32 storage at 1e-4), the facility-location node relaxations at 1e-8 against their
    HiGHS optima (1e-6 relative), and a re-run repeats every answer's bits."""
    import dataclasses

    from conftest import highs_objective
    from samaya_gb300.batch import BatchSolver
    from samaya_gb300.generators import (facility_location_lp, facility_node_bounds,
                                         random_sparse_lp)
    from samaya_gb300.problem import make_problem, model_solution
    rng = np.random.default_rng(6)
    probs = []
    for k in range(6):
        m = int(rng.integers(60, 300))
        n = int(np.ceil(m * rng.uniform(2, 3)))
        probs.append(make_problem(random_sparse_lp(m, n, seed=200 + k))[0])
    refs = [_oracle_objective(lp, 1e-8) for lp in probs]
    for prec, tol, bar in ((engine.FP64, 1e-7, 1e-5), (engine.FP32_REFINED, 1e-4, 1e-3)):
        s = BatchSolver.from_problems(probs, engine.PdlpOptions(
            tol=tol, algorithm=engine.HALPERN, precision=prec))
        res = s.solve()
        again = s.solve()
        s.close()
        for lp, r, r2, (st, ref) in zip(probs, res, again, refs):
            assert st == oracle.OPTIMAL and r.status == engine.OPTIMAL
            a = float(np.dot(lp.cost, r.x))
            assert abs(a - ref) <= bar * (1 + abs(ref)), (prec, a, ref)
            assert r.iterations == r2.iterations and np.array_equal(r.x, r2.x)
    model = facility_location_lp(20, 60, seed=3)
    lp, sc = make_problem(model)
    node_bounds = facility_node_bounds(model, 20, 8, seed=4)
    res = BatchSolver.shared(lp, _node_problems(lp, sc, model, node_bounds),
                             engine.PdlpOptions(tol=1e-8, algorithm=engine.HALPERN)).solve()
    for (mlo, mup), r in zip(node_bounds, res):
        node_model = dataclasses.replace(model, col_lower=mlo, col_upper=mup)
        st, ref = highs_objective(node_model)
        assert st == 0 and r.status == engine.OPTIMAL, (st, r.status)
        _, _, _, obj = model_solution(node_model, sc, r.x, r.y)
        assert abs(obj - ref) <= 1e-6 * (1 + abs(ref)), (obj, ref)
