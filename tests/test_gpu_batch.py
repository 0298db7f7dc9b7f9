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


def test_batch_uneven_sizes_match_single_solves(engine):
    """Random sparse LPs of uneven sizes (m from 60 to 600): each batched answer matches the
    single-LP engine's objective to 1e-6 relative at 1e-6, FP64 and FP32 storage."""
    from samaya_gb300.batch import BatchSolver
    from samaya_gb300.generators import random_sparse_lp
    from samaya_gb300.problem import make_problem
    rng = np.random.default_rng(5)
    probs = []
    for k in range(12):
        m = int(rng.integers(60, 600))
        n = int(np.ceil(m * rng.uniform(2, 3)))
        lp, _ = make_problem(random_sparse_lp(m, n, seed=100 + k))
        probs.append(lp)
    opts = engine.PdlpOptions(tol=1e-6, algorithm=engine.ENHANCED)
    res = BatchSolver.from_problems(probs, opts).solve()
    for lp, r in zip(probs, res):
        single = engine.solve_pdlp(lp, opts)
        assert r.status == single.status == engine.OPTIMAL
        a = float(np.dot(lp.cost, r.x))
        b = float(np.dot(lp.cost, single.x))
        assert abs(a - b) <= 1e-6 * (1 + abs(b)) * 10, (a, b)
    res32 = BatchSolver.from_problems(probs, engine.PdlpOptions(
        tol=1e-4, algorithm=engine.ENHANCED, precision=engine.FP32_REFINED)).solve()
    for lp, r in zip(probs, res32):
        single = engine.solve_pdlp(lp, engine.PdlpOptions(tol=1e-6, algorithm=engine.ENHANCED))
        assert r.status == engine.OPTIMAL
        a = float(np.dot(lp.cost, r.x))
        b = float(np.dot(lp.cost, single.x))
        assert abs(a - b) <= 1e-3 * (1 + abs(b)), (a, b)


def test_batch_shared_matrix_node_relaxations(engine):
    """Facility location node relaxations sharing one matrix: every node's objective matches a
    single-LP solve of that node to 1e-5 relative."""
    from samaya_gb300.batch import BatchSolver
    from samaya_gb300.generators import facility_location_lp, facility_node_bounds
    from samaya_gb300.problem import make_problem
    model = facility_location_lp(20, 60, seed=3)
    lp, sc = make_problem(model)
    bounds = _node_problems(lp, sc, model, facility_node_bounds(model, 20, 8, seed=4))
    opts = engine.PdlpOptions(tol=1e-6, algorithm=engine.ENHANCED)
    res = BatchSolver.shared(lp, bounds, opts).solve()
    for (lo, up), r in zip(bounds, res):
        node = engine.LpProblem(m=lp.m, n=lp.n, colptr=lp.colptr, rowidx=lp.rowidx, vals=lp.vals,
                                cost=lp.cost, lower=lo, upper=up)
        single = engine.solve_pdlp(node, opts)
        assert r.status == single.status
        if r.status == engine.OPTIMAL:
            a = float(np.dot(lp.cost, r.x))
            b = float(np.dot(lp.cost, single.x))
            assert abs(a - b) <= 1e-5 * (1 + abs(b)), (a, b)
