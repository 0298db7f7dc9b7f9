"""The oracle (a C restatement of the reference's CPU PDLP) agrees bit-for-bit with the
reference's own code, through the golden fixtures made from the reference
(tests/golden/make_golden.py), and with the reference library itself where it is built."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import GROUPS, load_group


@pytest.mark.parametrize("group", GROUPS)
def test_oracle_matches_reference_fixtures(oracle, group):
    cases = load_group(group)
    for c in cases:
        lp = c.lp
        r = oracle.pdlp_solve(*lp.arrays(), tol=c.tol, max_iter=c.max_iter)
        assert r.status == c.ref_status, (group, c.k)
        assert r.iterations == c.ref_iterations, (group, c.k)
        assert np.array_equal(r.x, c.ref_x), (group, c.k)
        assert np.array_equal(r.y, c.ref_y), (group, c.k)
        assert np.array_equal(np.array([r.primal_residual, r.dual_residual, r.gap]), c.ref_res)
        if c.ref_dual_ray is not None:
            assert np.array_equal(r.dual_ray, c.ref_dual_ray)
        else:
            assert r.dual_ray is None
        if c.ref_primal_ray is not None:
            assert np.array_equal(r.primal_ray, c.ref_primal_ray)
        else:
            assert r.primal_ray is None


@pytest.mark.parametrize("group", GROUPS)
def test_oracle_scaling_matches_reference_fixtures(oracle, group):
    for c in load_group(group):
        m = c.model
        col, row = oracle.compute_scaling(m.m, m.n, m.colptr, m.rowidx, m.vals)
        assert np.array_equal(col, c.col_scale) and np.array_equal(row, c.row_scale)
        colptr, rowidx, vals, cost, lower, upper = oracle.make_problem(m, col, row)
        assert np.array_equal(colptr, c.lp.colptr) and np.array_equal(rowidx, c.lp.rowidx)
        assert np.array_equal(vals, c.lp.vals) and np.array_equal(cost, c.lp.cost)
        assert np.array_equal(lower, c.lp.lower) and np.array_equal(upper, c.lp.upper)


def test_reference_statistics_of_the_families():
    """The groups exercise every outcome the reference tests count on: optima, Farkas
    certificates and improving rays."""
    statuses = {g: [c.ref_status for c in load_group(g)] for g in GROUPS}
    assert statuses["feasible8"].count(0) > 10
    assert statuses["infeasible8"].count(1) > 0
    assert statuses["loose8"].count(2) > 0


def test_config0_full_size_oracle(oracle):
    """The 2000 x 5000 random sparse LP (seed 0) at 1e-4: the oracle reproduces the reference's
    iterations and answer bit-for-bit (the model is regenerated from its seed and checked by
    digest)."""
    import hashlib
    import os

    from conftest import GOLDEN
    from samaya_gb300.generators import random_sparse_lp
    with np.load(os.path.join(GOLDEN, "config0.npz")) as z:
        d = {k: z[k] for k in z.files}
    model = random_sparse_lp(m=2000, n=5000, seed=0)
    h = hashlib.sha256()
    for k in ("colptr", "rowidx", "vals", "obj", "col_lower", "col_upper", "row_lower",
              "row_upper"):
        h.update(np.ascontiguousarray(getattr(model, k)).tobytes())
    h.update(str((model.m, model.n, model.maximize, model.obj_offset)).encode())
    assert h.digest() == d["k0_digest"].tobytes()
    col, row = oracle.compute_scaling(model.m, model.n, model.colptr, model.rowidx, model.vals)
    colptr, rowidx, vals, cost, lower, upper = oracle.make_problem(model, col, row)
    r = oracle.pdlp_solve(model.m, model.n, colptr, rowidx, vals, cost, lower, upper, tol=1e-4)
    assert r.status == int(d["k0_ref_status"][0])
    assert r.iterations == int(d["k0_ref_iterations"][0])
    assert np.array_equal(r.x, d["k0_ref_x"])
    assert np.array_equal(r.y, d["k0_ref_y"])


def test_oracle_against_live_reference(oracle):
    """Where the reference library is built (only in a container with the reference checkout),
    compare on fresh draws of every family too."""
    from oracle import ref
    if not ref.available():
        pytest.skip("the reference checkout is not present")
    from samaya_gb300.model import Model
    for family, seed in ((0, 7), (1, 8), (3, 9), (4, 10)):
        for k in range(10):
            model = Model.from_dict(ref.random_lp(family, 12, 12, seed, k))
            sc = ref.scale_model(model)
            args = (model.m, model.n, sc["colptr"], sc["rowidx"], sc["vals"], sc["cost"],
                    sc["lower"], sc["upper"])
            a = ref.pdlp_solve(*args, tol=1e-6, max_iter=20000)
            b = oracle.pdlp_solve(*args, tol=1e-6, max_iter=20000)
            assert a["status"] == b.status and a["iterations"] == b.iterations
            assert np.array_equal(a["x"], b.x) and np.array_equal(a["y"], b.y)


@pytest.mark.parametrize("group", GROUPS)
def test_engine_host_scaling_matches_reference_fixtures(group):
    """The engine library's host-side compute_scaling + make_problem (C++, no GPU) gives the
    reference's scaled LpProblem bit-for-bit."""
    from samaya_gb300 import _native
    _native.load(build_if_missing=True)
    from samaya_gb300.problem import make_problem
    for c in load_group(group):
        lp, sc = make_problem(c.model)
        assert np.array_equal(sc.col, c.col_scale) and np.array_equal(sc.row, c.row_scale)
        for k in ("colptr", "rowidx", "vals", "cost", "lower", "upper"):
            assert np.array_equal(getattr(lp, k), getattr(c.lp, k)), (group, c.k, k)


def test_verifier_restatement_on_the_dual_simplex_solutions(oracle):
    """The oracle's restatement of the reference's verify_lp_optimality passes the reference
    dual simplex's solutions of the 500 x 1200 LPs (their objectives to the bit) and rejects
    perturbed ones; where the reference is built, it agrees with the reference's verifier on
    every case."""
    import numpy as np
    from oracle import ref
    from samaya_gb300.generators import random_sparse_lp
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "config4.npz"))
    live = ref.available()
    for k in range(int(d["count"][0])):
        model = random_sparse_lp(500, 1200, seed=k)
        x, y = d[f"k{k}_x"], d[f"k{k}_y"]
        for xx, yy, expect in ((x, y, True), (x * 1.0001, y, False), (x, y * 1.01, False)):
            ok, rep = oracle.verify_lp(model, xx, yy)
            assert ok == expect, (k, rep)
            if expect:
                assert rep["objective"] == float(d[f"k{k}_simplex"][1])
            if live:
                ok_ref, obj_ref = ref.verify_optimal(model, xx, yy)
                assert ok_ref == ok and obj_ref == rep["objective"]
