"""Inert rows left out of the step launches: a row of A with no nonzeros whose logical has no
cost and 0 within its bounds keeps its dual and its logical at 0 in every iterate, so the
solves step only the other rows. Leaving them out must not change a bit of any solve (status,
iterations, x, y) in any precision or algorithm, against the same solve with every row
stepped (keep_inert_rows)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _with_empty_rows(model, seed):
    """The model with empty rows inserted (first, last and at random places) whose bounds all
    hold 0: free, fixed at 0, boxed around 0, one-sided."""
    from samaya_gb300.model import Model
    rng = np.random.default_rng(seed)
    bounds = [(-np.inf, np.inf), (0.0, 0.0), (-1.0, 2.0), (-np.inf, 0.5), (0.0, np.inf)]
    extra = 40
    m = model.m + extra
    empty = np.sort(np.concatenate([[0, m - 1], rng.choice(np.arange(1, m - 1), extra - 2,
                                                           replace=False)]))
    keep = np.setdiff1d(np.arange(m), empty)
    row_lower = np.empty(m)
    row_upper = np.empty(m)
    row_lower[keep], row_upper[keep] = model.row_lower, model.row_upper
    for t, i in enumerate(empty):
        row_lower[i], row_upper[i] = bounds[t % len(bounds)]
    return Model(**{**model.__dict__, "m": m, "rowidx": keep[model.rowidx].astype(np.int32),
                    "row_lower": row_lower, "row_upper": row_upper})


def _inert(model):
    """Rows with no nonzeros whose bounds hold 0 (the logicals carry no cost)."""
    empty = np.bincount(model.rowidx, minlength=model.m) == 0
    return int((empty & (model.row_lower <= 0) & (model.row_upper >= 0)).sum())


def _models():
    from samaya_gb300 import generators as g
    out = {"powerlaw": g.power_law_lp(m=20000, n=40000, seed=2),
           "random+empty": _with_empty_rows(g.random_sparse_lp(300, 800, seed=5), seed=1),
           "transport+empty": _with_empty_rows(g.transportation_lp(30, 60, seed=2), seed=2)}
    return {k: (v, _inert(v)) for k, v in out.items()}


CASES = [("REFERENCE", "FP64", 1e-6), ("HALPERN", "FP64", 1e-6),
         ("HALPERN", "FP32_THEN_FP64", 1e-6), ("ENHANCED", "FP32_REFINED", 1e-7)]
# The Halpern cases converge within this budget; the reference algorithm on the power-law LP and
# the enhanced refinement on two of the LPs stop at the limit, and the comparison then covers
# the iteration limit's answer.
MAX_ITERATIONS = 50000


@pytest.fixture(scope="module")
def models():
    return _models()


@pytest.mark.parametrize("name", ["powerlaw", "random+empty", "transport+empty"])
@pytest.mark.parametrize("algorithm,precision,tol", CASES)
def test_leaving_inert_rows_out_changes_no_bit(engine, models, name, algorithm, precision,
                                               tol):
    from samaya_gb300.problem import make_problem
    model, inert = models[name]
    assert inert > 0
    lp, _ = make_problem(model)
    out = []
    for keep in (False, True):
        opts = engine.PdlpOptions(tol=tol, precision=getattr(engine, precision),
                                  algorithm=getattr(engine, algorithm), inner_tol=1e-4,
                                  autotune=False, keep_inert_rows=keep,
                                  max_iterations=MAX_ITERATIONS)
        with engine.PdlpSolver(lp, opts) as s:
            rows, tiles, _, _ = s.step_rows()
            assert rows == (lp.m if keep else lp.m - inert)
            assert tiles > 0
            out.append(s.solve())
    a, b = out
    assert a.status == b.status
    assert a.status == engine.OPTIMAL or algorithm != "HALPERN"
    assert a.iterations == b.iterations
    assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)


def test_device_built_engine_finds_the_same_inert_rows(engine, models):
    """sg_pdlp_create_model marks the inert rows on the device: the same rows and tiles as the
    engine built from the host LpProblem."""
    from samaya_gb300.problem import make_problem
    opts = engine.PdlpOptions(autotune=False)
    for model, _ in models.values():
        lp, _ = make_problem(model)
        with engine.PdlpSolver(lp, opts) as s:
            host = s.step_rows()
        with engine.PdlpSolver.from_model(model, opts) as s:
            assert s.step_rows() == host


def test_an_empty_row_that_excludes_zero_is_stepped(engine):
    """An empty row whose bounds exclude 0 (the LP is then infeasible) is not inert: it is
    stepped, and the solve agrees with the one that steps every row."""
    from samaya_gb300 import generators as g
    from samaya_gb300.problem import make_problem
    base = _with_empty_rows(g.random_sparse_lp(200, 500, seed=7), seed=3)
    rl, ru = base.row_lower.copy(), base.row_upper.copy()
    empty = np.flatnonzero(np.bincount(base.rowidx, minlength=base.m) == 0)
    rl[empty[3]], ru[empty[3]] = 1.0, 2.0
    from samaya_gb300.model import Model
    model = Model(**{**base.__dict__, "row_lower": rl, "row_upper": ru})
    assert _inert(model) == _inert(base) - 1
    lp, _ = make_problem(model)
    out = []
    for keep in (False, True):
        opts = engine.PdlpOptions(tol=1e-6, autotune=False, keep_inert_rows=keep,
                                  max_iterations=100000)
        with engine.PdlpSolver(lp, opts) as s:
            rows, _, _, _ = s.step_rows()
            assert rows == (lp.m if keep else lp.m - _inert(model))
            out.append(s.solve())
    a, b = out
    assert a.status == b.status and a.status != engine.OPTIMAL
    assert a.iterations == b.iterations
