"""The seeded synthetic workloads (samaya_gb300/generators.py) have the shapes, sizes and value
distributions of the benchmark configurations, at small sizes (CPU only)."""
from __future__ import annotations

import numpy as np

from samaya_gb300 import generators as g


def _cols(model):
    return [model.rowidx[model.colptr[j]:model.colptr[j + 1]] for j in range(model.n)]


def test_random_sparse_lp_shape():
    """m equality rows, 6 distinct rows per column with N(0,1) values, 0 <= x <= 10, b = A x0
    (so the LP is feasible), deterministic in the seed."""
    md = g.random_sparse_lp(200, 500, seed=3)
    assert md.m == 200 and md.n == 500 and md.colptr[-1] == 6 * 500
    for rows in _cols(md):
        assert len(np.unique(rows)) == 6 and np.all(np.diff(rows) > 0)
    assert np.array_equal(md.row_lower, md.row_upper)
    assert np.all(md.col_lower == 0.0) and np.all(md.col_upper == 10.0)
    assert abs(float(np.mean(md.vals))) < 0.1 and 0.9 < float(np.std(md.vals)) < 1.1
    again = g.random_sparse_lp(200, 500, seed=3)
    assert np.array_equal(again.vals, md.vals) and np.array_equal(again.obj, md.obj)


def test_transportation_lp_shape():
    """S x D columns, two +1 entries each (supply row, demand row), integer costs in [1, 100],
    balanced supply and demand, x >= 0 with no upper bound."""
    md = g.transportation_lp(10, 20, seed=1)
    assert md.n == 200 and md.m == 30 and md.colptr[-1] == 400
    assert np.all(md.vals == 1.0)
    assert np.all(md.rowidx[0::2] < 10) and np.all(md.rowidx[1::2] >= 10)
    assert np.all(md.obj == np.round(md.obj)) and md.obj.min() >= 1 and md.obj.max() <= 100
    sup, dem = md.row_lower[:10], md.row_lower[10:]
    assert abs(sup.sum() - dem.sum()) <= 1e-9 * sup.sum()
    assert np.all(md.col_lower == 0.0) and np.all(np.isinf(md.col_upper))


def test_power_law_lp_shape():
    """6 distinct rows per column drawn Zipf(1.5) through a row permutation (so a few rows are
    very long), about 30% inequality rows, 0 <= x <= 5."""
    md = g.power_law_lp(m=2000, n=4000, seed=2)
    assert md.colptr[-1] == 6 * 4000
    for rows in _cols(md)[:500]:
        assert len(np.unique(rows)) == 6
    lengths = np.bincount(md.rowidx, minlength=md.m)
    assert lengths.max() > 50 * lengths.mean()
    ineq = np.isinf(md.row_lower)
    assert 0.25 < ineq.mean() < 0.35
    assert np.all(md.row_upper[~ineq] == md.row_lower[~ineq])
    assert np.all(md.col_lower == 0.0) and np.all(md.col_upper == 5.0)


def test_facility_location_and_node_bounds():
    """F open columns (capacity rows) then F x C assignment columns (demand row, capacity row);
    C demand equalities and F capacity rows <= 0; node bounds fix 5% of the open variables."""
    md = g.facility_location_lp(10, 40, seed=0)
    assert md.n == 10 + 400 and md.m == 50 and md.colptr[-1] == 10 + 800
    assert np.all(md.row_lower[:40] == 1.0) and np.all(md.row_upper[:40] == 1.0)
    assert np.all(np.isinf(md.row_lower[40:])) and np.all(md.row_upper[40:] == 0.0)
    nodes = g.facility_node_bounds(md, facilities=10, count=8, fraction=0.2, seed=1)
    assert len(nodes) == 8
    for lo, up in nodes:
        fixed = np.flatnonzero(lo[:10] == up[:10])
        assert len(fixed) == 2 and set(np.unique(lo[fixed])) <= {0.0, 1.0}
        assert np.array_equal(lo[10:], md.col_lower[10:])


def test_batch_a_sizes():
    """m ~ U[100, 5000], n = ceil(m U[2, 3])."""
    sizes = g.batch_a_sizes(64, seed=0)
    assert len(sizes) == 64
    for m, n in sizes:
        assert 100 <= m <= 5000 and 2 * m <= n <= 3 * m + 1
