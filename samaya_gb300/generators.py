"""Seeded synthetic LP generators for the PDLP workloads (numpy ``default_rng``).

Each returns a ``Model`` (min sense).  The shapes and distributions are the benchmark
configurations of the PDLP path:

* ``random_sparse_lp``  — m equality rows, n columns, k distinct uniform rows per column with
  N(0,1) values; x0 U[0,1] on a random half of the columns; b = A x0; 0 <= x <= 10;
  c = A'y0 + s with y0 ~ N(0,1), s ~ U[0,1].  (2000 x 5000 is the CPU-runnable case; batches and
  the differentiable layer draw many of these.)
* ``transportation_lp`` — S supplies x D demands, all-ones matrix with 2 nonzeros per column,
  integer costs U[1,100], integer supplies U[500,1500], integer demands U[200,800] rescaled to
  the total supply; equality rows; x >= 0.
* ``power_law_lp``      — m x n with k entries per column whose rows are Zipf(1.5) draws
  (truncated at m by rejection, made distinct within a column by redrawing) through a random
  row permutation; N(0,1) values; 70% equality / 30% <= rows with b = A x0 (+ U[0,1] slack on
  the inequalities), x0 ~ U[0,1], 0 <= x <= 5, c = A'y0 + s with y0 ~ N(0,1), y0 >= 0 on the
  inequality rows, s ~ U[0,1].
* ``facility_location_lp`` — capacitated facility location relaxation (F facilities x C
  customers: F open variables and F*C assignments in [0,1]; C demand equalities, F capacity
  rows), and ``facility_node_bounds`` — branch-and-bound style node bounds that fix a random
  fraction of the open variables to 0 or 1.
"""
from __future__ import annotations

import math

import numpy as np

from .model import Model


def _distinct_rows(rng, m, n, k, draw):
    """(n, k) row indices, distinct within each column, sorted; ``draw(size)`` samples rows."""
    rows = draw((n, k))
    for _ in range(1000):
        rows.sort(axis=1)
        dup = np.zeros(rows.shape, dtype=bool)
        dup[:, 1:] = rows[:, 1:] == rows[:, :-1]
        cnt = int(dup.sum())
        if cnt == 0:
            return rows
        rows[dup] = draw((cnt,))
    raise RuntimeError("could not draw distinct rows")


def _csc_from_rows(rows, vals, m):
    n, k = rows.shape
    colptr = np.arange(0, n * k + 1, k, dtype=np.int64)
    return colptr, rows.reshape(-1).astype(np.int32), vals.reshape(-1)


def _csc_matvec(colptr, rowidx, vals, x, m):
    cols = np.repeat(np.arange(len(colptr) - 1), np.diff(colptr))
    return np.bincount(rowidx, weights=vals * x[cols], minlength=m)


def _csc_rmatvec(colptr, rowidx, vals, y):
    n = len(colptr) - 1
    cols = np.repeat(np.arange(n), np.diff(colptr))
    return np.bincount(cols, weights=vals * y[rowidx], minlength=n)


def random_sparse_lp(m=2000, n=5000, k=6, seed=0, upper=10.0) -> Model:
    rng = np.random.default_rng(seed)
    k = min(k, m)
    rows = _distinct_rows(rng, m, n, k, lambda size: rng.integers(0, m, size=size))
    vals = rng.standard_normal((n, k))
    colptr, rowidx, v = _csc_from_rows(rows, vals, m)
    x0 = np.zeros(n)
    half = rng.permutation(n)[: n // 2]
    x0[half] = rng.random(len(half))
    b = _csc_matvec(colptr, rowidx, v, x0, m)
    y0 = rng.standard_normal(m)
    s = rng.random(n)
    c = _csc_rmatvec(colptr, rowidx, v, y0) + s
    return Model(m=m, n=n, colptr=colptr, rowidx=rowidx, vals=v, obj=c,
                 col_lower=np.zeros(n), col_upper=np.full(n, upper), row_lower=b.copy(),
                 row_upper=b.copy())


def transportation_lp(supplies=1000, demands=2000, seed=0) -> Model:
    rng = np.random.default_rng(seed)
    S, D = supplies, demands
    n = S * D
    m = S + D
    cost = rng.integers(1, 101, size=n).astype(np.float64)
    sup = rng.integers(500, 1501, size=S).astype(np.float64)
    dem = rng.integers(200, 801, size=D).astype(np.float64)
    dem = dem * (sup.sum() / dem.sum())
    i = np.repeat(np.arange(S, dtype=np.int64), D)
    j = np.tile(np.arange(D, dtype=np.int64), S)
    rowidx = np.empty(2 * n, dtype=np.int32)
    rowidx[0::2] = i
    rowidx[1::2] = S + j
    colptr = np.arange(0, 2 * n + 1, 2, dtype=np.int64)
    vals = np.ones(2 * n)
    rb = np.concatenate([sup, dem])
    return Model(m=m, n=n, colptr=colptr, rowidx=rowidx, vals=vals, obj=cost,
                 col_lower=np.zeros(n), col_upper=np.full(n, np.inf), row_lower=rb.copy(),
                 row_upper=rb.copy())


def power_law_lp(m=1_000_000, n=2_000_000, k=6, seed=0, exponent=1.5) -> Model:
    rng = np.random.default_rng(seed)
    perm = rng.permutation(m).astype(np.int64)

    def draw(size):
        z = rng.zipf(exponent, size=size)
        bad = z > m
        while bad.any():
            z[bad] = rng.zipf(exponent, size=int(bad.sum()))
            bad = z > m
        return perm[z - 1]

    rows = _distinct_rows(rng, m, n, k, draw)
    vals = rng.standard_normal((n, k))
    colptr, rowidx, v = _csc_from_rows(rows, vals, m)
    x0 = rng.random(n)
    ax = _csc_matvec(colptr, rowidx, v, x0, m)
    ineq = rng.random(m) < 0.3
    slack = rng.random(m)
    row_upper = ax + np.where(ineq, slack, 0.0)
    row_lower = np.where(ineq, -np.inf, ax)
    y0 = rng.standard_normal(m)
    y0 = np.where(ineq, np.abs(y0), y0)
    s = rng.random(n)
    c = _csc_rmatvec(colptr, rowidx, v, y0) + s
    return Model(m=m, n=n, colptr=colptr, rowidx=rowidx, vals=v, obj=c, col_lower=np.zeros(n),
                 col_upper=np.full(n, 5.0), row_lower=row_lower, row_upper=row_upper)


def facility_location_lp(facilities=100, customers=400, seed=0) -> Model:
    rng = np.random.default_rng(seed)
    F, C = facilities, customers
    fxy = rng.random((F, 2))
    cxy = rng.random((C, 2))
    dem = rng.integers(5, 36, size=C).astype(np.float64)
    cap = rng.uniform(2.0, 5.0, size=F) * dem.sum() / F
    fixed = rng.uniform(5000.0, 15000.0, size=F)
    dist = np.sqrt(((fxy[:, None, :] - cxy[None, :, :]) ** 2).sum(-1))  # F x C
    n = F + F * C
    m = C + F
    obj = np.concatenate([fixed, (100.0 * dist * dem[None, :]).reshape(-1)])
    # Columns: open_f (one entry, capacity row), then x_fc (demand row c, capacity row f).
    colptr = np.empty(n + 1, dtype=np.int64)
    colptr[0] = 0
    colptr[1:F + 1] = np.arange(1, F + 1)
    colptr[F + 1:] = F + 2 * np.arange(1, F * C + 1)
    rowidx = np.empty(F + 2 * F * C, dtype=np.int32)
    vals = np.empty(F + 2 * F * C)
    rowidx[:F] = C + np.arange(F)
    vals[:F] = -cap
    f = np.repeat(np.arange(F), C)
    c = np.tile(np.arange(C), F)
    rowidx[F::2] = c
    vals[F::2] = 1.0
    rowidx[F + 1::2] = C + f
    vals[F + 1::2] = dem[c]
    row_lower = np.concatenate([np.ones(C), np.full(F, -np.inf)])
    row_upper = np.concatenate([np.ones(C), np.zeros(F)])
    return Model(m=m, n=n, colptr=colptr, rowidx=rowidx, vals=vals, obj=obj,
                 col_lower=np.zeros(n), col_upper=np.ones(n), row_lower=row_lower,
                 row_upper=row_upper)


def facility_node_bounds(model: Model, facilities=100, count=256, fraction=0.05, seed=0):
    """``count`` (lower, upper) column-bound pairs: each fixes a random ``fraction`` of the open
    variables to 0 or 1, as branch-and-bound nodes do."""
    rng = np.random.default_rng(seed)
    out = []
    nfix = max(1, int(round(fraction * facilities)))
    for _ in range(count):
        lo = model.col_lower.copy()
        up = model.col_upper.copy()
        idx = rng.choice(facilities, size=nfix, replace=False)
        val = rng.integers(0, 2, size=nfix).astype(np.float64)
        lo[idx] = val
        up[idx] = val
        out.append((lo, up))
    return out


def batch_a_sizes(count=512, seed=0):
    """(m, n) of the uneven batch: m ~ U[100, 5000], n = ceil(m * U[2, 3])."""
    rng = np.random.default_rng(seed)
    ms = rng.integers(100, 5001, size=count)
    fs = rng.uniform(2.0, 3.0, size=count)
    return [(int(mm), int(math.ceil(mm * ff))) for mm, ff in zip(ms, fs)]
