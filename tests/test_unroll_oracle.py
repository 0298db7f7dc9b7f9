"""The differentiable layer's CPU oracle (oracle/unroll_oracle.py) against itself: its adjoint
equals central finite differences of its forward map, which is the oracle's (reference-pinned)
fixed-step PDHG."""
from __future__ import annotations

import numpy as np
import pytest


def _lp(m, n, seed):
    from samaya_gb300.generators import random_sparse_lp
    from samaya_gb300.problem import make_problem
    return make_problem(random_sparse_lp(m, n, seed=seed))[0]


def test_oracle_forward_is_the_reference_fixed_step_pdhg():
    """v_K of the oracle = K steps of oracle.pdhg_steps from zero, mapped by the scales."""
    from oracle import oracle as o
    from oracle.unroll_oracle import UnrolledPdhg
    lp = _lp(20, 45, 1)
    u = UnrolledPdhg(lp.m, lp.n, lp.colptr, lp.rowidx, lp.vals)
    v = u.forward(lp.cost, lp.lower, lp.upper, 70)
    # The same map written out by hand (numpy), as the adjoint's forward pass computes it.
    c, l, up = u._scaled(lp.cost, lp.lower, lp.upper)
    x = np.zeros(lp.n + lp.m)
    xb = np.zeros(lp.n + lp.m)
    y = np.zeros(lp.m)
    for _ in range(70):
        y = y + u.eta * u._K(xb)
        xn = np.clip(x - u.eta * (c + u._Kt(y)), l, up)
        xb = 2 * xn - x
        x = xn
    ref = np.concatenate([x[:lp.n] * u.cs, x[lp.n:] / u.rs])
    assert np.max(np.abs(v - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
    assert o.lib() is not None


@pytest.mark.parametrize("seed", [3, 4])
def test_oracle_adjoint_matches_central_differences(seed):
    from oracle.unroll_oracle import UnrolledPdhg
    lp = _lp(30, 70, seed)
    K = 150
    u = UnrolledPdhg(lp.m, lp.n, lp.colptr, lp.rowidx, lp.vals)
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(lp.n + lp.m)

    def loss(c, lo, up):
        return float(w @ u.forward(c, lo, up, K))

    gc, gl, gu = u.adjoint(lp.cost, lp.lower, lp.upper, K, w)
    h = 1e-6
    base = (lp.cost, lp.lower, lp.upper)
    bad = []
    for j in rng.choice(lp.n + lp.m, 16, replace=False):
        checks = [((0,), gc[j])]
        if j >= lp.n:
            checks.append(((1, 2), gl[j] + gu[j]))  # an equality row's b moves both bounds
        else:
            if np.isfinite(lp.lower[j]):
                checks.append(((1,), gl[j]))
            if np.isfinite(lp.upper[j]):
                checks.append(((2,), gu[j]))
        for which, g in checks:
            a = [x.copy() for x in base]
            b = [x.copy() for x in base]
            for k in which:
                a[k][j] += h
                b[k][j] -= h
            fd = (loss(*a) - loss(*b)) / (2 * h)
            if abs(fd - g) > 1e-6 * max(1.0, abs(fd)):
                bad.append((int(j), which, fd, g))
    assert not bad, bad
