"""The differentiable layer on the GPU: the unrolled PDHG and its hand-written adjoint against
the CPU oracle (oracle/unroll_oracle.py) and against central finite differences, and the
batched LP layer on 64 random sparse LPs (m = 500, n = 1200, K = 2000 unrolled iterations,
checkpoints every 64) with the envelope gradients checked against the reference dual simplex
(tests/golden/config4.npz)."""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lp(m, n, seed):
    from samaya_gb300.generators import random_sparse_lp
    from samaya_gb300.problem import make_problem
    return make_problem(random_sparse_lp(m, n, seed=seed))


def _batch(problems, inst=None):
    import samaya_gb300 as sg
    from samaya_gb300.batch import BatchSolver
    opts = sg.PdlpOptions(tol=1e-8, precision=sg.FP64, algorithm=sg.REFERENCE)
    if inst is None:
        return BatchSolver.from_problems(problems, opts)
    mats = [(p.m, p.n, p.colptr, p.rowidx, p.vals) for p in problems]
    return BatchSolver(mats, inst, opts)


def test_unroll_and_adjoint_match_the_oracle():
    """Three LPs of different sizes in one batch, K = 200 (a partial last segment after three
    of 64): v_K and the adjoint of a random linear loss agree with the oracle to 1e-9."""
    from oracle.unroll_oracle import UnrolledPdhg as Oracle
    from samaya_gb300.diff import UnrolledPdhg
    probs = [_lp(30, 70, 3)[0], _lp(45, 100, 4)[0], _lp(20, 45, 1)[0]]
    b = _batch(probs)
    un = UnrolledPdhg(b, iterations=200, checkpoint_every=64)
    v = un.forward()
    rng = np.random.default_rng(7)
    w = rng.standard_normal(v.size)
    gc, gl, gu = un.adjoint(w)
    off = 0
    for p in probs:
        nt = p.n + p.m
        o = Oracle(p.m, p.n, p.colptr, p.rowidx, p.vals)
        vo = o.forward(p.cost, p.lower, p.upper, 200)
        assert np.max(np.abs(v[off:off + nt] - vo)) <= 1e-9 * max(1.0, np.max(np.abs(vo)))
        oc, ol, ou = o.adjoint(p.cost, p.lower, p.upper, 200, w[off:off + nt])
        for got, ref in ((gc, oc), (gl, ol), (gu, ou)):
            scale = max(1.0, np.max(np.abs(ref)))
            assert np.max(np.abs(got[off:off + nt] - ref)) <= 1e-9 * scale
        off += nt
    # A second adjoint with the same seed vector is bit-identical.
    again = un.adjoint(w)
    assert all(np.array_equal(a, c) for a, c in zip((gc, gl, gu), again))
    b.close()


def _unrolled_x(lp, cost, lower, upper, K, every):
    """x_K of one LP through the GPU forward."""
    from samaya_gb300.diff import UnrolledPdhg
    b = _batch([lp], [(0, cost, lower, upper)])
    v = UnrolledPdhg(b, K, every).forward()
    b.close()
    return v[:lp.n]


def _central_difference(lp, arrs, which, j, h, K, every):
    """Central difference of 0.5 |x_K|^2 in one coordinate (which: 0 cost, 1 lower, 2 upper,
    3 both bounds = a row's b), written as ((x+ - x-) / 2h) . (x+ + x-) / 2, exact for the
    quadratic of a map that is linear on [p - h, p + h]."""
    plus = [a.copy() for a in arrs]
    minus = [a.copy() for a in arrs]
    for k in ((1, 2) if which == 3 else (which,)):
        plus[k][j] += h
        minus[k][j] -= h
    xp = _unrolled_x(lp, *plus, K, every)
    xm = _unrolled_x(lp, *minus, K, every)
    return float(np.dot((xp - xm) / (2 * h), (xp + xm) / 2))


def test_config4_layer_gradients():
    """64 LPs, m = 500, n = 1200 (nnz 7200 each), FP64; loss = sum obj* + 0.5 |x_K|^2 with x_K
    the 2000th PDHG iterate. Checks: every LP optimal at 1e-8; the unrolled part's gradient
    equals FP64 central differences (h = 1e-6) on 32 random coordinates to 1e-6 relative; the
    objective part's gradients (x* and the row duals) agree with the reference dual simplex on
    the eight LPs of the fixture."""
    torch = pytest.importorskip("torch")
    from samaya_gb300.diff import LpLayer
    B, m, n, K, every = 64, 500, 1200, 2000, 64
    built = [_lp(m, n, k) for k in range(B)]
    probs = [p for p, _ in built]
    cost = torch.tensor(np.stack([p.cost for p in probs]), requires_grad=True)
    lower = torch.tensor(np.stack([p.lower for p in probs]), requires_grad=True)
    upper = torch.tensor(np.stack([p.upper for p in probs]), requires_grad=True)
    layer = LpLayer(probs, tol=1e-8, iterations=K, checkpoint_every=every)
    obj, vstar, vk = layer(cost, lower, upper)
    loss = obj.sum() + 0.5 * (vk[:, :n] ** 2).sum()
    loss.backward()
    assert np.all(layer.last_status == 0), layer.last_status
    gc = cost.grad.numpy()
    gl = lower.grad.numpy()
    gu = upper.grad.numpy()
    # The unrolled part alone (objective gradient off).
    uc, ul, uu = layer.vjp(np.zeros(B), np.concatenate(
        [vk.detach().numpy()[:, :n], np.zeros((B, m))], axis=1))
    # Envelope part = total - unrolled part = (v*, max(d,0), min(d,0)).
    vs = vstar.numpy()
    assert np.allclose(gc - uc, vs, rtol=0, atol=1e-12 * max(1.0, np.abs(vs).max()))
    # Finite differences of the unrolled part. The map is piecewise linear with a kink wherever
    # one of its 2000 x 1700 projections changes side, so a step of 1e-6 can straddle one: a
    # coordinate counts when the central differences at h and h/2 agree (no kink within h),
    # and then must match the adjoint to 1e-6 relative; at least 32 coordinates must count.
    rng = np.random.default_rng(40)
    h = 1e-6
    bad, checked, kinks = [], 0, 0
    while checked < 32 and checked + kinks < 96:
        b = int(rng.integers(B))
        j = int(rng.integers(n + m))
        p = probs[b]
        if j < n:
            which = int(rng.integers(3))  # cost, lower, upper of a column (all finite)
        else:
            which = int(rng.choice([0, 3]))  # cost of a logical, or the row's b (both bounds)
        arrs = [p.cost.copy(), p.lower.copy(), p.upper.copy()]
        fd = _central_difference(p, arrs, which, j, h, K, every)
        fd_half = _central_difference(p, arrs, which, j, h / 2, K, every)
        if abs(fd - fd_half) > 1e-6 * max(1.0, abs(fd)):
            kinks += 1
            continue
        checked += 1
        g = {0: uc, 1: ul, 2: uu}[which][b, j] if which < 3 else ul[b, j] + uu[b, j]
        if abs(fd - g) > 1e-6 * max(1.0, abs(fd)):
            bad.append((b, j, which, fd, g))
    assert checked >= 32, (checked, kinks)
    assert not bad, bad
    # Objective part against the reference dual simplex (model space mapped to the LpProblem's:
    # x_lp = x / col_scale, dobj/db_lp = row_dual / row_scale).
    fx = np.load(os.path.join(os.path.dirname(__file__), "golden", "config4.npz"))
    for k in range(int(fx["count"][0])):
        lp, sc = built[k]
        simplex = fx[f"k{k}_simplex"]
        assert simplex[0] == 0 and simplex[3] == 1
        lp_obj = float(obj[k].detach())
        ref_obj = float(simplex[1]) - _lp_offset(k)
        assert abs(lp_obj - ref_obj) <= 1e-6 * (1 + abs(ref_obj)), (k, lp_obj, ref_obj)
        x_lp = fx[f"k{k}_x"] / sc.col
        assert np.max(np.abs(vs[k, :n] - x_lp)) <= 1e-3 * (1 + np.max(np.abs(x_lp)))
        # dobj/db: the row duals. Where the optimal duals are not unique (a degenerate vertex)
        # the two solvers may return different valid duals, so 99% of rows must agree.
        db = (gl - ul)[k, n:] + (gu - uu)[k, n:]
        ref_db = fx[f"k{k}_y"] / sc.row
        agree = np.abs(db - ref_db) <= 1e-4 * (1 + np.abs(ref_db))
        assert agree.mean() >= 0.99, (k, agree.mean())
    layer.close()


def _lp_offset(k):
    from samaya_gb300.generators import random_sparse_lp
    return random_sparse_lp(500, 1200, seed=k).obj_offset
