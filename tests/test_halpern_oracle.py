"""The oracle's reflected Halpern PDHG (``orc_halpern_steps``, the engine's Halpern variant
restated from its publication; no reference counterpart) checked on the CPU: against a dense
numpy statement of the same map, and by convergence to the optimum of the reference's pinned
PDLP on small LPs."""
from __future__ import annotations

import numpy as np

from conftest import load_group


def _dense(lp):
    a = np.zeros((lp.m, lp.n))
    cols = np.repeat(np.arange(lp.n), np.diff(lp.colptr))
    np.add.at(a, (lp.rowidx, cols), lp.vals)
    return np.hstack([a, -np.eye(lp.m)])  # K = [A -I]


def _numpy_halpern(K, c, lo, up, tau, sigma, steps, k, v, y, v0, y0):
    for _ in range(steps):
        vh = np.clip(v - tau * (c + K.T @ y), lo, up)
        refl = 2.0 * vh - v
        yh = y + sigma * (K @ refl)
        w = 1.0 / (k + 2)
        ry = 2.0 * yh - y
        v = refl + w * (v0 - refl)
        y = ry + w * (y0 - ry)
        k += 1
    return v, y, vh, yh


def _rel(a, b):
    if b.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


def test_halpern_oracle_matches_a_dense_restatement(oracle):
    rng = np.random.default_rng(31)
    for case in load_group("feasible8")[:6] + load_group("basic")[:4]:
        lp = case.lp
        K = _dense(lp)
        nt = lp.n + lp.m
        v = rng.uniform(-1, 1, nt)
        y = rng.uniform(-1, 1, lp.m)
        v0 = rng.uniform(-1, 1, nt)
        y0 = rng.uniform(-1, 1, lp.m)
        got = oracle.halpern_steps(lp.m, lp.n, lp.colptr, lp.rowidx, lp.vals, lp.cost, lp.lower,
                                   lp.upper, 0.2, 0.3, 7, 3, v, y, v0, y0)
        want = _numpy_halpern(K, lp.cost, lp.lower, lp.upper, 0.2, 0.3, 7, 3, v, y, v0, y0)
        for a, b in zip((got["v"], got["y"], got["v_hat"], got["y_hat"]), want):
            assert _rel(a, b) < 1e-12


def test_restarted_halpern_oracle_reaches_the_pinned_pdlp_optimum(oracle):
    """Halpern iterations restarted every 256 steps at T(z) converge to the objective of the
    reference's CPU PDLP (the pinned oracle) on small feasible LPs."""
    checked = 0
    for case in load_group("feasible8")[:4]:
        lp = case.lp
        if case.ref_status != oracle.OPTIMAL:
            continue
        K = _dense(lp)
        eta = 0.95 / np.linalg.norm(K, 2)
        nt = lp.n + lp.m
        v, y = np.zeros(nt), np.zeros(lp.m)
        ref = oracle.pdlp_solve(*lp.arrays(), tol=1e-9)
        ref_obj = float(lp.cost @ ref.x)
        obj = None
        for _ in range(400):
            st = oracle.halpern_steps(lp.m, lp.n, lp.colptr, lp.rowidx, lp.vals, lp.cost,
                                      lp.lower, lp.upper, eta, eta, 256, 0, v, y, v, y)
            v, y = st["v_hat"], st["y_hat"]  # restart at T(z)
            obj = float(lp.cost @ v)
            res = np.abs(K @ v).max()
            if abs(obj - ref_obj) <= 1e-7 * (1 + abs(ref_obj)) and res < 1e-7:
                break
        assert abs(obj - ref_obj) <= 1e-6 * (1 + abs(ref_obj)), (case.k, obj, ref_obj)
        checked += 1
    assert checked >= 3
