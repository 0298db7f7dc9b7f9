"""Step-level parity of every step kernel the solves run, against the oracle, through the C
ABI's inner seam: the classic fused PDHG steps (pdlp.cpp:574-641) and the reflected Halpern
steps (the engine's Halpern variant; the oracle restates the published method), each in FP64
and in FP32 storage, and the FP32 evaluation kernels against the oracle's seven sums.

Step sizes are tau = 0.7 / L, sigma = 0.9 / L with L an estimate of ||[A -I]||, as a solve
takes them (the iterates stay bounded). Tolerances, per entry against the vector's scale
(1 + max |oracle|; rows of thousands of nonzeros are summed in another order on the device):
FP64 kernels 1e-12; FP32 kernels, whose inputs are the FP64 data rounded to FP32 (the oracle
gets the same rounded data and runs in FP64), 1e-5 after 8 steps; FP32 evaluation sums 1e-5 of
(1 + |sum| + the sum of the absolute values of its terms)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_group

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5


def _f32(a):
    return np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)


def _problems():
    """Small LPs of the parity fixtures, a small transportation LP (shared column bounds
    x >= 0: the primal steps read no bound vectors) and a small power-law LP (rows split into
    segments and medium rows on warps)."""
    from samaya_gb300 import generators as g
    from samaya_gb300.problem import make_problem
    out = [c.lp for c in load_group("feasible8")[:6]]
    out += [c.lp for c in load_group("repeatable30")[:4]]
    out.append(make_problem(g.transportation_lp(20, 45, seed=3))[0])
    out.append(make_problem(g.power_law_lp(m=3000, n=20000, seed=5))[0])
    return out


def _equilibrated(lp, rng):
    """The LP with a random equilibration applied (rows rs, columns cs), as solve_pdlp applies
    Ruiz before the iterations."""
    m, n = lp.m, lp.n
    rs = rng.uniform(0.5, 2.0, size=m)
    cs = rng.uniform(0.5, 2.0, size=n)
    cols = np.repeat(np.arange(n), np.diff(lp.colptr))
    vals = rs[lp.rowidx] * lp.vals * cs[cols]
    cost, lower, upper = lp.cost.copy(), lp.lower.copy(), lp.upper.copy()
    cost[:n] *= cs
    lower[:n] /= cs
    upper[:n] /= cs
    cost[n:] *= rs
    lower[n:] *= rs
    upper[n:] *= rs
    return dict(m=m, n=n, colptr=lp.colptr, rowidx=lp.rowidx, vals=vals, cost=cost,
                lower=lower, upper=upper, rs=rs, cs=cs)


def _device(engine, e, precision):
    opts = engine.PdlpOptions(precision=precision, autotune=False)
    return engine.PdhgDevice(e["m"], e["n"], e["colptr"], e["rowidx"], e["vals"], e["cost"],
                             e["lower"], e["upper"], options=opts)


def _start(rng, e):
    nt = e["n"] + e["m"]
    # A random point inside and outside the bounds, and a random anchor.
    return (rng.uniform(-2, 2, nt), rng.uniform(-2, 2, e["m"]), rng.uniform(-2, 2, nt),
            rng.uniform(-2, 2, e["m"]))


def _steps(e):
    """(tau, sigma) = (0.7, 0.9) / L, L = 1.05 x a power-iteration estimate of ||[A -I]||."""
    n, m = e["n"], e["m"]
    cols = np.repeat(np.arange(n), np.diff(e["colptr"]))
    rows = e["rowidx"]
    u = np.random.default_rng(1).standard_normal(n + m)
    L = 1.0
    for _ in range(30):
        ku = np.bincount(rows, weights=e["vals"] * u[cols], minlength=m) - u[n:]
        w = np.concatenate([np.bincount(cols, weights=e["vals"] * ku[rows], minlength=n), -ku])
        L = np.sqrt(np.linalg.norm(w) / max(np.linalg.norm(u), 1e-300))
        u = w / max(np.linalg.norm(w), 1e-300)
    L *= 1.05
    return 0.7 / L, 0.9 / L


def _check64(a, b):
    if b.size:
        assert np.max(np.abs(a - b)) <= FP64_TOL * (1.0 + np.max(np.abs(b)))


def _check32(a, b):
    if b.size:
        assert np.max(np.abs(a - b)) <= FP32_TOL * (1.0 + np.max(np.abs(b)))


MODES = [("fp64", 0), ("fp32_switch", 2), ("fp32_refined", 1)]


@pytest.mark.parametrize("name,precision", MODES)
def test_halpern_steps_match_the_oracle(engine, oracle, name, precision):
    """Eight reflected Halpern iterations (halpern_primal_kernel, then halpern_dual_kernel)
    from a random point and anchor: the iterate and T(z) against orc_halpern_steps."""
    rng = np.random.default_rng(901 + precision)
    check = _check64 if precision == 0 else _check32
    for lp in _problems():
        e = _equilibrated(lp, rng)
        v, y, v0, y0 = _start(rng, e)
        tau, sigma = _steps(e)
        k0 = 5
        dev = _device(engine, e, precision)
        dev.set_original(e["cs"], e["rs"], lp.cost, lp.lower, lp.upper)
        dev.set_state(v, y, v0, y0, precision=0 if precision == 0 else 1)
        for s in range(8):
            dev.halpern_step(tau, sigma, k0 + s)
            dev.advance()
        got = dev.download()
        dev.close()
        data = {k: e[k] for k in ("vals", "cost", "lower", "upper")}
        if precision != 0:
            data = {k: _f32(a) for k, a in data.items()}
            v, y, v0, y0 = _f32(v), _f32(y), _f32(v0), _f32(y0)
            tau, sigma = float(np.float32(tau)), float(np.float32(sigma))
        want = oracle.halpern_steps(e["m"], e["n"], e["colptr"], e["rowidx"], data["vals"],
                                    data["cost"], data["lower"], data["upper"], tau, sigma, 8,
                                    k0, v, y, v0, y0)
        check(got["v"], want["v"])
        check(got["y"], want["y"])
        check(got["v_erg"], want["v_hat"])
        check(got["y_erg"], want["y_hat"])


@pytest.mark.parametrize("name,precision", MODES[1:])
def test_fp32_classic_steps_match_the_oracle(engine, oracle, name, precision):
    """Eight classic fused steps (dual_step_kernel, primal_step_kernel) in FP32 storage and
    arithmetic against the oracle's FP64 steps on the FP32-rounded problem."""
    rng = np.random.default_rng(911 + precision)
    for lp in _problems():
        e = _equilibrated(lp, rng)
        v, y, _, _ = _start(rng, e)
        tau, sigma = _steps(e)
        dev = _device(engine, e, precision)
        dev.set_original(e["cs"], e["rs"], lp.cost, lp.lower, lp.upper)
        dev.set_state(v, y, v, y, precision=1)
        for it in range(8):
            dev.step(tau, sigma, 1.0, it)
            dev.advance()
        got = dev.download()
        dev.close()
        data = {k: _f32(e[k]) for k in ("vals", "cost", "lower", "upper")}
        v, y = _f32(v), _f32(y)
        state = dict(v=v.copy(), v_prev=v.copy(), y=y.copy(), v_erg=np.zeros_like(v),
                     y_erg=np.zeros_like(y))
        st = oracle.pdhg_steps(e["m"], e["n"], e["colptr"], e["rowidx"], data["vals"],
                               data["cost"], data["lower"], data["upper"],
                               float(np.float32(tau)), float(np.float32(sigma)), 8, 0, state)
        for a, b in ((got["v"], st["v"]), (got["y"], st["y"]), (got["v_erg"], st["v_erg"]),
                     (got["y_erg"], st["y_erg"])):
            _check32(a, b)


def test_fp64_classic_steps_from_a_set_state_match_the_oracle(engine, oracle):
    """The classic FP64 steps from a random point (not zero) on every problem, including the
    split and medium rows of the power-law LP."""
    rng = np.random.default_rng(921)
    for lp in _problems():
        e = _equilibrated(lp, rng)
        v, y, _, _ = _start(rng, e)
        tau, sigma = _steps(e)
        dev = _device(engine, e, 0)
        dev.set_original(e["cs"], e["rs"], lp.cost, lp.lower, lp.upper)
        dev.set_state(v, y, v, y)
        for it in range(8):
            dev.step(tau, sigma, 1.0, it)
            dev.advance()
        got = dev.download()
        dev.close()
        state = dict(v=v.copy(), v_prev=v.copy(), y=y.copy(), v_erg=np.zeros_like(v),
                     y_erg=np.zeros_like(y))
        st = oracle.pdhg_steps(e["m"], e["n"], e["colptr"], e["rowidx"], e["vals"], e["cost"],
                               e["lower"], e["upper"], tau, sigma, 8, 0, state)
        for a, b in ((got["v"], st["v"]), (got["y"], st["y"]), (got["v_erg"], st["v_erg"]),
                     (got["y_erg"], st["y_erg"])):
            _check64(a, b)


def _sum_magnitudes(e, v, y):
    """Sums of the absolute values of the terms of the objective sums (primal c'v and the
    dual's bound terms), the scale of their rounding error."""
    n, m = e["n"], e["m"]
    cols = np.repeat(np.arange(n), np.diff(e["colptr"]))
    aty = np.bincount(cols, weights=e["vals"] * y[e["rowidx"]], minlength=n)
    g = np.concatenate([e["cost"][:n] + aty, e["cost"][n:] - y])
    lo, up = e["lower"], e["upper"]
    hl, hu = np.isfinite(lo), np.isfinite(up)
    lam = np.where(hl & hu, g, np.where(hl, np.maximum(g, 0), np.where(hu, np.minimum(g, 0), 0)))
    bound = np.where(lam > 0, np.where(hl, lo, 0.0), np.where(lam < 0, np.where(hu, up, 0.0), 0.0))
    mags = np.zeros(7)
    mags[2] = np.sum(np.abs(e["cost"] * v))
    mags[3] = np.sum(np.abs(lam * bound))
    return mags


@pytest.mark.parametrize("precision", [2, 1])
def test_fp32_evaluation_matches_the_oracle_sums(engine, oracle, precision):
    """eval_rows32_kernel + eval_cols32_kernel (the FP32 solves' evaluation, in the given
    problem's own space): the seven sums of the current and the average iterate against the
    oracle's FP64 sums of the same FP32 vectors on the FP32-rounded problem (unit scales)."""
    rng = np.random.default_rng(931 + precision)
    compared = 0
    for lp in _problems():
        e = _equilibrated(lp, rng)
        v, y, _, _ = _start(rng, e)
        dev = _device(engine, e, precision)
        dev.set_original(e["cs"], e["rs"], lp.cost, lp.lower, lp.upper)
        dev.set_state(v, y, v, y, precision=1)
        tau, sigma = _steps(e)
        for it in range(3):
            dev.step(tau, sigma, 1.0, it)
            dev.advance()
        dev.step(tau, sigma, 1.0, 3)
        st = dev.download()
        data = {k: _f32(e[k]) for k in ("vals", "cost", "lower", "upper")}
        d = dict(e, **data)
        ones_n, ones_m = np.ones(e["n"]), np.ones(e["m"])
        for which, (vv, yy) in ((0, (st["v_new"], st["y_new"])), (1, (st["v_erg"], st["y_erg"]))):
            s = dev.evaluate(which)
            host = oracle.eval_sums(e["m"], e["n"], e["colptr"], e["rowidx"], data["vals"],
                                    data["cost"], data["lower"], data["upper"], ones_n, ones_m,
                                    vv, yy)
            tol = FP32_TOL * (1.0 + np.abs(host) + _sum_magnitudes(d, vv, yy))
            assert np.all(np.abs(s - host) <= tol), (which, s, host)
            compared += 1
        dev.close()
    assert compared == 2 * len(_problems())
