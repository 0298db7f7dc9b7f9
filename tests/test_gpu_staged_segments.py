"""Staged long-row segments in the dual steps: the segments of rows longer than a tile are
streamed into shared memory by bulk copies (two chunks of 2,048 nonzeros in flight, completing
on mbarriers) instead of being loaded by the threads. Checked at step level against the oracle
(through the seam, which runs the solves' dual tiles when no inert rows are left out) and at
solve level against the same solve with the segments loaded directly (the nonzeros are summed
in another order, so the two agree to the tolerance)."""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_steps import _check32, _check64, _equilibrated, _f32, _start, _steps

pytestmark = pytest.mark.gpu


def _powerlaw(m, n, seed):
    from samaya_gb300 import generators as g
    from samaya_gb300.problem import make_problem
    return make_problem(g.power_law_lp(m=m, n=n, seed=seed))[0]


def _opts(engine, precision, staging):
    # 8192 nonzeros per tile: the longest rows (about 20,000 nonzeros) split into segments of
    # four chunks, with unaligned starts and ends.
    return engine.PdlpOptions(precision=precision, autotune=False, keep_inert_rows=True,
                              segment_staging=staging, tile_nnz=8192)


@pytest.mark.parametrize("precision", [0, 2])
def test_staged_halpern_steps_match_the_oracle(engine, oracle, precision):
    """Eight reflected Halpern iterations with staged segments from a random point and anchor,
    against orc_halpern_steps (FP64 1e-12, FP32 storage 1e-5)."""
    rng = np.random.default_rng(971 + precision)
    check = _check64 if precision == 0 else _check32
    lp = _powerlaw(3000, 20000, 5)
    e = _equilibrated(lp, rng)
    v, y, v0, y0 = _start(rng, e)
    tau, sigma = _steps(e)
    dev = engine.PdhgDevice(e["m"], e["n"], e["colptr"], e["rowidx"], e["vals"], e["cost"],
                            e["lower"], e["upper"], options=_opts(engine, precision, 1))
    rows, tiles, groups, staged = dev.step_rows()
    assert rows == lp.m and staged == 1
    dev.set_original(e["cs"], e["rs"], lp.cost, lp.lower, lp.upper)
    dev.set_state(v, y, v0, y0, precision=0 if precision == 0 else 1)
    for s in range(8):
        dev.halpern_step(tau, sigma, 3 + s)
        dev.advance()
    got = dev.download()
    dev.close()
    data = {k: e[k] for k in ("vals", "cost", "lower", "upper")}
    if precision != 0:
        data = {k: _f32(a) for k, a in data.items()}
        v, y, v0, y0 = _f32(v), _f32(y), _f32(v0), _f32(y0)
        tau, sigma = float(np.float32(tau)), float(np.float32(sigma))
    want = oracle.halpern_steps(e["m"], e["n"], e["colptr"], e["rowidx"], data["vals"],
                                data["cost"], data["lower"], data["upper"], tau, sigma, 8, 3,
                                v, y, v0, y0)
    check(got["v"], want["v"])
    check(got["y"], want["y"])
    check(got["v_erg"], want["v_hat"])
    check(got["y_erg"], want["y_hat"])


def test_staged_classic_fp64_steps_match_the_oracle(engine, oracle):
    """The classic fused FP64 steps (dual_step_kernel) with staged segments."""
    rng = np.random.default_rng(981)
    lp = _powerlaw(3000, 20000, 6)
    e = _equilibrated(lp, rng)
    v, y, _, _ = _start(rng, e)
    tau, sigma = _steps(e)
    dev = engine.PdhgDevice(e["m"], e["n"], e["colptr"], e["rowidx"], e["vals"], e["cost"],
                            e["lower"], e["upper"], options=_opts(engine, 0, 1))
    assert dev.step_rows()[3] == 1
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


@pytest.mark.parametrize("precision", ["FP64", "FP32_THEN_FP64"])
def test_solves_with_and_without_staging_agree(engine, precision):
    """A 20,000 x 40,000 power-law LP to 1e-6 (Halpern) with staged segments and without: both
    optimal with objectives within 1e-5 relative (each meets the 1e-6 relative gap test, which
    lets either objective move by about 1e-6 of the objectives' sum); a re-run of the staged
    solve repeats its bits."""
    lp = _powerlaw(20000, 40000, 2)
    out = {}
    for staging in (1, 0, 1):
        opts = engine.PdlpOptions(tol=1e-6, precision=getattr(engine, precision),
                                  algorithm=engine.HALPERN, inner_tol=1e-5, autotune=False,
                                  segment_staging=staging, tile_nnz=8192)
        with engine.PdlpSolver(lp, opts) as s:
            assert s.step_rows()[3] == (1 if staging == 1 else 0)
            r = s.solve()
        if staging in out:
            a = out[staging]
            assert a.iterations == r.iterations
            assert np.array_equal(a.x, r.x) and np.array_equal(a.y, r.y)
        out[staging] = r
    a, b = out[1], out[0]
    assert a.status == b.status == engine.OPTIMAL
    assert abs(a.primal_objective - b.primal_objective) <= 1e-5 * (1 + abs(b.primal_objective))
