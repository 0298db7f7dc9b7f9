"""Row groups in the dual steps: runs of up to 32 consecutive rows whose k-th nonzeros lie in
neighbouring columns (the demand rows of a transportation LP) are staged through shared memory
so that one gather reads neighbouring entries (kind-3 tiles). Checked at step level against
the oracle (the same tolerances as the other step kernels, through the seam, which runs the
solves' dual tiles) and at solve level against the solve without groups (the rows are summed in
another order, so the two agree to the tolerance, not bit for bit)."""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_steps import _check32, _check64, _equilibrated, _f32, _start, _steps

pytestmark = pytest.mark.gpu


def _transport(supplies, demands, seed):
    from samaya_gb300 import generators as g
    from samaya_gb300.problem import make_problem
    return make_problem(g.transportation_lp(supplies, demands, seed=seed))[0]


@pytest.mark.parametrize("precision", [0, 2])
def test_group_halpern_steps_match_the_oracle(engine, oracle, precision):
    """Eight reflected Halpern iterations with the demand rows (150 and 700 nonzeros) in row
    groups, from a random point and anchor, against orc_halpern_steps."""
    rng = np.random.default_rng(951 + precision)
    check = _check64 if precision == 0 else _check32
    for lp in (_transport(150, 70, 3), _transport(700, 45, 4)):
        e = _equilibrated(lp, rng)
        v, y, v0, y0 = _start(rng, e)
        tau, sigma = _steps(e)
        opts = engine.PdlpOptions(precision=precision, autotune=False, row_groups=1)
        dev = engine.PdhgDevice(e["m"], e["n"], e["colptr"], e["rowidx"], e["vals"], e["cost"],
                                e["lower"], e["upper"], options=opts)
        rows, tiles, groups, _ = dev.step_rows()
        assert rows == lp.m and groups >= 2
        dev.set_original(e["cs"], e["rs"], lp.cost, lp.lower, lp.upper)
        dev.set_state(v, y, v0, y0, precision=0 if precision == 0 else 1)
        for s in range(8):
            dev.halpern_step(tau, sigma, 5 + s)
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
                                    5, v, y, v0, y0)
        check(got["v"], want["v"])
        check(got["y"], want["y"])
        check(got["v_erg"], want["v_hat"])
        check(got["y_erg"], want["y_hat"])


def test_group_classic_fp64_steps_match_the_oracle(engine, oracle):
    """The classic fused FP64 steps (dual_step_kernel) with row groups."""
    rng = np.random.default_rng(961)
    lp = _transport(300, 64, 5)
    e = _equilibrated(lp, rng)
    v, y, _, _ = _start(rng, e)
    tau, sigma = _steps(e)
    opts = engine.PdlpOptions(precision=0, autotune=False, row_groups=1)
    dev = engine.PdhgDevice(e["m"], e["n"], e["colptr"], e["rowidx"], e["vals"], e["cost"],
                            e["lower"], e["upper"], options=opts)
    assert dev.step_rows()[2] >= 2
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
def test_solves_with_and_without_row_groups_agree(engine, precision):
    """A 400 x 300 transportation LP to 1e-8 with the demand rows grouped and without: both
    optimal, objectives within 1e-8 relative; re-running the grouped solve repeats its bits."""
    lp = _transport(400, 300, 6)
    out = {}
    for groups in (1, -1, 1):
        opts = engine.PdlpOptions(tol=1e-8, precision=getattr(engine, precision),
                                  algorithm=engine.HALPERN, inner_tol=1e-6, autotune=False,
                                  row_groups=groups)
        with engine.PdlpSolver(lp, opts) as s:
            g = s.step_rows()[2]
            assert (g > 0) == (groups == 1)
            r = s.solve()
        if groups in out:
            a = out[groups]
            assert a.iterations == r.iterations
            assert np.array_equal(a.x, r.x) and np.array_equal(a.y, r.y)
        out[groups] = r
    a, b = out[1], out[-1]
    assert a.status == b.status == engine.OPTIMAL
    assert abs(a.primal_objective - b.primal_objective) <= 1e-8 * (1 + abs(b.primal_objective))
