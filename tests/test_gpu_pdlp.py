"""End-to-end parity of the GPU PDLP engine with the reference's CPU PDLP (golden fixtures made
from the reference's own code) and with its simplex oracles — the counterparts of the
reference's tests/test_pdlp.cpp and tests/test_gpu.cpp solve tests."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_group

pytestmark = pytest.mark.gpu


def model_objective(case, x):
    """Objective in the model's space of a PDLP answer x (LpProblem space): x_model = x * col
    scale, obj = offset + c'x (tests/test_pdlp.cpp:105-127)."""
    m = case.model
    xm = x[:m.n] * case.col_scale
    return m.obj_offset + float(np.dot(m.obj, xm))


def solve(engine, case, **kw):
    opts = engine.PdlpOptions(tol=case.tol, max_iterations=case.max_iter, **kw)
    return engine.solve_pdlp(case.lp, opts)


def test_basic_box_lp(engine):
    """pdlp_basic (tests/test_pdlp.cpp:54-83): min x, 1 <= x <= 2, no rows."""
    case = load_group("basic")[0]
    r = solve(engine, case)
    assert r.status == engine.OPTIMAL
    assert r.iterations > 0
    assert r.primal_residual < case.tol and r.dual_residual < case.tol and r.gap < case.tol
    assert abs(r.x[0] - 1.0) < 1e-4


def test_random_feasible_objectives_and_iterations(engine):
    """pdlp_random_feasible (tests/test_pdlp.cpp:85-232): 50 LPs at 1e-8; every optimum's
    objective within 1e-6 (1 + |ref|) of the dense reference simplex, statuses agree with the
    reference's CPU PDLP, and the mean iteration count stays at most 1500."""
    optimal, iters, mismatches = 0, 0, []
    for case in load_group("feasible8"):
        r = solve(engine, case)
        if r.status != case.ref_status:
            mismatches.append((case.k, r.status, case.ref_status))
            continue
        if r.status == engine.OPTIMAL:
            st, ref_obj = case.refnlp
            assert int(st) == 0
            obj = model_objective(case, r.x)
            if abs(obj - ref_obj) > 1e-6 * (1 + abs(ref_obj)):
                mismatches.append((case.k, obj, ref_obj))
            optimal += 1
            iters += r.iterations
    assert not mismatches, mismatches
    assert optimal > 10
    assert iters / optimal <= 1500


def test_against_reference_cpu_pdlp_at_1e4(engine):
    """pdlp_vs_simplex (tests/test_pdlp.cpp:234-400) LPs at 1e-4: same status as the reference's
    CPU PDLP and optimal objectives within 1e-4 relative of its objective. (At 1e-4 the
    reference's own PDLP stops on two of these LPs with objectives far from the simplex optimum,
    so agreement with the simplex is required only where the reference's PDLP has it.)"""
    bad = []
    for case in load_group("vs_simplex10"):
        r = solve(engine, case)
        if r.status != case.ref_status:
            bad.append(("status", case.k, r.status, case.ref_status))
            continue
        if r.status != engine.OPTIMAL:
            continue
        obj = model_objective(case, r.x)
        ref_obj = model_objective(case, case.ref_x)
        if abs(obj - ref_obj) > 1e-4 * (1 + abs(ref_obj)):
            bad.append(("vs reference pdlp", case.k, obj, ref_obj))
        if case.simplex is not None and int(case.simplex[0]) == 0:
            sx = float(case.simplex[1])
            ref_close = abs(ref_obj - sx) <= 1e-3 * (1 + abs(sx))
            if ref_close and abs(obj - sx) > 1e-3 * (1 + abs(sx)):
                bad.append(("vs simplex", case.k, obj, sx))
    assert not bad, bad


def test_gpu_matches_cpu_solutions(engine):
    """gpu_pdlp_vs_cpu (tests/test_gpu.cpp:407-477): at 1e-6 the GPU answer's x matches the CPU
    PDLP's x within 1e-4 relative on every LP both solve."""
    passed = total = 0
    for case in load_group("gpu_vs_cpu6"):
        if case.refnlp is None or int(case.refnlp[0]) != 0:
            continue
        total += 1
        r = solve(engine, case)
        if r.status == case.ref_status == engine.OPTIMAL:
            n = case.lp.n
            rel = np.abs(r.x[:n] - case.ref_x[:n]) / np.maximum(
                1.0, np.maximum(np.abs(r.x[:n]), np.abs(case.ref_x[:n])))
            passed += int(rel.max() <= 1e-4)
        elif r.status == case.ref_status:
            passed += 1
    assert total > 0 and passed == total


def test_runs_are_bit_repeatable(engine):
    """gpu_pdlp_runs_are_repeatable (tests/test_gpu.cpp:675-697): two solves give the same
    iteration count and bit-identical x, y."""
    for case in load_group("repeatable30"):
        with engine.PdlpSolver(case.lp, engine.PdlpOptions(tol=case.tol,
                                                           max_iterations=case.max_iter)) as s:
            a = s.solve()
            b = s.solve()
        c = solve(engine, case)
        assert a.status == b.status == c.status
        assert a.iterations == b.iterations == c.iterations
        assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)
        assert np.array_equal(a.x, c.x) and np.array_equal(a.y, c.y)


def test_infeasible_and_unbounded_detection(engine):
    """pdlp_infeasible_unbounded (tests/test_pdlp.cpp:402-478): the device-side Farkas and ray
    checks detect the certificates the reference's CPU PDLP detects."""
    detected = {1: 0, 2: 0}
    agree = total = 0
    for group, status in (("infeasible8", 1), ("loose8", 2)):
        for case in load_group(group):
            if case.refnlp is None or int(case.refnlp[0]) != status:
                continue
            r = solve(engine, case)
            total += 1
            agree += int(r.status == case.ref_status)
            if r.status == status:
                detected[status] += 1
                if status == 1:
                    assert r.dual_ray.shape == (case.lp.m,)
                else:
                    assert r.primal_ray.shape == (case.lp.n,)
    assert detected[1] > 0 and detected[2] > 0
    assert agree >= int(0.8 * total)


def test_random_sparse_lp_objective_vs_dual_simplex(engine):
    """The 200 x 500 random sparse LPs at 1e-4: objective within 1e-4 relative of the reference
    dual simplex (the bar for the plain FP64 path at 1e-4)."""
    for case in load_group("config0_small"):
        r = solve(engine, case)
        assert r.status == engine.OPTIMAL
        ref_obj = float(case.simplex[1])
        obj = model_objective(case, r.x)
        assert abs(obj - ref_obj) <= 1e-4 * (1 + abs(ref_obj)), (obj, ref_obj)


@pytest.mark.parametrize("precision,algorithm", [("FP32_REFINED", "ENHANCED"),
                                                  ("FP32_THEN_FP64", "ENHANCED"),
                                                  ("FP64", "HALPERN"),
                                                  ("FP32_THEN_FP64", "HALPERN")])
def test_mixed_precision_reaches_fp64_tolerance(engine, precision, algorithm):
    """The FP32 paths (refinement; FP32 phase then FP64 phase) and the reflected Halpern
    iteration on the 200 x 500 random sparse LPs at 1e-8: the FP64 relative KKT of the answer
    meets 1e-8, the answer lies within its bounds, and the objective agrees with the reference
    dual simplex to 1e-6 relative."""
    for case in load_group("config0_small"):
        opts = engine.PdlpOptions(tol=1e-8, precision=getattr(engine, precision),
                                  algorithm=getattr(engine, algorithm))
        r = engine.solve_pdlp(case.lp, opts)
        assert r.status == engine.OPTIMAL, (precision, r.status_name, r.iterations)
        assert max(r.primal_residual, r.dual_residual, abs(r.gap)) < 1e-8
        slack = 1e-9 * (1.0 + np.abs(r.x))  # the unscaling's round-off
        assert np.all(r.x >= case.lp.lower - slack) and np.all(r.x <= case.lp.upper + slack)
        ref_obj = float(case.simplex[1])
        obj = model_objective(case, r.x)
        assert abs(obj - ref_obj) <= 1e-6 * (1 + abs(ref_obj)), (obj, ref_obj)


def test_transport_mixed_precision_matches_fp64():
    """A 100 x 200 transportation LP at 1e-8: both FP32 paths and the Halpern iteration (FP64
    and FP32 then FP64) reach the FP64 path's objective to 1e-7 relative, and repeated runs of
    each are bit-identical."""
    import samaya_gb300 as sg
    from samaya_gb300.generators import transportation_lp
    from samaya_gb300.problem import make_problem
    lp, _ = make_problem(transportation_lp(100, 200, seed=3))
    base = sg.PdlpOptions(tol=1e-8, algorithm=sg.ENHANCED)
    r64 = sg.solve_pdlp(lp, base)
    assert r64.status == sg.OPTIMAL
    o64 = float(np.dot(lp.cost, r64.x))
    for prec, alg in ((sg.FP32_REFINED, sg.ENHANCED), (sg.FP32_THEN_FP64, sg.ENHANCED),
                      (sg.FP64, sg.HALPERN), (sg.FP32_THEN_FP64, sg.HALPERN)):
        opts = sg.PdlpOptions(tol=1e-8, algorithm=alg, precision=prec)
        a = sg.solve_pdlp(lp, opts)
        b = sg.solve_pdlp(lp, opts)
        assert a.status == sg.OPTIMAL, (prec, a.status_name)
        assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)
        o = float(np.dot(lp.cost, a.x))
        assert abs(o - o64) <= 1e-7 * (1 + abs(o64)), (prec, o, o64)


def _verify(engine, case_model, scaling, r):
    """The reference's verify_lp_optimality (oracle restatement) of a GPU answer, mapped to the
    model's space as samaya's solve_pdlp_lp maps it (src/core/solver.cpp:415-440)."""
    from oracle import oracle as o
    from samaya_gb300.problem import model_solution
    x, _act, row_dual, _obj = model_solution(case_model, scaling, r.x, r.y)
    return o.verify_lp(case_model, x, row_dual)


def test_solutions_pass_the_reference_verifier(engine):
    """Optimal answers at 1e-8 against the reference's independent verifier (default tolerances
    1e-6, include/samaya/verify.hpp:17-21). The reference's acceptance bar for PDLP answers
    (tests/test_pdlp.cpp:497-540, which sends an answer that fails verification to crossover and
    the dual simplex) is that at least 80% pass; its own CPU PDLP passes every one of these, and
    so must the engine with the reference algorithm in FP64. Every precision mode with the
    enhanced algorithm, and the Halpern iteration, must reach the 80% bar on the 50
    pdlp_random_feasible LPs and the 200 x 500 random sparse LPs together."""
    from samaya_gb300.problem import Scaling
    cases = [("feasible8", c) for c in load_group("feasible8") if c.ref_status == engine.OPTIMAL]
    cases += [("config0_small", c) for c in load_group("config0_small")]
    failures = {}
    modes = [("fp64-reference", engine.FP64, engine.REFERENCE)] + [
        (f"{name}-enhanced", prec, engine.ENHANCED) for name, prec in (
            ("fp64", engine.FP64), ("fp32-then-fp64", engine.FP32_THEN_FP64),
            ("fp32-refined", engine.FP32_REFINED))] + [
        ("fp64-halpern", engine.FP64, engine.HALPERN),
        ("fp32-then-fp64-halpern", engine.FP32_THEN_FP64, engine.HALPERN)]
    for mode, prec, alg in modes:
        failures[mode] = []
        for grp, case in cases:
            r = engine.solve_pdlp(case.lp, engine.PdlpOptions(
                tol=1e-8, max_iterations=case.max_iter, precision=prec, algorithm=alg))
            ok, rep = _verify(engine, case.model, Scaling(case.col_scale, case.row_scale), r)
            if r.status != engine.OPTIMAL or not ok:
                failures[mode].append((grp, case.k, r.status_name, rep))
    assert not failures["fp64-reference"], failures["fp64-reference"]
    for mode, bad in failures.items():
        assert len(bad) <= 0.2 * len(cases), (mode, bad)


def test_autotuned_tiles_agree_with_the_built_in_rule(engine):
    """A 20000 x 50000 random sparse LP (300,000 nonzeros: large enough to be tuned): the tile
    shape the autotuner picks is one of its candidates, a second engine on the same structure
    gets the same shape from the cache, and the solve agrees with the built-in rule's (status;
    objective to 1e-3 relative at 1e-4, where the summation order may differ)."""
    from samaya_gb300.generators import random_sparse_lp
    from samaya_gb300.problem import make_problem
    lp, _ = make_problem(random_sparse_lp(20000, 50000, seed=4))
    base = dict(tol=1e-4, algorithm=engine.REFERENCE)
    with engine.PdlpSolver(lp, engine.PdlpOptions(autotune=False, **base)) as s0:
        r0 = s0.solve()
        rule = s0.tile_shapes()
    with engine.PdlpSolver(lp, engine.PdlpOptions(autotune=True, **base)) as s1:
        r1 = s1.solve()
        tuned = s1.tile_shapes()
    with engine.PdlpSolver(lp, engine.PdlpOptions(autotune=True, **base)) as s2:
        assert s2.tile_shapes() == tuned
    for name in ("A", "At"):
        assert tuned[name][0] in (rule[name][0] // 2, rule[name][0], 2 * rule[name][0],
                                  4 * rule[name][0]), (tuned, rule)
    assert r0.status == r1.status == engine.OPTIMAL
    o0 = float(np.dot(lp.cost, r0.x))
    o1 = float(np.dot(lp.cost, r1.x))
    assert abs(o0 - o1) <= 1e-3 * (1 + abs(o0)), (o0, o1)


_TILE_CACHE_SCRIPT = """
import sys
sys.path.insert(0, {root!r})
import samaya_gb300 as sg
from samaya_gb300.generators import random_sparse_lp
from samaya_gb300.problem import make_problem
lp, _ = make_problem(random_sparse_lp(20000, 50000, seed=4))
with sg.PdlpSolver(lp, sg.PdlpOptions(tol=1e-4, algorithm=sg.REFERENCE)) as s:
    print(s.tile_shapes())
"""


def test_tile_cache_file_carries_the_tuned_shapes(tmp_path):
    """SG_TILE_CACHE: a first process tunes the 20000 x 50000 LP's operators and appends its
    choices to the file; a second process reads them instead of timing (same shapes, file not
    grown)."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = tmp_path / "tiles.txt"
    env = dict(os.environ, SG_TILE_CACHE=str(path))
    script = _TILE_CACHE_SCRIPT.format(root=root)
    first = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True,
                           text=True, timeout=600)
    assert first.returncode == 0, first.stderr
    lines = path.read_text().splitlines()
    assert len(lines) == 2 and all(len(x.split()) == 16 for x in lines), lines
    second = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True,
                            text=True, timeout=600)
    assert second.returncode == 0, second.stderr
    assert second.stdout == first.stdout
    assert path.read_text().splitlines() == lines


def test_reference_algorithm_iteration_counts_match_the_reference(engine):
    """SG_ALGORITHM_REFERENCE in FP64 follows the reference's CPU PDLP step for step: on the
    parity fixtures it stops with the reference's status after the reference's number of
    iterations (every evaluation, restart and primal-weight decision the same), whenever the
    reference itself stops before its iteration limit."""
    counted, differ = 0, []
    for group in ("feasible8", "vs_simplex10", "gpu_vs_cpu6", "repeatable30", "config0_small"):
        for case in load_group(group):
            r = solve(engine, case, algorithm=engine.REFERENCE)
            counted += 1
            if r.status != case.ref_status or r.iterations != case.ref_iterations:
                differ.append((group, case.k, r.status, case.ref_status, r.iterations,
                               case.ref_iterations))
    assert counted > 100
    assert not differ, differ


def test_device_equilibration_and_step_size_match_the_oracle(engine, oracle):
    """The device setup of the reference algorithm — 10 passes of L2 Ruiz
    (pdlp.cpp:109-187), the power-iteration estimate of ||[A_eq -I]|| (pdlp.cpp:36-103) and
    eta = 0.99 / ||[A_eq -I]|| (pdlp.cpp:311-315) — against the oracle's to 1e-12 relative."""
    from samaya_gb300.generators import random_sparse_lp
    from samaya_gb300.problem import make_problem
    cases = [c.lp for c in load_group("feasible8")[:10] if c.lp.m > 0]
    cases += [c.lp for c in load_group("config0_small")]
    cases.append(make_problem(random_sparse_lp(2000, 5000, seed=0))[0])
    for lp in cases:
        with engine.PdlpSolver(lp, engine.PdlpOptions(algorithm=engine.REFERENCE)) as s:
            cs, rs, norm, eta = s.equilibration()
        o_rs, o_cs, _, _, o_norm = oracle.setup(*lp.arrays()[:5])
        assert np.max(np.abs(cs - o_cs) / np.abs(o_cs)) <= 1e-12
        assert np.max(np.abs(rs - o_rs) / np.abs(o_rs)) <= 1e-12
        assert abs(norm - o_norm) <= 1e-12 * o_norm
        assert abs(eta - 0.99 / o_norm) <= 1e-12 * eta
