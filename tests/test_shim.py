"""The samaya integration compiled against samaya's own headers and library (CPU test; it runs
only where the samaya checkout and its compiled library, oracle/_ref, exist).

tests/shim/shim_main.cpp routes samaya's solve_pdlp through the GB300 binding
(samaya_gb300/shim/solve_pdlp_gpu.cpp) and drives samaya's Solver through the C API additions
(samaya_gb300/shim/samaya_c_pdlp.cpp). Without a usable GPU (CUDA_VISIBLE_DEVICES empty) the
binding must hand every solve to samaya's own CPU PDLP (reference src/lp/pdlp.cpp:228-246, the
GPU fallback), with the results samaya gives without the binding."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAMAYA_OPTIMAL = 1
LP_DUAL_SIMPLEX, LP_PDLP = 1, 4


def _write_mps(model, path):
    """Free-format MPS of a Model (rows E / L / G, bounds LO / UP / MI / PL)."""
    m, n = model.m, model.n

    def num(v):
        return repr(float(v))
    lines = ["NAME test", "ROWS", " N obj"]
    kinds = []
    for i in range(m):
        lo, up = model.row_lower[i], model.row_upper[i]
        kinds.append("E" if lo == up else ("L" if np.isinf(lo) else "G"))
        lines.append(f" {kinds[-1]} r{i}")
    lines.append("COLUMNS")
    for j in range(n):
        lines.append(f" x{j} obj {num(model.obj[j])}")
        for p in range(model.colptr[j], model.colptr[j + 1]):
            lines.append(f" x{j} r{model.rowidx[p]} {num(model.vals[p])}")
    lines.append("RHS")
    for i in range(m):
        rhs = model.row_upper[i] if kinds[i] in ("E", "L") else model.row_lower[i]
        lines.append(f" rhs r{i} {num(rhs)}")
    lines.append("BOUNDS")
    for j in range(n):
        lo, up = model.col_lower[j], model.col_upper[j]
        lines.append(f" MI bnd x{j}" if np.isinf(lo) else f" LO bnd x{j} {num(lo)}")
        if not np.isinf(up):
            lines.append(f" UP bnd x{j} {num(up)}")
    lines.append("ENDATA")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    from oracle import ref
    if not ref.available() or shutil.which("g++") is None:
        pytest.skip("the samaya checkout (or g++) is not present")
    lib_ref = ref.build()
    from samaya_gb300 import build as b
    lib_sg = b.build()
    out = tmp_path_factory.mktemp("shim") / "shim_main"
    src = ref.REFERENCE_ROOT
    cmd = ["g++", "-std=c++20", "-O2", "-I", os.path.join(src, "include"), "-I",
           os.path.join(src, "src"), "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "samaya_gb300", "shim"),
           os.path.join(ROOT, "tests", "shim", "shim_main.cpp"),
           os.path.join(ROOT, "samaya_gb300", "shim", "solve_pdlp_gpu.cpp"),
           os.path.join(ROOT, "samaya_gb300", "shim", "samaya_c_pdlp.cpp"),
           os.path.join(ROOT, "samaya_gb300", "shim", "read_mps_fast.cpp"),
           "-L", os.path.dirname(lib_ref), "-lsamaya_ref", "-L", os.path.dirname(lib_sg),
           "-lsamaya_gb300", f"-Wl,-rpath,{os.path.dirname(lib_ref)}",
           f"-Wl,-rpath,{os.path.dirname(lib_sg)}", "-ldl", "-lpthread", "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def _run(exe, mps, method, use_gpu, tol, sol=None):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    args = [str(exe), str(mps), str(method), str(use_gpu), repr(tol)] + ([str(sol)] if sol else [])
    p = subprocess.run(args, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    status, obj, verified, engine, cpu = p.stdout.split()
    return int(status), float(obj), int(verified), int(engine), int(cpu)


def test_samaya_c_api_reaches_pdlp_and_falls_back_to_the_cpu(shim, tmp_path, oracle):
    """samaya_solve_params(model, PDLP, use_gpu = 1, ...) on a 60 x 150 random sparse LP with
    no GPU visible: the binding answers on samaya's CPU PDLP (one CPU solve, no engine solve),
    the status is optimal and verified, the objective is the one samaya gives with use_gpu = 0
    (bit for bit) and agrees with its dual simplex to 1e-6, and samaya_solve_get_solution
    returns a solution the verifier restatement accepts."""
    from samaya_gb300.generators import random_sparse_lp
    model = random_sparse_lp(60, 150, seed=3)
    mps = tmp_path / "lp.mps"
    _write_mps(model, mps)
    sol = tmp_path / "sol.bin"
    st, obj, verified, engine, cpu = _run(shim, mps, LP_PDLP, 1, 1e-8, sol)
    assert st == SAMAYA_OPTIMAL and verified == 1
    assert engine == 0 and cpu == 1
    st0, obj0, _, engine0, cpu0 = _run(shim, mps, LP_PDLP, 0, 1e-8)
    assert st0 == SAMAYA_OPTIMAL and obj0 == obj and engine0 == 0 and cpu0 == 1
    sts, objs, _, _, cpus = _run(shim, mps, LP_DUAL_SIMPLEX, 1, 1e-8)
    assert sts == SAMAYA_OPTIMAL and cpus == 0
    assert abs(obj - objs) <= 1e-6 * (1 + abs(objs))
    data = np.fromfile(sol, dtype=np.float64)
    x, y = data[:model.n], data[model.n:]
    ok, rep = oracle.verify_lp(model, x, y)
    assert ok, rep


def _write_replay(path, x, y, status, iterations):
    with open(path, "wb") as f:
        f.write(np.array([len(x) - len(y), len(y)], dtype=np.int64).tobytes())
        f.write(np.array([status], dtype=np.int32).tobytes())
        f.write(np.array([iterations], dtype=np.int64).tobytes())
        f.write(np.ascontiguousarray(x, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(y, dtype=np.float64).tobytes())


def _crossover(exe, mps, replay=None, dual=False):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", SG_SHIM_REPLAY=str(replay or ""))
    args = [str(exe), "--crossover", str(mps)] + (["dual"] if dual else [])
    p = subprocess.run(args, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    st, obj, iters, crossed, verified, engine, cpu, replayed = p.stdout.split()
    return dict(status=int(st), objective=float(obj), simplex=int(iters), crossover=int(crossed),
                verified=int(verified), replayed=int(replayed))


def test_crossover_from_the_engine_point(shim, tmp_path):
    """Crossover seeding from the GPU point (samaya's --crossover path, src/core/solver.cpp:
    451-461, 541-571): samaya's Solver, presolve off, takes the engine's 1e-8 answer (computed
    on a GB300 by tests/golden/make_engine_answers.py and replayed here) as its PDLP point,
    guesses the crossover basis from it and finishes with the simplex. On every LP the
    crossover is accepted, the answer is optimal and verified with the dual simplex's
    objective (1e-9 relative), and the simplex work left is at most half of the dual simplex's
    from its own start, and at most 5% of it over all the LPs (measured: 0 / 370, 177 / 416 on
    the degenerate facility-location LP, 9 / 1,790, 0 / 2,188)."""
    path = os.path.join(ROOT, "tests", "golden", "engine_answers.npz")
    if not os.path.exists(path):
        pytest.skip("no engine answers (made on a GPU machine)")
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_engine_answers import crossover_lps
    answers = np.load(path)
    seeded_total = fresh_total = 0
    for name, model in crossover_lps():
        mps = tmp_path / f"{name}.mps"
        _write_mps(model, mps)
        replay = tmp_path / f"{name}.bin"
        meta = answers[f"{name}_meta"]
        assert int(meta[0]) == 0  # the engine's answer is optimal
        _write_replay(replay, answers[f"{name}_x"], answers[f"{name}_y"], int(meta[0]),
                      int(meta[1]))
        seeded = _crossover(shim, mps, replay=replay)
        fresh = _crossover(shim, mps, dual=True)
        assert seeded["replayed"] == 1 and seeded["crossover"] == 1, (name, seeded)
        assert seeded["status"] == fresh["status"] == SAMAYA_OPTIMAL
        assert seeded["verified"] == fresh["verified"] == 1
        assert abs(seeded["objective"] - fresh["objective"]) <= 1e-9 * (
            1 + abs(fresh["objective"])), (name, seeded, fresh)
        assert seeded["simplex"] <= 0.5 * fresh["simplex"], (name, seeded, fresh)
        seeded_total += seeded["simplex"]
        fresh_total += fresh["simplex"]
    assert seeded_total <= 0.05 * fresh_total, (seeded_total, fresh_total)


def _read(exe, path):
    p = subprocess.run([str(exe), "--read", str(path)], capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr
    same, fast, own, t_fast, t_own = p.stdout.split()
    return dict(same=int(same), fast=int(fast), samaya=int(own), t_fast=float(t_fast),
                t_own=float(t_own))


def test_read_mps_binding_gives_samayas_model(shim, tmp_path):
    """samaya_gb300::read_mps (the fast reader's binding) returns the Model samaya::read_mps
    returns, every field bit for bit, on the accepted MPS cases; what the fast reader declines
    (the quadratic sections) goes to samaya's reader with the same result; on a file that
    neither reads, the binding throws samaya's error (exit status 3)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from mps_cases import accepted_cases, rejected_cases
    for name, text in accepted_cases():
        path = tmp_path / f"{name}.mps"
        path.write_bytes(text.encode())
        r = _read(shim, path)
        assert r["same"] == 1 and r["fast"] == 1 and r["samaya"] == 0, (name, r)
    for name, text, status, samaya in rejected_cases():
        path = tmp_path / f"{name}.mps"
        path.write_bytes(text.encode())
        if samaya == "reads":
            r = _read(shim, path)
            assert r["same"] == 1 and r["fast"] == 0 and r["samaya"] == 1, (name, r)
        else:
            p = subprocess.run([str(shim), "--read", str(path)], capture_output=True,
                               text=True, timeout=600)
            assert p.returncode == 3, (name, p.stdout, p.stderr)


def test_read_mps_binding_on_the_transportation_lp(shim, tmp_path):
    """The 93 MB transportation LP (1000 x 2000): the same Model as samaya's reader; the binding
    (fast reader plus samaya's from_triplets) takes a fraction of samaya's time."""
    from samaya_gb300 import generators as g
    from samaya_gb300.mps import write_mps
    path = tmp_path / "transport.mps"
    write_mps(g.transportation_lp(1000, 2000, seed=0), path)
    r = _read(shim, path)
    assert r["same"] == 1 and r["fast"] == 1, r
    assert r["t_fast"] < 0.5 * r["t_own"], r


def test_cli_chain_with_the_fast_reader(shim, tmp_path):
    """The CLI's `--lp-method pdlp --gpu model.mps` chain with the fast reader's binding in
    place of samaya::read_mps: samaya's Solver, with solve_pdlp routed through the engine's
    binding (no GPU here: samaya's CPU PDLP), answers bit for bit as it does from samaya's own
    reader, optimal and verified."""
    from samaya_gb300 import generators as g
    from samaya_gb300.mps import write_mps
    for k, model in enumerate((g.random_sparse_lp(60, 150, seed=3),
                               g.transportation_lp(8, 12, seed=4))):
        path = tmp_path / f"lp{k}.mps"
        write_mps(model, path)
        env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
        p = subprocess.run([str(shim), "--cli", str(path), "1e-7"], capture_output=True,
                           text=True, env=env, timeout=600)
        assert p.returncode == 0, p.stderr
        same, status, objective, verified, fast, engine, cpu = p.stdout.split()
        assert same == "1" and status == str(SAMAYA_OPTIMAL) and verified == "1", p.stdout
        assert fast == "1" and engine == "0" and int(cpu) >= 2, p.stdout
