"""Kernel-level parity of the GPU engine with the oracle (the reference's CPU arithmetic), through
the C ABI's inner seam — the counterpart of the reference's tests/test_gpu.cpp kernel tests."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_group

pytestmark = pytest.mark.gpu


def _csc_from_rows(m, n, rows_cols_vals):
    """CSC arrays of an m x n matrix given per-row (cols, vals)."""
    trip = []
    for i, (cols, vals) in enumerate(rows_cols_vals):
        for j, v in zip(cols, vals):
            trip.append((j, i, v))
    trip.sort()
    colptr = np.zeros(n + 1, dtype=np.int64)
    rowidx = np.array([t[1] for t in trip], dtype=np.int32)
    vals = np.array([t[2] for t in trip])
    for j, _, _ in trip:
        colptr[j + 1] += 1
    return np.cumsum(colptr), rowidx, vals


def _dense(m, n, colptr, rowidx, vals):
    a = np.zeros((m, n))
    for j in range(n):
        for p in range(colptr[j], colptr[j + 1]):
            a[rowidx[p], j] += vals[p]
    return a


def test_spmv_rows_of_every_length_match_the_cpu(engine):
    """Empty rows, rows shorter than a team, 300-nonzero rows (the reference's tile-width test,
    tests/test_gpu.cpp:699-756) and rows longer than a tile (split and recombined)."""
    rng = np.random.default_rng(614)
    m, n = 3000, 20000
    rows = []
    for i in range(m):
        if i % 97 == 0:
            length = 0
        elif i == 5:
            length = 19000  # split into segments
        elif i == 1234:
            length = 4097   # one nonzero past a tile
        elif i % 41 == 0:
            length = 300
        else:
            length = 1 + int(rng.integers(0, 12))
        cols = np.sort(rng.choice(n, size=length, replace=False))
        rows.append((cols, rng.uniform(-1, 1, size=length)))
    colptr, rowidx, vals = _csc_from_rows(m, n, rows)
    A = _dense(m, n, colptr, rowidx, vals)
    dev = engine.PdhgDevice(m, n, colptr, rowidx, vals, np.zeros(n + m), np.zeros(n + m),
                            np.zeros(n + m))
    x = rng.uniform(-1, 1, size=n)
    y_cpu = A @ x
    a = dev.spmv(x)
    b = dev.spmv(x)
    assert np.array_equal(a, b)
    assert np.max(np.abs(a - y_cpu) / np.maximum(np.abs(y_cpu), 1.0)) < 1e-12
    yt = rng.uniform(-1, 1, size=m)
    t_cpu = A.T @ yt
    t = dev.spmv(yt, transpose=True)
    assert np.max(np.abs(t - t_cpu) / np.maximum(np.abs(t_cpu), 1.0)) < 1e-12
    assert np.array_equal(t, dev.spmv(yt, transpose=True))


@pytest.mark.parametrize("split", [0, 300, 1000])
def test_spmv_medium_rows_on_several_warps_match_the_cpu(engine, split):
    """A 2000 x 60000 operator with 2.6M nonzeros (4096-nonzero tiles): rows of 129 to 4096
    nonzeros (a warp per row, or with a team split of `split` nonzeros per warp teams of 2, 4
    and 8 warps; unaligned starts), rows one past a tile, short and empty rows; both products
    against scipy to 1e-12 and bit-identical on repeat."""
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(615)
    m, n = 2000, 60000
    pattern = [129, 300, 511, 513, 700, 1023, 1030, 2047, 2049, 3001, 4096, 4097, 7, 0, 33]
    lengths = np.array([pattern[i % len(pattern)] for i in range(m)])
    rows = np.repeat(np.arange(m), lengths)
    cols = np.concatenate([rng.choice(n, size=k, replace=False) for k in lengths])
    vals = rng.uniform(-1, 1, size=rows.size)
    A = sp.csc_matrix((vals, (rows, cols)), shape=(m, n))
    A.sort_indices()
    colptr = A.indptr.astype(np.int64)
    rowidx = A.indices.astype(np.int32)
    dev = engine.PdhgDevice(m, n, colptr, rowidx, A.data.copy(), np.zeros(n + m),
                            np.zeros(n + m), np.zeros(n + m),
                            options=engine.PdlpOptions(autotune=False, tile_split=split))
    x = rng.uniform(-1, 1, size=n)
    y_cpu = A @ x
    a = dev.spmv(x)
    assert np.array_equal(a, dev.spmv(x))
    assert np.max(np.abs(a - y_cpu) / np.maximum(np.abs(y_cpu), 1.0)) < 1e-12
    yt = rng.uniform(-1, 1, size=m)
    t_cpu = A.T @ yt
    t = dev.spmv(yt, transpose=True)
    assert np.max(np.abs(t - t_cpu) / np.maximum(np.abs(t_cpu), 1.0)) < 1e-12
    assert np.array_equal(t, dev.spmv(yt, transpose=True))


def _equilibrated(case, rng):
    """A small LP with a random equilibration applied as solve_pdlp applies it (the reference's
    make_device_lp, tests/test_gpu.cpp:404-446)."""
    lp = case.lp
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


def test_evaluate_matches_oracle_sums(engine, oracle):
    """gpu_evaluate_matches_host_sums (tests/test_gpu.cpp:606-638): the device's seven sums of
    the current and the average iterate equal the oracle's to 1e-11 and repeat bit-for-bit."""
    rng = np.random.default_rng(611)
    compared = 0
    for case in load_group("feasible8")[:20]:
        e = _equilibrated(case, rng)
        dev = engine.PdhgDevice(e["m"], e["n"], e["colptr"], e["rowidx"], e["vals"], e["cost"],
                                e["lower"], e["upper"])
        lp = case.lp
        dev.set_original(e["cs"], e["rs"], lp.cost, lp.lower, lp.upper)
        for it in range(7):
            dev.step(0.3, 0.3, 1.0, it)
            dev.advance()
        dev.step(0.3, 0.3, 1.0, 7)
        st = dev.download()
        for which, (v, y) in ((0, (st["v_new"], st["y_new"])), (1, (st["v_erg"], st["y_erg"]))):
            s = dev.evaluate(which)
            again = dev.evaluate(which)
            host = oracle.eval_sums(lp.m, lp.n, lp.colptr, lp.rowidx, lp.vals, lp.cost, lp.lower,
                                    lp.upper, e["cs"], e["rs"], v, y)
            assert np.all(np.abs(s - host) <= 1e-11 * (1.0 + np.abs(host))), (case.k, s, host)
            assert np.array_equal(s, again)
            compared += 1
        dev.close()
    assert compared == 40


def test_steps_match_oracle_steps(engine, oracle):
    """Eight fused PDHG steps on the device follow the oracle's steps (pdlp.cpp:574-641) to
    round-off."""
    rng = np.random.default_rng(7)
    for case in load_group("feasible8")[:10] + load_group("repeatable30"):
        e = _equilibrated(case, rng)
        dev = engine.PdhgDevice(e["m"], e["n"], e["colptr"], e["rowidx"], e["vals"], e["cost"],
                                e["lower"], e["upper"])
        lp = case.lp
        dev.set_original(e["cs"], e["rs"], lp.cost, lp.lower, lp.upper)
        state = dict(v=np.zeros(lp.n + lp.m), v_prev=np.zeros(lp.n + lp.m), y=np.zeros(lp.m),
                     v_erg=np.zeros(lp.n + lp.m), y_erg=np.zeros(lp.m))
        for it in range(8):
            dev.step(0.25, 0.35, 1.0, it)
            dev.advance()
        st = oracle.pdhg_steps(lp.m, lp.n, e["colptr"], e["rowidx"], e["vals"], e["cost"],
                               e["lower"], e["upper"], 0.25, 0.35, 8, 0, state)
        got = dev.download()
        for a, b in ((got["v"], st["v"]), (got["y"], st["y"]), (got["v_erg"], st["v_erg"]),
                     (got["y_erg"], st["y_erg"])):
            assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)) < 1e-12
        dev.close()


def test_restart_distance_and_restart_to(engine):
    """gpu_restart_distance_and_restart_to (tests/test_gpu.cpp:640-673)."""
    rng = np.random.default_rng(612)
    case = load_group("repeatable30")[0]
    e = _equilibrated(case, rng)
    dev = engine.PdhgDevice(e["m"], e["n"], e["colptr"], e["rowidx"], e["vals"], e["cost"],
                            e["lower"], e["upper"])
    lp = case.lp
    dev.set_original(e["cs"], e["rs"], lp.cost, lp.lower, lp.upper)
    for it in range(5):
        dev.step(0.3, 0.3, 1.0, it)
        dev.advance()
    dev.step(0.3, 0.3, 1.0, 5)
    st = dev.download()
    dv, dy = dev.restart_distance(1)
    host_dv = float(np.sum(st["v_erg"] ** 2))
    host_dy = float(np.sum(st["y_erg"] ** 2))
    assert abs(dv - host_dv) <= 1e-12 * (1 + host_dv)
    assert abs(dy - host_dy) <= 1e-12 * (1 + host_dy)
    assert host_dv > 0
    dev.restart_to(1)
    got = dev.download()
    assert np.array_equal(got["v"], st["v_erg"]) and np.array_equal(got["v_new"], st["v_erg"])
    assert np.array_equal(got["y"], st["y_erg"]) and np.array_equal(got["y_new"], st["y_erg"])
    dv, dy = dev.restart_distance(0)
    assert dv == 0.0 and dy == 0.0
