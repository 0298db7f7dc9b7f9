"""The engine's host-side model code under AddressSanitizer and UBSan (CPU test): sg_scale_model
(samaya_gb300/csrc/sg_model.cpp) and the threaded checks and transpose of sg_pdlp_create
(samaya_gb300/csrc/sg_transpose.cpp), built with -fsanitize=address,undefined together with
tests/c/host_sanitize_driver.cpp, on generated LPs of every family (empty rows and columns, free
and fixed bounds, maximisation), on the edge sizes m = 0 and n = 1, and on invalid models (a row
index out of range, a NaN value, an infinite cost, decreasing column starts). No sanitizer
report; the sanitized build's LpProblem is the library's, byte for byte; the checks and the
transpose give the same results at 1 and 4 threads, and the CSR is the library's
sg_csc_to_csr."""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _write(path, model):
    with open(path, "wb") as f:
        f.write(np.array([model.m, model.n, int(model.maximize), int(model.colptr[-1])],
                         dtype=np.int64).tobytes())
        for a, t in ((model.colptr, np.int64), (model.rowidx, np.int32), (model.vals, np.float64),
                     (model.obj, np.float64), (model.col_lower, np.float64),
                     (model.col_upper, np.float64), (model.row_lower, np.float64),
                     (model.row_upper, np.float64)):
            f.write(np.ascontiguousarray(a, dtype=t).tobytes())


def _models():
    from samaya_gb300 import generators as g
    from samaya_gb300.model import Model
    out = [g.random_sparse_lp(120, 300, seed=1), g.transportation_lp(20, 30, seed=2),
           g.power_law_lp(m=3000, n=6000, seed=3), g.facility_location_lp(8, 30, seed=4)]
    base = g.random_sparse_lp(60, 150, seed=5)
    cl, cu = base.col_lower.copy(), base.col_upper.copy()
    cl[::3], cu[::3] = -np.inf, np.inf
    cl[1::5] = cu[1::5] = 0.5
    out.append(Model(**{**base.__dict__, "col_lower": cl, "col_upper": cu, "maximize": True}))
    # empty rows and columns: drop the entries of a few columns and never touch a few rows
    keep = np.ones(base.nnz, dtype=bool)
    for j in (0, 7, 8):
        keep[base.colptr[j]:base.colptr[j + 1]] = False
    keep &= base.rowidx >= 3
    counts = np.array([keep[base.colptr[j]:base.colptr[j + 1]].sum() for j in range(base.n)])
    colptr = np.concatenate([[0], np.cumsum(counts)])
    out.append(Model(**{**base.__dict__, "colptr": colptr, "rowidx": base.rowidx[keep],
                        "vals": base.vals[keep]}))
    out.append(Model(m=0, n=3, colptr=np.zeros(4), rowidx=np.zeros(0), vals=np.zeros(0),
                     obj=np.array([1.0, -2.0, 0.5]), col_lower=np.zeros(3),
                     col_upper=np.full(3, 4.0), row_lower=np.zeros(0), row_upper=np.zeros(0)))
    out.append(Model(m=2, n=1, colptr=np.array([0, 2]), rowidx=np.array([0, 1]),
                     vals=np.array([2.0, -3.0]), obj=np.array([1.0]), col_lower=np.zeros(1),
                     col_upper=np.full(1, np.inf), row_lower=np.array([1.0, -np.inf]),
                     row_upper=np.array([np.inf, 6.0])))
    bad = []
    r = base.rowidx.copy()
    r[5] = base.m + 2
    bad.append(Model(**{**base.__dict__, "rowidx": r}))
    v = base.vals.copy()
    v[9] = np.nan
    bad.append(Model(**{**base.__dict__, "vals": v}))
    o = base.obj.copy()
    o[2] = np.inf
    bad.append(Model(**{**base.__dict__, "obj": o}))
    cp = base.colptr.copy()
    cp[4] = cp[5] + 1
    bad.append(Model(**{**base.__dict__, "colptr": cp}))
    return out, bad


def _library_scale(model):
    from samaya_gb300 import _native
    lib = _native.load(build_if_missing=True)
    m, n, nnz = model.m, model.n, int(model.colptr[-1])
    oc = np.zeros(n + 1, dtype=np.int64)
    orow = np.zeros(max(nnz, 1), dtype=np.int32)
    ov = np.zeros(max(nnz, 1))
    cost, lower, upper = np.zeros(n + m), np.zeros(n + m), np.zeros(n + m)
    cs, rs = np.zeros(max(n, 1)), np.zeros(max(m, 1))
    k = ctypes.c_int64(0)

    def p(a, t):
        return np.ascontiguousarray(a, dtype=t).ctypes.data_as(ctypes.POINTER(
            {np.int64: ctypes.c_int64, np.int32: ctypes.c_int32, np.float64: ctypes.c_double}[t]))
    keep = [np.ascontiguousarray(a, dtype=t) for a, t in (
        (model.colptr, np.int64), (model.rowidx, np.int32), (model.vals, np.float64),
        (model.obj, np.float64), (model.col_lower, np.float64), (model.col_upper, np.float64),
        (model.row_lower, np.float64), (model.row_upper, np.float64))]
    D = ctypes.POINTER(ctypes.c_double)
    st = lib.sg_scale_model(m, n, keep[0].ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                            keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                            *[a.ctypes.data_as(D) for a in keep[2:]], int(model.maximize),
                            oc.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                            orow.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                            ov.ctypes.data_as(D), cost.ctypes.data_as(D),
                            lower.ctypes.data_as(D), upper.ctypes.data_as(D),
                            cs.ctypes.data_as(D), rs.ctypes.data_as(D), ctypes.byref(k))
    del p
    if st != 0:
        return st, b""
    parts = [oc, orow[:k.value], ov[:k.value], cost, lower, upper, cs[:n], rs[:m]]
    return st, b"".join(a.tobytes() for a in parts)


def test_host_model_code_is_clean_under_sanitizers(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "host_sanitize"
    csrc = os.path.join(ROOT, "samaya_gb300", "csrc")
    build = subprocess.run(
        ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
         "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-pthread", "-I", csrc, "-I",
         os.path.join(ROOT, "include"), os.path.join(csrc, "sg_model.cpp"),
         os.path.join(csrc, "sg_transpose.cpp"),
         os.path.join(HERE, "c", "host_sanitize_driver.cpp"), "-o", str(exe)],
        capture_output=True, text=True)
    if build.returncode != 0 and "sanitize" in build.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert build.returncode == 0, build.stderr
    good, bad = _models()
    paths = []
    for k, model in enumerate(good + bad):
        p = tmp_path / f"model{k}.bin"
        _write(p, model)
        paths.append(p)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:halt_on_error=1",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    run = subprocess.run([str(exe)], input="\n".join(map(str, paths)) + "\n",
                         capture_output=True, text=True, env=env, timeout=600)
    assert run.returncode == 0 and "runtime error" not in run.stderr, run.stderr[-3000:]
    from samaya_gb300 import _native
    lib = _native.load()
    for k, (model, p) in enumerate(zip(good + bad, paths)):
        out = (tmp_path / f"model{k}.bin.out").read_bytes()
        st_lib, lp = _library_scale(model)
        st = int(np.frombuffer(out[:8], dtype=np.int64)[0])
        assert st == st_lib, k
        pos = 8 + len(lp)
        assert out[8:pos] == lp, k
        checks = np.frombuffer(out[pos:pos + 32], dtype=np.int64)
        assert checks[0] == checks[2] and checks[1] == checks[3], k  # 1 and 4 threads agree
        valid = k < len(good)
        assert (checks[0] == 0 and checks[1] == 0) == valid, (k, checks)
        rest = out[pos + 32:]
        if not valid:
            assert rest == b"", k
            continue
        m, n, nnz = model.m, model.n, int(model.colptr[-1])
        size = 8 + 4 * (m + 1) + 4 * nnz + 8 * nnz
        assert len(rest) == 2 * size and rest[:size] == rest[size:], k
        assert int(np.frombuffer(rest[:8], dtype=np.int64)[0]) == 0
        ptr = np.zeros(m + 1, dtype=np.int32)
        idx = np.zeros(max(nnz, 1), dtype=np.int32)
        val = np.zeros(max(nnz, 1))
        cp = np.ascontiguousarray(model.colptr, dtype=np.int64)
        ri = np.ascontiguousarray(model.rowidx, dtype=np.int32)
        vv = np.ascontiguousarray(model.vals, dtype=np.float64)
        assert lib.sg_csc_to_csr(m, n, cp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                 ri.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                 vv.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                 ptr.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                 idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                 val.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
        want = ptr.tobytes() + idx[:nnz].tobytes() + val[:nnz].tobytes()
        assert rest[8:size] == want, k
