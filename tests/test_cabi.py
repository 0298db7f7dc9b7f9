"""The C-ABI library builds, loads and exports every function include/*.h declares; argument
checks that need no GPU behave like the reference's (errors are codes, never exceptions)."""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

from samaya_gb300 import _native


def _lib():
    return _native.load(build_if_missing=True)


def test_every_declared_symbol_is_exported():
    lib = _lib()
    names = _native.declared_symbols()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_error_strings_and_defaults():
    lib = _lib()
    assert lib.sg_pdlp_error_string(0) == b"ok"
    assert lib.sg_pdlp_error_string(-1) == b"invalid argument"
    assert lib.sg_pdlp_error_string(-5).startswith(b"problem too large")
    o = _native.Opts()
    lib.sg_pdlp_default_opts(ctypes.byref(o))
    assert o.tol == 1e-8 and o.max_iterations == -1 and o.precision == 0


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def test_invalid_problems_are_rejected_before_any_device_work():
    lib = _lib()
    h = ctypes.c_void_p()
    colptr = np.array([0, 2, 3], dtype=np.int64)
    rowidx = np.array([0, 5, 1], dtype=np.int32)  # row 5 out of range for m = 2
    vals = np.array([1.0, 2.0, 3.0])
    v = np.zeros(4)
    rc = lib.sg_pdlp_create(ctypes.byref(h), 2, 2, _p(colptr, ctypes.c_int64),
                            _p(rowidx, ctypes.c_int32), _p(vals, ctypes.c_double),
                            _p(v, ctypes.c_double), _p(v, ctypes.c_double),
                            _p(v, ctypes.c_double), None)
    assert rc == -1 and not h.value
    assert b"row index" in lib.sg_pdlp_last_error()
    rowidx[1] = 1
    vals[0] = np.nan
    rc = lib.sg_pdlp_create(ctypes.byref(h), 2, 2, _p(colptr, ctypes.c_int64),
                            _p(rowidx, ctypes.c_int32), _p(vals, ctypes.c_double),
                            _p(v, ctypes.c_double), _p(v, ctypes.c_double),
                            _p(v, ctypes.c_double), None)
    assert rc == -1
    bad = np.array([0, 2, 1], dtype=np.int64)  # decreasing column starts
    vals[0] = 1.0
    rc = lib.sg_pdlp_create(ctypes.byref(h), 2, 2, _p(bad, ctypes.c_int64),
                            _p(rowidx, ctypes.c_int32), _p(vals, ctypes.c_double),
                            _p(v, ctypes.c_double), _p(v, ctypes.c_double),
                            _p(v, ctypes.c_double), None)
    assert rc == -1
    assert b"column starts" in lib.sg_pdlp_last_error()
    # A cost that is not finite, a bound that is NaN (structural or logical).
    for arr, k, value in (("cost", 1, np.inf), ("lower", 3, np.nan), ("upper", 0, np.nan)):
        vecs = {"cost": np.zeros(4), "lower": np.zeros(4), "upper": np.zeros(4)}
        vecs[arr][k] = value
        rc = lib.sg_pdlp_create(ctypes.byref(h), 2, 2, _p(colptr, ctypes.c_int64),
                                _p(rowidx, ctypes.c_int32), _p(vals, ctypes.c_double),
                                _p(vecs["cost"], ctypes.c_double),
                                _p(vecs["lower"], ctypes.c_double),
                                _p(vecs["upper"], ctypes.c_double), None)
        assert rc == -1 and not h.value
        assert b"cost or bound" in lib.sg_pdlp_last_error()
    # The row-index and value checks run on several host threads: a bad entry near the end of
    # a large matrix is found too.
    nnz = 3_000_000
    big_ptr = np.arange(0, nnz + 1, 3, dtype=np.int64)
    big_rows = np.tile(np.array([0, 1, 2], dtype=np.int32), nnz // 3)
    big_vals = np.ones(nnz)
    big_rows[-2] = 7
    nb = len(big_ptr) - 1
    zero = np.zeros(nb + 3)
    rc = lib.sg_pdlp_create(ctypes.byref(h), 3, nb, _p(big_ptr, ctypes.c_int64),
                            _p(big_rows, ctypes.c_int32), _p(big_vals, ctypes.c_double),
                            _p(zero, ctypes.c_double), _p(zero, ctypes.c_double),
                            _p(zero, ctypes.c_double), None)
    assert rc == -1 and b"row index" in lib.sg_pdlp_last_error()
    assert lib.sg_pdlp_solve(None, None, None, None, None, None) == -1
    lib.sg_pdlp_destroy(None)


def test_no_device_is_reported_as_an_error_code():
    """Where no GPU is usable (this machine, or CUDA_VISIBLE_DEVICES empty) the availability
    query answers SG_ERR_NO_DEVICE; on a GPU machine there is nothing to check."""
    lib = _lib()
    if _has_gpu():
        pytest.skip("a GPU is visible")
    major, minor = ctypes.c_int(0), ctypes.c_int(0)
    buf = ctypes.create_string_buffer(64)
    assert lib.sg_pdlp_available(ctypes.byref(major), ctypes.byref(minor), buf, 64) == -2


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def _csr_reference(m, n, colptr, rowidx, vals):
    """Sequential stable counting sort (the reference's SparseMatrix::transpose,
    src/linalg/sparse_matrix.cpp:48-78)."""
    ptr = np.zeros(m + 1, dtype=np.int64)
    np.add.at(ptr, rowidx.astype(np.int64) + 1, 1)
    ptr = np.cumsum(ptr)
    nxt = ptr[:-1].copy()
    idx = np.zeros(len(rowidx), dtype=np.int32)
    val = np.zeros(len(rowidx))
    for j in range(n):
        for p in range(colptr[j], colptr[j + 1]):
            q = nxt[rowidx[p]]
            nxt[rowidx[p]] += 1
            idx[q] = j
            val[q] = vals[p]
    return ptr, idx, val


def test_csc_to_csr_matches_the_sequential_transpose():
    """The threaded CSC -> CSR (the engine's row-major copy of A) against the sequential
    counting sort: a skewed 300 x 40000 matrix large enough for several threads (empty rows
    and columns, one dense row), a transportation-shaped matrix, an empty matrix; errors for a
    bad row index and a non-finite value."""
    lib = _lib()
    rng = np.random.default_rng(7)

    def run(m, n, colptr, rowidx, vals):
        ptr = np.zeros(m + 1, dtype=np.int32)
        idx = np.zeros(max(len(rowidx), 1), dtype=np.int32)
        val = np.zeros(max(len(rowidx), 1))
        rc = lib.sg_csc_to_csr(m, n, _p(colptr, ctypes.c_int64), _p(rowidx, ctypes.c_int32),
                               _p(vals, ctypes.c_double), _p(ptr, ctypes.c_int32),
                               _p(idx, ctypes.c_int32), _p(val, ctypes.c_double))
        return rc, ptr, idx[:len(rowidx)], val[:len(rowidx)]

    m, n = 300, 40000
    counts = rng.integers(0, 60, size=n)
    counts[::7] = 0
    cols = []
    for j in range(n):
        k = int(counts[j])
        rows = rng.choice(np.arange(1, m), size=min(k, m - 1), replace=False)
        if j % 3 == 0:
            rows = np.union1d(rows, [0])  # row 0 dense
        cols.append(np.sort(rows))
    colptr = np.zeros(n + 1, dtype=np.int64)
    colptr[1:] = np.cumsum([len(c) for c in cols])
    rowidx = np.concatenate(cols).astype(np.int32)
    vals = rng.standard_normal(len(rowidx))
    rc, ptr, idx, val = run(m, n, colptr, rowidx, vals)
    assert rc == 0
    rptr, ridx, rval = _csr_reference(m, n, colptr, rowidx, vals)
    assert np.array_equal(ptr, rptr) and np.array_equal(idx, ridx) and np.array_equal(val, rval)

    s, d = 40, 90
    j = np.arange(s * d)
    colptr = (2 * np.arange(s * d + 1)).astype(np.int64)
    rowidx = np.stack([j // d, s + j % d], axis=1).reshape(-1).astype(np.int32)
    vals = np.ones(len(rowidx))
    rc, ptr, idx, val = run(s + d, s * d, colptr, rowidx, vals)
    rptr, ridx, rval = _csr_reference(s + d, s * d, colptr, rowidx, vals)
    assert rc == 0 and np.array_equal(ptr, rptr) and np.array_equal(idx, ridx)

    rc, ptr, _, _ = run(3, 2, np.zeros(3, dtype=np.int64), np.zeros(0, dtype=np.int32),
                        np.zeros(0))
    assert rc == 0 and np.array_equal(ptr, np.zeros(4))

    colptr = np.array([0, 2, 3], dtype=np.int64)
    rc, _, _, _ = run(2, 2, colptr, np.array([0, 5, 1], dtype=np.int32), np.ones(3))
    assert rc == -1
    rc, _, _, _ = run(2, 2, colptr, np.array([0, 1, 1], dtype=np.int32),
                      np.array([1.0, np.inf, 2.0]))
    assert rc == -1


def test_plain_c_caller_reads_mps(tmp_path):
    """include/sg_mps.h and include/sg_pdlp.h compile as C99; a C program linked with the
    library reads an MPS file through sg_mps_* (the same sizes, sense, offset and entries as the
    Python binding), reports a refused file with its status and message, and gets
    SG_ERR_NO_DEVICE on a machine without a GPU."""
    import shutil
    import subprocess
    from samaya_gb300 import build, mps
    from samaya_gb300 import generators as g
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lib = build.build()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = tmp_path / "mps_reader_c"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic", "-I",
                    os.path.join(root, "include"), os.path.join(root, "tests", "c",
                                                                "mps_reader_c.c"),
                    "-L", os.path.dirname(lib), "-lsamaya_gb300",
                    f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", str(exe)], check=True)
    model = g.random_sparse_lp(50, 120, seed=4)
    path = tmp_path / "lp.mps"
    mps.write_mps(model, path)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([str(exe), str(path)], capture_output=True, text=True, env=env,
                         check=True).stdout.split("\n")
    f = mps.read_mps(path)
    got = out[0].split()
    assert got[0] == "read", out
    assert [int(v) for v in got[1:6]] == [f.model.m, f.model.n, f.model.nnz, 0, 0]
    assert float(got[6]) == f.model.obj_offset
    assert float(got[7]) == pytest.approx(float(np.sum(f.model.vals)), rel=1e-12)
    assert got[8:] == ["R0", "C0"]
    assert out[1] == "available -2"
    bad = tmp_path / "bad.mps"
    bad.write_text("NAME x\nROWS\n N obj\nCOLUMNS\n x r 1\nENDATA\n")
    out = subprocess.run([str(exe), str(bad)], capture_output=True, text=True, env=env,
                         check=True).stdout
    assert out.startswith("error -8 not valid free MPS: line 5: unknown row 'r'"), out


def test_scale_model_refuses_malformed_models():
    """sg_scale_model answers SG_ERR_INVALID_ARGUMENT, writing nothing past its outputs, for
    column starts that do not begin at 0 or decrease, a row index out of range, a value or cost
    that is not finite, or a NaN bound; a valid model gives SG_OK."""
    from samaya_gb300 import generators as g
    lib = _lib()
    base = g.random_sparse_lp(30, 70, seed=2)

    def run(**kw):
        md = {k: np.array(getattr(base, k), copy=True) for k in (
            "colptr", "rowidx", "vals", "obj", "col_lower", "col_upper", "row_lower",
            "row_upper")}
        for k, f in kw.items():
            f(md[k])
        m, n, nnz = base.m, base.n, int(base.colptr[-1])
        cp = np.ascontiguousarray(md["colptr"], dtype=np.int64)
        ri = np.ascontiguousarray(md["rowidx"], dtype=np.int32)
        d = [np.ascontiguousarray(md[k], dtype=np.float64) for k in (
            "vals", "obj", "col_lower", "col_upper", "row_lower", "row_upper")]
        oc = np.zeros(n + 1, dtype=np.int64)
        orow = np.zeros(nnz, dtype=np.int32)
        ov = np.zeros(nnz)
        outs = [np.zeros(n + m) for _ in range(3)] + [np.zeros(n), np.zeros(m)]
        k = ctypes.c_int64(0)
        D = ctypes.POINTER(ctypes.c_double)
        return lib.sg_scale_model(m, n, _p(cp, ctypes.c_int64), _p(ri, ctypes.c_int32),
                                  *[a.ctypes.data_as(D) for a in d], 0,
                                  _p(oc, ctypes.c_int64), _p(orow, ctypes.c_int32),
                                  ov.ctypes.data_as(D), *[a.ctypes.data_as(D) for a in outs],
                                  ctypes.byref(k))

    def at(i, v):
        def f(a):
            a[i] = v
        return f
    assert run() == 0
    assert run(colptr=at(0, 1)) == -1
    assert run(colptr=at(5, int(base.colptr[6]) + 1)) == -1
    assert run(rowidx=at(3, base.m)) == -1
    assert run(rowidx=at(3, -1)) == -1
    assert run(vals=at(7, np.nan)) == -1
    assert run(vals=at(7, np.inf)) == -1
    assert run(obj=at(2, np.inf)) == -1
    assert run(col_upper=at(4, np.nan)) == -1
    assert run(row_lower=at(1, np.nan)) == -1
    assert run(col_upper=at(4, np.inf), row_lower=at(1, -np.inf)) == 0


def test_batch_create_checks_every_matrix_before_the_device():
    """sg_batch_create checks each matrix's column starts (from 0, never decreasing) and entries
    before it looks for a GPU: a malformed matrix is SG_ERR_INVALID_ARGUMENT with its reason,
    and on a machine without a GPU a valid batch is SG_ERR_NO_DEVICE."""
    from samaya_gb300 import _native
    from samaya_gb300.batch import BatchSolver
    from samaya_gb300 import generators as g
    from samaya_gb300.problem import make_problem
    lp = make_problem(g.random_sparse_lp(20, 50, seed=1))[0]
    good = (lp.m, lp.n, lp.colptr, lp.rowidx, lp.vals)
    cp = lp.colptr.copy()
    cp[3] = cp[4] + 1
    bad = (lp.m, lp.n, cp, lp.rowidx, lp.vals)
    inst = [(1, lp.cost, lp.lower, lp.upper)]
    with pytest.raises(_native.EngineError) as e:
        BatchSolver([good, bad], inst)
    assert e.value.code == -1 and "column starts decrease" in str(e.value)
    if not _has_gpu():
        with pytest.raises(_native.EngineError) as e:
            BatchSolver([good], [(0, lp.cost, lp.lower, lp.upper)])
        assert e.value.code == -2


def test_unscale_needs_row_scales_for_row_outputs():
    lib = _lib()
    x_lp = np.zeros(5)
    x = np.zeros(3)
    act = np.zeros(2)
    cs = np.ones(3)
    D = ctypes.POINTER(ctypes.c_double)
    assert lib.sg_unscale_solution(2, 3, cs.ctypes.data_as(D), None, 0, x_lp.ctypes.data_as(D),
                                   None, x.ctypes.data_as(D), act.ctypes.data_as(D), None) == -1
    assert lib.sg_unscale_solution(2, 3, cs.ctypes.data_as(D), None, 0, x_lp.ctypes.data_as(D),
                                   None, x.ctypes.data_as(D), None, None) == 0
