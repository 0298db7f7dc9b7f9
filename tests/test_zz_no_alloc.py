"""The allocation-free SpMV entry point (sg_spmv_noalloc) gives the product of a plain CSR
product on the CPU and of the engine's regular SpMV entry point (sg_spmv), on two calls in a
row.

It serves callers that cannot call cudaMalloc (a solver under a memory pool or budget that
forbids driver allocations, a plug-in whose device memory belongs to another runtime): every
array is the caller's device memory, and the only scratch is a fixed device array inside the
library. The test owns its device buffers (torch); the entry point itself allocates nothing.
The file is named to be collected last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _matrix(rng, m, n):
    """CSR rows of every kind: empty, short, a warp's worth, rows spanning several 2048-nonzero
    chunks, and trailing empty rows."""
    lens = []
    for i in range(m):
        if i % 53 == 0 or i >= m - 3:
            lens.append(0)
        elif i in (7, 300):
            lens.append(5000)      # spans chunks
        elif i == 900:
            lens.append(2048)      # exactly a chunk
        elif i % 17 == 0:
            lens.append(int(rng.integers(33, 400)))
        else:
            lens.append(int(rng.integers(1, 12)))
    ptr = np.zeros(m + 1, dtype=np.int64)
    ptr[1:] = np.cumsum(lens)
    idx = np.concatenate([np.sort(rng.choice(n, size=l, replace=False)) for l in lens if l] +
                         [np.zeros(0, dtype=np.int64)]).astype(np.int32)
    val = rng.uniform(-1.0, 1.0, size=int(ptr[-1]))
    return ptr, idx, val


def _csc(m, n, ptr, idx, val):
    rows = np.repeat(np.arange(m), np.diff(ptr))
    order = np.lexsort((rows, idx))
    colptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(colptr, idx + 1, 1)
    return np.cumsum(colptr), rows[order].astype(np.int32), val[order]


def _csr_product(ptr, idx, val, x):
    """y = A x by rows on the CPU (numpy), the independent check."""
    m = len(ptr) - 1
    rows = np.repeat(np.arange(m), np.diff(ptr))
    return np.bincount(rows, weights=val * x[idx], minlength=m)


def test_noalloc_spmv_matches_the_engine_spmv(engine):
    torch = pytest.importorskip("torch")
    from samaya_gb300 import _native
    lib = _native.load()
    f = lib.sg_spmv_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    rng = np.random.default_rng(2024)
    m, n = 1200, 9000
    ptr, idx, val = _matrix(rng, m, n)
    nnz = int(ptr[-1])
    colptr, rowidx, cval = _csc(m, n, ptr, idx, val)
    ref = engine.PdhgDevice(m, n, colptr, rowidx, cval, np.zeros(n + m), np.zeros(n + m),
                            np.zeros(n + m))
    dev = torch.device("cuda", 0)
    d_ptr = torch.from_numpy(ptr.astype(np.int32)).to(dev)
    d_idx = torch.from_numpy(idx).to(dev)
    d_val = torch.from_numpy(val).to(dev)
    d_y = torch.full((m,), float("nan"), dtype=torch.float64, device=dev)
    side = torch.cuda.Stream(device=dev)

    def call(x, count=nnz, stream=None):
        d_x = torch.from_numpy(x).to(dev)
        d_y.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = f(m, count, d_ptr.data_ptr(), d_idx.data_ptr(), d_val.data_ptr(), d_x.data_ptr(),
               d_y.data_ptr(), None if stream is None else stream.cuda_stream)
        assert rc == 0, lib.sg_pdlp_last_error()
        torch.cuda.synchronize()
        return d_y.cpu().numpy()

    def close(got, want):
        assert np.all(np.isfinite(got))
        return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), 1.0)))

    # Two calls in a row (the scratch keeps the first call's carries), the second on a stream
    # of the caller's.
    for k, stream in enumerate((None, side)):
        x = rng.uniform(-1.0, 1.0, size=n)
        got = call(x, stream=stream)
        assert close(got, _csr_product(ptr, idx, val, x)) < 1e-12, k
        assert close(got, ref.spmv(x)) < 1e-12, k
    # A count that differs from row_ptr[m] sizes the launch only: every row is still written.
    x = rng.uniform(-1.0, 1.0, size=n)
    want = _csr_product(ptr, idx, val, x)
    for count in (nnz - 3000, nnz + 5000):
        assert close(call(x, count=count), want) < 1e-12, count
    # Beyond the stated maximum the call is refused with a clear code, before any device work.
    too_many = 65536 * 2048 + 1
    assert f(m, too_many, d_ptr.data_ptr(), d_idx.data_ptr(), d_val.data_ptr(),
             d_val.data_ptr(), d_y.data_ptr(), None) == -5
    assert b"more nonzeros" in lib.sg_pdlp_last_error()
    ref.close()
