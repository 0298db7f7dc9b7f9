// Host CSC -> CSR of the constraint matrix (the rows of K = A), checked and multi-threaded.
//
// The reference builds its row-major copy with a sequential counting sort,
// SparseMatrix::transpose (src/linalg/sparse_matrix.cpp:48-78), before it uploads both operators
// (src/gpu/pdhg_core.cu:172-190, 242-273). Here the same
// stable counting sort runs over column ranges in parallel: every thread counts the rows of its
// columns, a prefix over (row, thread) gives each thread its own slots in every row, and the
// threads then place their entries in column order. The result is identical to the sequential
// sort for any thread count (each row lists its columns in increasing order).
#include "sg_transpose.h"

#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <new>
#include <cmath>
#include <thread>
#include <vector>

#include "../../include/sg_pdlp.h"

namespace sg {

namespace {

// Runs f(t) for t in [0, threads) on up to threads - 1 helpers and the caller; parts whose
// helper could not be started run on the caller. f must not throw.
template <typename F>
void parallel_for(int threads, const F& f) {
  std::vector<std::thread> pool;
  int started = 1;
  try {
    pool.reserve(static_cast<size_t>(std::max(0, threads - 1)));
    for (int t = 1; t < threads; ++t) {
      pool.emplace_back(f, t);
      ++started;
    }
  } catch (...) {
  }
  for (int t = started; t < threads; ++t) f(t);
  f(0);
  for (auto& th : pool) th.join();
}

}  // namespace

int csc_to_csr(int m, int n, const int64_t* colptr, const int32_t* rowidx, const double* val,
               int* kptr, int* kidx, double* kval, int max_threads, const char** why) {
  const long long nnz = colptr[n];
  // Threads: one per ~512K nonzeros, at most max_threads (and 16), and few enough that the
  // per-thread row counters (threads x m ints) stay small next to the matrix.
  int threads = static_cast<int>(std::min<long long>(nnz / (1LL << 19) + 1, 16));
  threads = std::min(threads, std::max(1, max_threads));
  const unsigned hw = std::thread::hardware_concurrency();
  if (hw > 0) threads = std::min(threads, static_cast<int>(hw));
  while (threads > 1 && static_cast<long long>(threads) * m > std::max<long long>(nnz, 1) * 2) {
    --threads;
  }
  threads = std::max(threads, 1);
  // Column ranges of about equal nonzeros.
  std::vector<int> col0(static_cast<size_t>(threads) + 1, n);
  col0[0] = 0;
  for (int t = 1; t < threads; ++t) {
    const long long target = nnz * t / threads;
    col0[t] = static_cast<int>(std::upper_bound(colptr, colptr + n + 1, target) - colptr) - 1;
    col0[t] = std::max(col0[t], col0[t - 1]);
  }
  // Per-thread row counters, allocated here so that the workers never allocate.
  std::vector<std::vector<int>> cnt(static_cast<size_t>(threads),
                                    std::vector<int>(static_cast<size_t>(m), 0));
  std::atomic<int> bad{0};
  parallel_for(threads, [&](int t) {
    std::vector<int>& c = cnt[static_cast<size_t>(t)];
    for (int j = col0[t]; j < col0[t + 1]; ++j) {
      for (long long p = colptr[j]; p < colptr[j + 1]; ++p) {
        const int r = rowidx[p];
        if (r < 0 || r >= m) {
          bad.store(1);
          return;
        }
        if (!std::isfinite(val[p])) {
          bad.store(2);
          return;
        }
        ++c[static_cast<size_t>(r)];
      }
    }
  });
  if (bad.load() != 0) {
    if (why) *why = bad.load() == 1 ? "row index out of range" : "matrix value not finite";
    return 1;
  }
  // Row starts, and each thread's first slot in every row (turning the counts into offsets).
  kptr[0] = 0;
  for (int i = 0; i < m; ++i) {
    int off = kptr[i];
    for (int t = 0; t < threads; ++t) {
      const int c = cnt[static_cast<size_t>(t)][static_cast<size_t>(i)];
      cnt[static_cast<size_t>(t)][static_cast<size_t>(i)] = off;
      off += c;
    }
    kptr[i + 1] = off;
  }
  parallel_for(threads, [&](int t) {
    std::vector<int>& next = cnt[static_cast<size_t>(t)];
    for (int j = col0[t]; j < col0[t + 1]; ++j) {
      for (long long p = colptr[j]; p < colptr[j + 1]; ++p) {
        const int q = next[static_cast<size_t>(rowidx[p])]++;
        kidx[q] = j;
        kval[q] = val[p];
      }
    }
  });
  return 0;
}

int check_nonzeros(int m, long long nnz, const int32_t* rowidx, const double* val,
                   int max_threads, const char** why) {
  int threads = static_cast<int>(std::min<long long>(nnz / (1LL << 19) + 1, 16));
  threads = std::min(threads, std::max(1, max_threads));
  const unsigned hw = std::thread::hardware_concurrency();
  if (hw > 0) threads = std::min(threads, static_cast<int>(hw));
  threads = std::max(threads, 1);
  std::atomic<int> bad_row{0}, bad_val{0};
  parallel_for(threads, [&](int t) {
    const long long p0 = nnz * t / threads;
    const long long p1 = nnz * (t + 1) / threads;
    int br = 0, bv = 0;
    for (long long p = p0; p < p1; ++p) {
      br |= rowidx[p] < 0 || rowidx[p] >= m;
      bv |= !std::isfinite(val[p]);
    }
    if (br) bad_row.store(1);
    if (bv) bad_val.store(1);
  });
  if (bad_row.load()) {
    *why = "row index out of range";
    return 1;
  }
  if (bad_val.load()) {
    *why = "matrix value not finite";
    return 1;
  }
  return 0;
}

int check_columns(int m, int n, const int64_t* colptr, const double* cost, const double* lower,
                  const double* upper, int* tptr, bool* shared, int max_threads,
                  const char** why) {
  const long long nt = static_cast<long long>(n) + m;
  int threads = static_cast<int>(std::min<long long>(nt / (1LL << 18) + 1, 16));
  threads = std::min(threads, std::max(1, max_threads));
  const unsigned hw = std::thread::hardware_concurrency();
  if (hw > 0) threads = std::min(threads, static_cast<int>(hw));
  threads = std::max(threads, 1);
  std::atomic<int> bad_start{0}, bad_vec{0}, differ{0};
  const double l0 = n > 0 ? lower[0] : 0.0;
  const double u0 = n > 0 ? upper[0] : 0.0;
  parallel_for(threads, [&](int t) {
    const long long k0 = nt * t / threads;
    const long long k1 = nt * (t + 1) / threads;
    int bs = 0, bv = 0, df = 0;
    for (long long k = k0; k < k1; ++k) {
      if (k < n) {
        bs |= colptr[k + 1] < colptr[k];
        tptr[k] = static_cast<int>(colptr[k]);
        df |= !(lower[k] == l0 && upper[k] == u0);
      }
      bv |= !std::isfinite(cost[k]) || std::isnan(lower[k]) || std::isnan(upper[k]);
    }
    if (bs) bad_start.store(1);
    if (bv) bad_vec.store(1);
    if (df) differ.store(1);
  });
  tptr[n] = static_cast<int>(colptr[n]);
  *shared = n > 0 && differ.load() == 0;
  if (bad_start.load()) {
    *why = "column starts must not decrease";
    return 1;
  }
  if (bad_vec.load()) {
    *why = "cost or bound not valid";
    return 1;
  }
  return 0;
}

}  // namespace sg

extern "C" {

/* See include/sg_pdlp.h. */
int sg_csc_to_csr(int m, int n, const int64_t* a_colptr, const int32_t* a_rowidx,
                  const double* a_val, int32_t* csr_ptr, int32_t* csr_idx, double* csr_val) {
  if (m < 0 || n < 0 || a_colptr == nullptr || csr_ptr == nullptr || a_colptr[0] != 0) {
    return SG_ERR_INVALID_ARGUMENT;
  }
  for (int j = 0; j < n; ++j) {
    if (a_colptr[j + 1] < a_colptr[j]) return SG_ERR_INVALID_ARGUMENT;
  }
  const long long nnz = a_colptr[n];
  if (nnz >= static_cast<long long>(INT32_MAX)) return SG_ERR_TOO_LARGE;
  if (nnz > 0 && (a_rowidx == nullptr || a_val == nullptr || csr_idx == nullptr ||
                  csr_val == nullptr)) {
    return SG_ERR_INVALID_ARGUMENT;
  }
  try {
    const char* why = nullptr;
    return sg::csc_to_csr(m, n, a_colptr, a_rowidx, a_val, csr_ptr, csr_idx, csr_val, 16,
                          &why) == 0
               ? SG_OK
               : SG_ERR_INVALID_ARGUMENT;
  } catch (const std::bad_alloc&) {
    return SG_ERR_OUT_OF_MEMORY;
  } catch (...) {
    return SG_ERR_INTERNAL;
  }
}

}  // extern "C"
