// y = A x for a CSR matrix already in device memory, with no allocation of any kind.
//
// Some callers cannot call cudaMalloc: a solver running under a memory pool or budget that
// forbids driver allocations, or a plug-in living in a process whose device memory is handed
// out by another runtime. This entry point serves them: the caller passes device pointers for
// every input and output, and the only scratch the kernels need — one carry record per chunk
// of nonzeros — sits in a file-scope __device__ array that every GPU loading the library holds
// until the process exits.
//
// Work split (deterministic, no atomics): the nonzeros are cut into chunks of kChunkNnz; the CTA
// of a chunk owns the rows that start inside it and sums each owned row up to the chunk's end;
// a row that runs past its chunk is continued by the following CTAs, each writing one carry
// (row, partial sum of its slice) to the scratch; a second kernel adds every carried row's
// partials in chunk order. Same values as the engine's load-balanced tile SpMV up to summation
// order (round-off).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/sg_pdlp.h"

namespace sg {
void set_last_error(const char* message);  // sg_capi.cpp
}  // namespace sg

namespace {

constexpr int kChunkNnz = 2048;
constexpr int kThreads = 256;
constexpr int kMaxChunks = SG_SPMV_NOALLOC_MAX_CHUNKS;

struct Carry {
  double value;  // partial sum of the chunk's slice of the carried row
  int row;       // -1: no carried row in this chunk
  int pad;
};

// The scratch: one carry per chunk (16 bytes each).
static __device__ __align__(256) Carry g_noalloc_carry[kMaxChunks];

// First index r in [lo, hi) with ptr[r] >= key (hi when none).
__device__ __forceinline__ int lower_bound_ptr(const int* ptr, int lo, int hi, long long key) {
  while (lo < hi) {
    const int mid = lo + ((hi - lo) >> 1);
    if (static_cast<long long>(ptr[mid]) < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// One CTA per chunk [k0, k1): owned rows (start in the chunk; the last chunk also owns the
// trailing empty rows) by one warp each, plus the carry of the row that enters the chunk.
__global__ void __launch_bounds__(kThreads) spmv_chunk_kernel(int m, const int* __restrict__ ptr,
                                                              const int* __restrict__ idx,
                                                              const double* __restrict__ val,
                                                              const double* __restrict__ x,
                                                              double* __restrict__ y,
                                                              Carry* __restrict__ carry,
                                                              int chunks) {
  const int c = blockIdx.x;
  // The matrix's own nonzero count decides the chunk bounds: chunks past it are empty, and the
  // last chunk runs to its end (owned rows and the carried row alike), so a grid sized from a
  // count that differs from row_ptr[m] still writes every row once.
  const long long nnz = ptr[m];
  const bool last_chunk = c == chunks - 1;
  long long k0 = static_cast<long long>(c) * kChunkNnz;
  if (k0 > nnz) k0 = nnz;
  const long long k1 = last_chunk ? nnz : (k0 + kChunkNnz < nnz ? k0 + kChunkNnz : nnz);
  // Rows starting in [k0, k1); the last chunk takes every row starting at or after k0.
  const int r_begin = c == 0 ? 0 : lower_bound_ptr(ptr, 0, m, k0);
  const int r_end = last_chunk ? m : lower_bound_ptr(ptr, 0, m, k1);
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  constexpr int kWarps = kThreads / 32;
  for (int r = r_begin + warp; r < r_end; r += kWarps) {
    const long long b = ptr[r];
    long long e = ptr[r + 1];
    if (e > k1 && !last_chunk) e = k1;
    double s = 0.0;
    for (long long q = b + lane; q < e; q += 32) s += val[q] * x[idx[q]];
    s = warp_sum(s);
    if (lane == 0) y[r] = s;
  }
  // The row entering this chunk from an earlier one (it started before k0).
  if (threadIdx.x < 32) {
    int row = -1;
    double s = 0.0;
    if (c > 0 && r_begin > 0) {
      const int r = r_begin - 1;
      const long long e_row = ptr[r + 1];
      if (e_row > k0) {
        row = r;
        const long long e = e_row < k1 ? e_row : k1;
        for (long long q = k0 + lane; q < e; q += 32) s += val[q] * x[idx[q]];
      }
    }
    s = warp_sum(s);
    if (lane == 0) {
      carry[c].row = row;
      carry[c].value = s;
    }
  }
}

// Adds the carried partials of each row to its owner's sum, in chunk order (one thread per
// chunk; the first chunk of a run of equal rows does the run).
__global__ void spmv_carry_kernel(double* __restrict__ y, const Carry* __restrict__ carry,
                                  int chunks) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= chunks) return;
  const int row = carry[c].row;
  if (row < 0) return;
  if (c > 0 && carry[c - 1].row == row) return;
  double s = y[row];
  for (int g = c; g < chunks && carry[g].row == row; ++g) s += carry[g].value;
  y[row] = s;
}

// The scratch's device address, looked up once per device (cudaGetSymbolAddress, with that
// device current). A cudaDeviceReset of the device unloads the module and makes the address
// stale; sg_spmv_noalloc is not meant to be called after one.
std::mutex g_setup_mutex;
Carry* g_carry_ptr[64] = {nullptr};

int scratch_for_current_device(Carry** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SG_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_carry_ptr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_carry);
    if (e != cudaSuccess || p == nullptr) return SG_ERR_CUDA;
    g_carry_ptr[dev] = static_cast<Carry*>(p);
  }
  *out = g_carry_ptr[dev];
  return SG_OK;
}

int refuse(int code, const char* message) {
  sg::set_last_error(message);
  return code;
}

}  // namespace

extern "C" int sg_spmv_noalloc(int m, long long nnz, const int* d_row_ptr, const int* d_col_idx,
                               const double* d_val, const double* d_x, double* d_y,
                               void* stream) {
  if (m < 0 || nnz < 0 || d_row_ptr == nullptr || d_y == nullptr ||
      (nnz > 0 && (d_col_idx == nullptr || d_val == nullptr || d_x == nullptr))) {
    return refuse(SG_ERR_INVALID_ARGUMENT, "sg_spmv_noalloc: negative size or NULL pointer");
  }
  const long long chunks_ll = nnz == 0 ? 1 : (nnz + kChunkNnz - 1) / kChunkNnz;
  if (chunks_ll > kMaxChunks) {
    return refuse(SG_ERR_TOO_LARGE,
                  "sg_spmv_noalloc: more nonzeros than its fixed scratch covers "
                  "(SG_SPMV_NOALLOC_MAX_CHUNKS * 2048)");
  }
  if (m == 0) return SG_OK;
  Carry* carry = nullptr;
  const int rc = scratch_for_current_device(&carry);
  if (rc != SG_OK) return refuse(rc, "sg_spmv_noalloc: no scratch address on this device");
  int chunks = static_cast<int>(chunks_ll);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // cudaLaunchKernel reports the error of this launch only (the caller's earlier errors stay
  // where they are).
  const int* rp = d_row_ptr;
  const int* ci = d_col_idx;
  const double* va = d_val;
  const double* xv = d_x;
  double* yv = d_y;
  void* chunk_args[] = {&m, &rp, &ci, &va, &xv, &yv, &carry, &chunks};
  cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(spmv_chunk_kernel),
                                   dim3(chunks), dim3(kThreads), chunk_args, 0, s);
  if (e == cudaSuccess) {
    const Carry* cc = carry;
    void* carry_args[] = {&yv, &cc, &chunks};
    e = cudaLaunchKernel(reinterpret_cast<const void*>(spmv_carry_kernel),
                         dim3((chunks + 255) / 256), dim3(256), carry_args, 0, s);
  }
  if (e != cudaSuccess) {
    sg::set_last_error(cudaGetErrorString(e));
    return SG_ERR_CUDA;
  }
  return SG_OK;
}
