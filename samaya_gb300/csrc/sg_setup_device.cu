// samaya's model setup on the device: the power-of-two scaling (compute_scaling, reference
// src/linalg/scaling.cpp:79-149: geometric-mean passes, then equilibration, factors rounded to
// powers of two), the computational form (make_problem, src/lp/lp_solver.cpp:28-51) and the
// row-major copy of A the engine iterates with (the transpose, src/linalg/sparse_matrix.cpp:
// 48-78). Every value is the one the host code gives (sg_scale_model, sg_csc_to_csr): the
// extremes are min / max (exact in any order), the scale factors come from the same IEEE
// products, square roots and quotients, and the few factors whose nearest power of two
// depends on the last bit of a logarithm are finished on the host with the host's own code.
//
// The transpose is a stable sort of the nonzeros by row (CUB's radix sort, a CUDA toolkit
// library, run once per problem); everything else is the kernels below.
#include "sg_setup_device.cuh"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "../../include/sg_pdlp.h"
#include "sg_transpose.h"

namespace sg {

namespace {

constexpr int kT = 256;
constexpr int kMaxAmbiguous = 4096;

int grid_for(long long count) {
  const long long g = (count + kT - 1) / kT;
  return static_cast<int>(std::max<long long>(1, std::min<long long>(g, 152LL * 16)));
}

__device__ __forceinline__ unsigned long long key_of(double v) {
  return static_cast<unsigned long long>(__double_as_longlong(v));
}

__device__ __forceinline__ double clamp_scale(double v) {
  return fmin(fmax(v, 0x1p-40), 0x1p40);
}

// The column of every nonzero (thread per column).
template <typename P>
__global__ void column_of_kernel(int n, const P* __restrict__ cp, int32_t* __restrict__ col) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    for (P p = cp[j]; p < cp[j + 1]; ++p) col[p] = j;
  }
}

// flags[0]: a row index out of range; flags[1]: a value not finite.
__global__ void check_kernel(int m, long long nnz, const int32_t* __restrict__ row,
                             const double* __restrict__ val, int* flags) {
  for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < nnz;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    if (row[p] < 0 || row[p] >= m) flags[0] = 1;
    if (!isfinite(val[p])) flags[1] = 1;
  }
}

template <typename T>
__global__ void fill_kernel(T* p, long long count, T v) {
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < count;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    p[k] = v;
  }
}

// Smallest and largest |a_ij| r_i c_j over the nonzeros (non-negative doubles order as their
// bit patterns): ext[0] min, ext[1] max.
__global__ void spread_kernel(long long nnz, const int32_t* __restrict__ row,
                              const int32_t* __restrict__ col, const double* __restrict__ val,
                              const double* __restrict__ r, const double* __restrict__ c,
                              unsigned long long* ext) {
  unsigned long long lo = key_of(INFINITY), hi = 0ull;
  for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < nnz;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    const unsigned long long k = key_of(fabs(val[p]) * r[row[p]] * c[col[p]]);
    lo = k < lo ? k : lo;
    hi = k > hi ? k : hi;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long l2 = __shfl_down_sync(0xffffffffu, lo, o);
    const unsigned long long h2 = __shfl_down_sync(0xffffffffu, hi, o);
    lo = l2 < lo ? l2 : lo;
    hi = h2 > hi ? h2 : hi;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&ext[0], lo);
    atomicMax(&ext[1], hi);
  }
}

// Row extremes of |a_ij| c_j (rmin, rmax as bit patterns). The lanes of a warp that share a
// row combine first, so a row present in most columns does not serialise on its atomics.
__global__ void row_extremes_kernel(long long nnz, const int32_t* __restrict__ row,
                                    const int32_t* __restrict__ col,
                                    const double* __restrict__ val, const double* __restrict__ c,
                                    unsigned long long* rmin, unsigned long long* rmax) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const long long first = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  // Every lane runs the same number of rounds (warp-uniform bound) so the match is complete.
  const long long warp_base = first - (threadIdx.x & 31);
  for (long long base = warp_base; base < nnz; base += stride) {
    const long long p = base + (threadIdx.x & 31);
    const bool live = p < nnz;
    const int i = live ? row[p] : -1;
    const unsigned long long k = live ? key_of(fabs(val[p]) * c[col[p]]) : 0ull;
    const unsigned mask = __match_any_sync(0xffffffffu, i);
    unsigned long long lo = live ? k : key_of(INFINITY), hi = k;
    for (unsigned mm = mask; mm != 0u; mm &= mm - 1u) {
      const int src = __ffs(mm) - 1;
      const unsigned long long o = __shfl_sync(mask, k, src);
      lo = o < lo ? o : lo;
      hi = o > hi ? o : hi;
    }
    if (live && (threadIdx.x & 31) == __ffs(mask) - 1) {
      atomicMin(&rmin[i], lo);
      atomicMax(&rmax[i], hi);
    }
  }
}

// Geometric pass, rows: r_i = clamp(1 / sqrt(min * max)) where the row has a nonzero.
__global__ void row_geometric_kernel(int m, const unsigned long long* __restrict__ rmin,
                                     const unsigned long long* __restrict__ rmax, double* r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const double hi = __longlong_as_double(static_cast<long long>(rmax[i]));
    const double lo = __longlong_as_double(static_cast<long long>(rmin[i]));
    if (hi > 0.0) r[i] = clamp_scale(1.0 / sqrt(lo * hi));
  }
}

// Equilibration, rows: r_i = clamp(1 / max) where the row has a nonzero.
__global__ void row_equilibrate_kernel(int m, const unsigned long long* __restrict__ rmax,
                                       double* r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const double hi = __longlong_as_double(static_cast<long long>(rmax[i]));
    if (hi > 0.0) r[i] = clamp_scale(1.0 / hi);
  }
}

// Columns (thread per column): geometric pass c_j = clamp(1 / sqrt(min * max)) or
// equilibration c_j = clamp(1 / max) of |a_ij| r_i.
__global__ void column_scale_kernel(int n, const int64_t* __restrict__ cp,
                                    const int32_t* __restrict__ row,
                                    const double* __restrict__ val, const double* __restrict__ r,
                                    double* c, int geometric) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double lo = INFINITY, hi = 0.0;
    for (int64_t p = cp[j]; p < cp[j + 1]; ++p) {
      const double v = fabs(val[p]) * r[row[p]];
      lo = fmin(lo, v);
      hi = fmax(hi, v);
    }
    if (hi > 0.0) c[j] = clamp_scale(geometric ? 1.0 / sqrt(lo * hi) : 1.0 / hi);
  }
}

// Nearest power of two, 2^lround(log2 v) (1 for a value that is not positive and finite).
// Where log2 v lies within 1e-9 of a half-integer the rounding could depend on the last bit of
// the logarithm: the entry is listed for the host (amb_count, amb_index) and left as is.
__global__ void power_of_two_kernel(int count, double* f, int* amb_count, int* amb_index,
                                    int index_offset) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const double v = f[k];
    if (!(v > 0.0) || !isfinite(v)) {
      f[k] = 1.0;
      continue;
    }
    const double L = log2(v);
    const double frac = L - floor(L);
    if (fabs(frac - 0.5) < 1e-9) {
      const int slot = atomicAdd(amb_count, 1);
      if (slot < kMaxAmbiguous) amb_index[slot] = index_offset + k;
      continue;
    }
    f[k] = ldexp(1.0, static_cast<int>(llround(L)));
  }
}

// make_problem's matrix: a_ij r_i c_j, zeros dropped (flag per nonzero, then the scatter to the
// exclusive-scan positions).
__global__ void product_flags_kernel(long long nnz, const int32_t* __restrict__ row,
                                     const int32_t* __restrict__ col,
                                     const double* __restrict__ val, const double* __restrict__ r,
                                     const double* __restrict__ c, int* keep) {
  for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < nnz;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    keep[p] = val[p] * r[row[p]] * c[col[p]] != 0.0 ? 1 : 0;
  }
}

__global__ void product_scatter_kernel(long long nnz, const int32_t* __restrict__ row,
                                       const int32_t* __restrict__ col,
                                       const double* __restrict__ val,
                                       const double* __restrict__ r, const double* __restrict__ c,
                                       const int* __restrict__ pos, int32_t* lp_row,
                                       double* lp_val) {
  for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < nnz;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double v = val[p] * r[row[p]] * c[col[p]];
    if (v != 0.0) {
      lp_row[pos[p]] = row[p];
      lp_val[pos[p]] = v;
    }
  }
}

// Column starts of the scaled matrix: the scan position at each model column start.
__global__ void lp_colptr_kernel(int n, const int64_t* __restrict__ cp, const int* __restrict__ pos,
                                 int64_t* lp_cp64, int* lp_cp32) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j <= n; j += gridDim.x * blockDim.x) {
    const int v = pos[cp[j]];
    lp_cp64[j] = v;
    lp_cp32[j] = v;
  }
}

// make_problem's vectors: cost sense c_j C_j (0 for the logicals), bounds l_j / C_j and
// row bounds times R_i.
__global__ void problem_vectors_kernel(int n, int m, double sense, const double* __restrict__ obj,
                                       const double* __restrict__ cl, const double* __restrict__ cu,
                                       const double* __restrict__ rl, const double* __restrict__ ru,
                                       const double* __restrict__ r, const double* __restrict__ c,
                                       double* cost, double* lower, double* upper) {
  const int nt = n + m;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
    if (k < n) {
      cost[k] = sense * obj[k] * c[k];
      lower[k] = cl[k] / c[k];
      upper[k] = cu[k] / c[k];
    } else {
      const int i = k - n;
      cost[k] = 0.0;
      lower[k] = rl[i] * r[i];
      upper[k] = ru[i] * r[i];
    }
  }
}

__global__ void iota_kernel(int count, int* v) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    v[k] = k;
  }
}

// Row-major copy from the nonzeros sorted by row (stable: column order kept inside a row).
__global__ void gather_rows_kernel(int nnz, const int* __restrict__ perm,
                                   const int32_t* __restrict__ lp_col,
                                   const double* __restrict__ lp_val, int* kidx, double* kval) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) {
    const int p = perm[k];
    kidx[k] = lp_col[p];
    kval[k] = lp_val[p];
  }
}

// Row starts: the first sorted position of each row (binary search over the sorted rows).
__global__ void row_starts_kernel(int m, int nnz, const int* __restrict__ rows_sorted, int* kptr) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= m; i += gridDim.x * blockDim.x) {
    int lo = 0, hi = nnz;
    while (lo < hi) {
      const int mid = lo + ((hi - lo) >> 1);
      if (rows_sorted[mid] < i) lo = mid + 1; else hi = mid;
    }
    kptr[i] = lo;
  }
}

// Inert rows: no nonzeros, and a logical with no cost and 0 within its bounds.
__global__ void inert_rows_kernel(int m, int n, const int* __restrict__ kptr,
                                  const double* __restrict__ cost,
                                  const double* __restrict__ lower,
                                  const double* __restrict__ upper, char* inert) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    inert[i] = kptr[i + 1] == kptr[i] && cost[n + i] == 0.0 && lower[n + i] <= 0.0 &&
               upper[n + i] >= 0.0;
  }
}

// The host's nearest power of two (sg_scale_model's own rule).
double host_power_of_two(double v) {
  if (!(v > 0.0) || !std::isfinite(v)) return 1.0;
  return std::ldexp(1.0, static_cast<int>(std::lround(std::log2(v))));
}

// Device buffers of one setup, freed on destruction.
struct Buffers {
  std::vector<void*> owned;
  ~Buffers() {
    for (void* p : owned) cudaFree(p);
  }
  template <typename T>
  cudaError_t get(T** p, size_t count) {
    *p = nullptr;
    const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) owned.push_back(*p);
    return e;
  }
};

// The model's LpProblem in device memory.
struct DeviceSetup {
  Buffers buf;
  int m = 0, n = 0;
  long long nnz_in = 0;
  long long nnz = 0;        // after zeros are dropped
  int64_t* lp_cp64 = nullptr;
  int* lp_cp32 = nullptr;
  int32_t* lp_row = nullptr;
  double* lp_val = nullptr;
  double* cost = nullptr;
  double* lower = nullptr;
  double* upper = nullptr;
  double* r = nullptr;
  double* c = nullptr;
};

#define SG_DEV(call)                                                       \
  do {                                                                     \
    const cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) {                                               \
      if (err) *err = std::string("device setup: ") + cudaGetErrorString(e_); \
      return e_ == cudaErrorMemoryAllocation ? kErrOutOfMemory : kErrCuda; \
    }                                                                      \
  } while (0)

int check_host(const ModelView& mv, std::string* err) {
  if (mv.m < 0 || mv.n < 0 || mv.colptr == nullptr || mv.obj == nullptr ||
      mv.col_lower == nullptr || mv.col_upper == nullptr ||
      (mv.m > 0 && (mv.row_lower == nullptr || mv.row_upper == nullptr))) {
    if (err) *err = "invalid argument";
    return kErrInvalidArgument;
  }
  if (mv.colptr[0] != 0) {
    if (err) *err = "column starts must begin at 0";
    return kErrInvalidArgument;
  }
  for (int j = 0; j < mv.n; ++j) {
    if (mv.colptr[j + 1] < mv.colptr[j]) {
      if (err) *err = "column starts must not decrease";
      return kErrInvalidArgument;
    }
  }
  const long long nnz = mv.colptr[mv.n];
  if (nnz >= static_cast<long long>(std::numeric_limits<int>::max()) ||
      static_cast<long long>(mv.n) + mv.m >= std::numeric_limits<int>::max()) {
    if (err) *err = "matrix too large for 32-bit offsets";
    return kErrTooLarge;
  }
  if (nnz > 0 && (mv.rowidx == nullptr || mv.val == nullptr)) {
    if (err) *err = "null matrix arrays";
    return kErrInvalidArgument;
  }
  for (int j = 0; j < mv.n; ++j) {
    if (!std::isfinite(mv.obj[j]) || std::isnan(mv.col_lower[j]) || std::isnan(mv.col_upper[j])) {
      if (err) *err = "cost or bound not valid";
      return kErrInvalidArgument;
    }
  }
  for (int i = 0; i < mv.m; ++i) {
    if (std::isnan(mv.row_lower[i]) || std::isnan(mv.row_upper[i])) {
      if (err) *err = "row bound not valid";
      return kErrInvalidArgument;
    }
  }
  return kOk;
}

// compute_scaling + make_problem on the device (see the file comment).
int build_problem(const ModelView& mv, cudaStream_t s, DeviceSetup* d, std::string* err) {
  int rc = check_host(mv, err);
  if (rc != kOk) return rc;
  const int m = mv.m, n = mv.n;
  const long long nnz = mv.colptr[n];
  d->m = m;
  d->n = n;
  d->nnz_in = nnz;
  Buffers& b = d->buf;
  int64_t* cp = nullptr;
  int32_t* row = nullptr;
  int32_t* col = nullptr;
  double* val = nullptr;
  SG_DEV(b.get(&cp, static_cast<size_t>(n) + 1));
  SG_DEV(b.get(&row, static_cast<size_t>(nnz)));
  SG_DEV(b.get(&col, static_cast<size_t>(nnz)));
  SG_DEV(b.get(&val, static_cast<size_t>(nnz)));
  SG_DEV(cudaMemcpyAsync(cp, mv.colptr, (static_cast<size_t>(n) + 1) * sizeof(int64_t),
                         cudaMemcpyHostToDevice, s));
  if (nnz > 0) {
    SG_DEV(cudaMemcpyAsync(row, mv.rowidx, static_cast<size_t>(nnz) * sizeof(int32_t),
                           cudaMemcpyHostToDevice, s));
    SG_DEV(cudaMemcpyAsync(val, mv.val, static_cast<size_t>(nnz) * sizeof(double),
                           cudaMemcpyHostToDevice, s));
  }
  int* flags = nullptr;
  unsigned long long* ext = nullptr;
  int* amb = nullptr;  // [0] count, then the indices
  SG_DEV(b.get(&flags, 2));
  SG_DEV(b.get(&ext, 2));
  SG_DEV(b.get(&amb, 1 + kMaxAmbiguous));
  SG_DEV(cudaMemsetAsync(flags, 0, 2 * sizeof(int), s));
  if (n > 0) column_of_kernel<<<grid_for(n), kT, 0, s>>>(n, cp, col);
  if (nnz > 0) check_kernel<<<grid_for(nnz), kT, 0, s>>>(m, nnz, row, val, flags);
  {
    int hflags[2] = {0, 0};
    SG_DEV(cudaGetLastError());
    SG_DEV(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, s));
    SG_DEV(cudaStreamSynchronize(s));
    if (hflags[0] || hflags[1]) {
      if (err) *err = hflags[0] ? "row index out of range" : "matrix value not finite";
      return kErrInvalidArgument;
    }
  }
  SG_DEV(b.get(&d->r, static_cast<size_t>(m)));
  SG_DEV(b.get(&d->c, static_cast<size_t>(n)));
  double* r = d->r;
  double* c = d->c;
  if (m > 0) fill_kernel<double><<<grid_for(m), kT, 0, s>>>(r, m, 1.0);
  if (n > 0) fill_kernel<double><<<grid_for(n), kT, 0, s>>>(c, n, 1.0);
  if (nnz > 0) {
    double* r_prev = nullptr;
    double* c_prev = nullptr;
    unsigned long long* rmin = nullptr;
    unsigned long long* rmax = nullptr;
    SG_DEV(b.get(&r_prev, static_cast<size_t>(m)));
    SG_DEV(b.get(&c_prev, static_cast<size_t>(n)));
    SG_DEV(b.get(&rmin, static_cast<size_t>(m)));
    SG_DEV(b.get(&rmax, static_cast<size_t>(m)));
    const unsigned long long inf_key = 0x7ff0000000000000ull;
    auto spread = [&](double* out) -> int {
      unsigned long long init[2] = {inf_key, 0ull};
      SG_DEV(cudaMemcpyAsync(ext, init, sizeof(init), cudaMemcpyHostToDevice, s));
      spread_kernel<<<grid_for(nnz), kT, 0, s>>>(nnz, row, col, val, r, c, ext);
      SG_DEV(cudaGetLastError());
      unsigned long long h[2];
      SG_DEV(cudaMemcpyAsync(h, ext, sizeof(h), cudaMemcpyDeviceToHost, s));
      SG_DEV(cudaStreamSynchronize(s));
      double lo, hi;
      memcpy(&lo, &h[0], sizeof(double));
      memcpy(&hi, &h[1], sizeof(double));
      *out = hi > 0.0 ? hi / lo : 1.0;
      return kOk;
    };
    auto row_extremes = [&]() {
      fill_kernel<unsigned long long><<<grid_for(m), kT, 0, s>>>(rmin, m, inf_key);
      fill_kernel<unsigned long long><<<grid_for(m), kT, 0, s>>>(rmax, m, 0ull);
      row_extremes_kernel<<<grid_for(nnz), kT, 0, s>>>(nnz, row, col, val, c, rmin, rmax);
    };
    // Geometric-mean passes: at most 10, stop when a pass gains less than 10% or worsens the
    // spread (restoring the factors before it).
    double ratio = 0.0;
    rc = spread(&ratio);
    if (rc != kOk) return rc;
    for (int pass = 0; pass < 10 && ratio > 1.0; ++pass) {
      SG_DEV(cudaMemcpyAsync(r_prev, r, static_cast<size_t>(m) * sizeof(double),
                             cudaMemcpyDeviceToDevice, s));
      SG_DEV(cudaMemcpyAsync(c_prev, c, static_cast<size_t>(n) * sizeof(double),
                             cudaMemcpyDeviceToDevice, s));
      row_extremes();
      row_geometric_kernel<<<grid_for(m), kT, 0, s>>>(m, rmin, rmax, r);
      column_scale_kernel<<<grid_for(n), kT, 0, s>>>(n, cp, row, val, r, c, 1);
      double next = 0.0;
      rc = spread(&next);
      if (rc != kOk) return rc;
      if (next > ratio) {
        SG_DEV(cudaMemcpyAsync(r, r_prev, static_cast<size_t>(m) * sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
        SG_DEV(cudaMemcpyAsync(c, c_prev, static_cast<size_t>(n) * sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
        break;
      }
      const bool small_gain = next > 0.9 * ratio;
      ratio = next;
      if (small_gain) break;
    }
    // Equilibration: every row and then every column maximum to about 1.
    row_extremes();
    row_equilibrate_kernel<<<grid_for(m), kT, 0, s>>>(m, rmax, r);
    column_scale_kernel<<<grid_for(n), kT, 0, s>>>(n, cp, row, val, r, c, 0);
    // Powers of two; ambiguous entries finished on the host.
    SG_DEV(cudaMemsetAsync(amb, 0, sizeof(int), s));
    if (m > 0) power_of_two_kernel<<<grid_for(m), kT, 0, s>>>(m, r, amb, amb + 1, 0);
    if (n > 0) power_of_two_kernel<<<grid_for(n), kT, 0, s>>>(n, c, amb, amb + 1, m);
    SG_DEV(cudaGetLastError());
    int count = 0;
    SG_DEV(cudaMemcpyAsync(&count, amb, sizeof(int), cudaMemcpyDeviceToHost, s));
    SG_DEV(cudaStreamSynchronize(s));
    if (count > kMaxAmbiguous) {
      // More than the list holds (not met in practice): every factor of both kinds that is
      // not yet a power of two is finished on the host.
      std::vector<double> hr(static_cast<size_t>(m)), hc(static_cast<size_t>(n));
      SG_DEV(cudaMemcpy(hr.data(), r, hr.size() * sizeof(double), cudaMemcpyDeviceToHost));
      SG_DEV(cudaMemcpy(hc.data(), c, hc.size() * sizeof(double), cudaMemcpyDeviceToHost));
      for (double& f : hr) f = host_power_of_two(f);
      for (double& f : hc) f = host_power_of_two(f);
      SG_DEV(cudaMemcpy(r, hr.data(), hr.size() * sizeof(double), cudaMemcpyHostToDevice));
      SG_DEV(cudaMemcpy(c, hc.data(), hc.size() * sizeof(double), cudaMemcpyHostToDevice));
    } else if (count > 0) {
      std::vector<int> idx(static_cast<size_t>(count));
      SG_DEV(cudaMemcpy(idx.data(), amb + 1, idx.size() * sizeof(int), cudaMemcpyDeviceToHost));
      for (int k : idx) {
        double* p = k < m ? r + k : c + (k - m);
        double v = 0.0;
        SG_DEV(cudaMemcpy(&v, p, sizeof(double), cudaMemcpyDeviceToHost));
        v = host_power_of_two(v);
        SG_DEV(cudaMemcpy(p, &v, sizeof(double), cudaMemcpyHostToDevice));
      }
    }
  }
  // make_problem: the scaled matrix without zeros, and the vectors.
  int* keep = nullptr;
  int* pos = nullptr;
  SG_DEV(b.get(&keep, static_cast<size_t>(nnz) + 1));
  SG_DEV(b.get(&pos, static_cast<size_t>(nnz) + 1));
  SG_DEV(cudaMemsetAsync(keep, 0, (static_cast<size_t>(nnz) + 1) * sizeof(int), s));
  if (nnz > 0) product_flags_kernel<<<grid_for(nnz), kT, 0, s>>>(nnz, row, col, val, r, c, keep);
  {
    size_t temp = 0;
    SG_DEV(cub::DeviceScan::ExclusiveSum(nullptr, temp, keep, pos, static_cast<int>(nnz) + 1, s));
    void* tmp = nullptr;
    SG_DEV(b.get(reinterpret_cast<char**>(&tmp), temp));
    SG_DEV(cub::DeviceScan::ExclusiveSum(tmp, temp, keep, pos, static_cast<int>(nnz) + 1, s));
  }
  int kept = 0;
  SG_DEV(cudaMemcpyAsync(&kept, pos + nnz, sizeof(int), cudaMemcpyDeviceToHost, s));
  SG_DEV(cudaStreamSynchronize(s));
  d->nnz = kept;
  SG_DEV(b.get(&d->lp_cp64, static_cast<size_t>(n) + 1));
  SG_DEV(b.get(&d->lp_cp32, static_cast<size_t>(n) + 1));
  SG_DEV(b.get(&d->lp_row, static_cast<size_t>(kept)));
  SG_DEV(b.get(&d->lp_val, static_cast<size_t>(kept)));
  if (nnz > 0) {
    product_scatter_kernel<<<grid_for(nnz), kT, 0, s>>>(nnz, row, col, val, r, c, pos, d->lp_row,
                                                        d->lp_val);
  }
  lp_colptr_kernel<<<grid_for(static_cast<long long>(n) + 1), kT, 0, s>>>(n, cp, pos, d->lp_cp64,
                                                                          d->lp_cp32);
  const size_t nt = static_cast<size_t>(n) + m;
  double* vec_in = nullptr;  // obj, col_lower, col_upper (n each), row_lower, row_upper (m each)
  SG_DEV(b.get(&vec_in, 3 * static_cast<size_t>(n) + 2 * static_cast<size_t>(m)));
  SG_DEV(cudaMemcpyAsync(vec_in, mv.obj, n * sizeof(double), cudaMemcpyHostToDevice, s));
  SG_DEV(cudaMemcpyAsync(vec_in + n, mv.col_lower, n * sizeof(double), cudaMemcpyHostToDevice, s));
  SG_DEV(cudaMemcpyAsync(vec_in + 2 * static_cast<size_t>(n), mv.col_upper, n * sizeof(double),
                         cudaMemcpyHostToDevice, s));
  if (m > 0) {
    SG_DEV(cudaMemcpyAsync(vec_in + 3 * static_cast<size_t>(n), mv.row_lower, m * sizeof(double),
                           cudaMemcpyHostToDevice, s));
    SG_DEV(cudaMemcpyAsync(vec_in + 3 * static_cast<size_t>(n) + m, mv.row_upper,
                           m * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  SG_DEV(b.get(&d->cost, nt));
  SG_DEV(b.get(&d->lower, nt));
  SG_DEV(b.get(&d->upper, nt));
  if (nt > 0) {
    problem_vectors_kernel<<<grid_for(static_cast<long long>(nt)), kT, 0, s>>>(
        n, m, mv.maximize ? -1.0 : 1.0, vec_in, vec_in + n, vec_in + 2 * static_cast<size_t>(n),
        vec_in + 3 * static_cast<size_t>(n), vec_in + 3 * static_cast<size_t>(n) + m, r, c,
        d->cost, d->lower, d->upper);
  }
  SG_DEV(cudaGetLastError());
  SG_DEV(cudaStreamSynchronize(s));
  return kOk;
}

}  // namespace

int scale_model_device(const ModelView& mv, int64_t* lp_colptr, int32_t* lp_rowidx,
                       double* lp_val, double* cost, double* lower, double* upper,
                       double* col_scale, double* row_scale, int64_t* lp_nnz, std::string* err) {
  if (lp_colptr == nullptr || cost == nullptr || lower == nullptr || upper == nullptr ||
      col_scale == nullptr || lp_nnz == nullptr || (mv.m > 0 && row_scale == nullptr)) {
    if (err) *err = "invalid argument";
    return kErrInvalidArgument;
  }
  if (device_info(nullptr, nullptr, nullptr, 0) != kOk) {
    if (err) *err = "no sm_103 GPU";
    return kErrNoDevice;
  }
  cudaStream_t s = nullptr;
  SG_DEV(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  int rc;
  {
    DeviceSetup d;
    rc = build_problem(mv, s, &d, err);
    if (rc == kOk) {
      const size_t n = static_cast<size_t>(mv.n), m = static_cast<size_t>(mv.m);
      const size_t nt = n + m;
      cudaError_t e = cudaMemcpy(lp_colptr, d.lp_cp64, (n + 1) * sizeof(int64_t),
                                 cudaMemcpyDeviceToHost);
      if (e == cudaSuccess && d.nnz > 0) {
        e = cudaMemcpy(lp_rowidx, d.lp_row, static_cast<size_t>(d.nnz) * sizeof(int32_t),
                       cudaMemcpyDeviceToHost);
      }
      if (e == cudaSuccess && d.nnz > 0) {
        e = cudaMemcpy(lp_val, d.lp_val, static_cast<size_t>(d.nnz) * sizeof(double),
                       cudaMemcpyDeviceToHost);
      }
      if (e == cudaSuccess) e = cudaMemcpy(cost, d.cost, nt * sizeof(double), cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy(lower, d.lower, nt * sizeof(double), cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy(upper, d.upper, nt * sizeof(double), cudaMemcpyDeviceToHost);
      if (e == cudaSuccess && n > 0) {
        e = cudaMemcpy(col_scale, d.c, n * sizeof(double), cudaMemcpyDeviceToHost);
      }
      if (e == cudaSuccess && m > 0) {
        e = cudaMemcpy(row_scale, d.r, m * sizeof(double), cudaMemcpyDeviceToHost);
      }
      if (e != cudaSuccess) {
        if (err) *err = std::string("device setup: ") + cudaGetErrorString(e);
        rc = kErrCuda;
      }
      *lp_nnz = d.nnz;
    }
  }
  cudaStreamDestroy(s);
  return rc;
}

int create_engine_from_model(Engine** out, const ModelView& mv, const Options& opt,
                             double* col_scale, double* row_scale, std::string* err) {
  *out = nullptr;
  if (device_info(nullptr, nullptr, nullptr, 0) != kOk) {
    if (err) *err = "no sm_103 GPU";
    return kErrNoDevice;
  }
  cudaStream_t s = nullptr;
  SG_DEV(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  int rc;
  {
    DeviceSetup d;
    rc = build_problem(mv, s, &d, err);
    Buffers t;
    DeviceLp lp;
    if (rc == kOk) {
      const int m = mv.m, n = mv.n, nnz = static_cast<int>(d.nnz);
      lp.m = m;
      lp.n = n;
      lp.nnz = nnz;
      // The row-major copy: a stable sort of the nonzeros by row.
      int* col = nullptr;
      int* keys = nullptr;
      int* perm_in = nullptr;
      int* perm = nullptr;
      int* kptr = nullptr;
      int* kidx = nullptr;
      double* kval = nullptr;
      cudaError_t e = cudaSuccess;
      auto step = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
      };
      step(t.get(&col, static_cast<size_t>(nnz)));
      step(t.get(&keys, static_cast<size_t>(nnz)));
      step(t.get(&perm_in, static_cast<size_t>(nnz)));
      step(t.get(&perm, static_cast<size_t>(nnz)));
      step(t.get(&kptr, static_cast<size_t>(m) + 1));
      step(t.get(&kidx, static_cast<size_t>(nnz)));
      step(t.get(&kval, static_cast<size_t>(nnz)));
      if (e == cudaSuccess && n > 0) {
        column_of_kernel<<<grid_for(n), kT, 0, s>>>(n, d.lp_cp64, col);
      }
      if (e == cudaSuccess && nnz > 0) {
        iota_kernel<<<grid_for(nnz), kT, 0, s>>>(nnz, perm_in);
        int bits = 1;
        while (bits < 31 && (1LL << bits) <= m) ++bits;
        size_t temp = 0;
        step(cub::DeviceRadixSort::SortPairs(nullptr, temp, d.lp_row, keys, perm_in, perm, nnz,
                                             0, bits, s));
        char* tmp = nullptr;
        step(t.get(&tmp, temp));
        step(cub::DeviceRadixSort::SortPairs(tmp, temp, d.lp_row, keys, perm_in, perm, nnz, 0,
                                             bits, s));
        gather_rows_kernel<<<grid_for(nnz), kT, 0, s>>>(nnz, perm, col, d.lp_val, kidx, kval);
      }
      char* inert = nullptr;
      step(t.get(&inert, static_cast<size_t>(m)));
      if (e == cudaSuccess) {
        row_starts_kernel<<<grid_for(static_cast<long long>(m) + 1), kT, 0, s>>>(m, nnz, keys,
                                                                                kptr);
        if (m > 0) {
          inert_rows_kernel<<<grid_for(m), kT, 0, s>>>(m, n, kptr, d.cost, d.lower, d.upper,
                                                       inert);
        }
        step(cudaGetLastError());
      }
      lp.kptr_host.resize(static_cast<size_t>(m) + 1);
      lp.tptr_host.resize(static_cast<size_t>(n) + 1);
      lp.row_inert.resize(static_cast<size_t>(m));
      if (e == cudaSuccess) {
        step(cudaMemcpyAsync(lp.kptr_host.data(), kptr, lp.kptr_host.size() * sizeof(int),
                             cudaMemcpyDeviceToHost, s));
        step(cudaMemcpyAsync(lp.tptr_host.data(), d.lp_cp32, lp.tptr_host.size() * sizeof(int),
                             cudaMemcpyDeviceToHost, s));
        if (m > 0) {
          step(cudaMemcpyAsync(lp.row_inert.data(), inert, static_cast<size_t>(m),
                               cudaMemcpyDeviceToHost, s));
        }
        step(cudaStreamSynchronize(s));
      }
      if (e == cudaSuccess && col_scale != nullptr && n > 0) {
        step(cudaMemcpy(col_scale, d.c, static_cast<size_t>(n) * sizeof(double),
                        cudaMemcpyDeviceToHost));
      }
      if (e == cudaSuccess && row_scale != nullptr && m > 0) {
        step(cudaMemcpy(row_scale, d.r, static_cast<size_t>(m) * sizeof(double),
                        cudaMemcpyDeviceToHost));
      }
      if (e != cudaSuccess) {
        if (err) *err = std::string("device setup: ") + cudaGetErrorString(e);
        rc = e == cudaErrorMemoryAllocation ? kErrOutOfMemory : kErrCuda;
      } else {
        lp.kptr = kptr;
        lp.kidx = kidx;
        lp.kval = kval;
        lp.tptr = d.lp_cp32;
        lp.tidx = d.lp_row;
        lp.tval = d.lp_val;
        lp.cost = d.cost;
        lp.lower = d.lower;
        lp.upper = d.upper;
        // Shared column bounds, each 0 or infinite: dividing by the positive column factors
        // keeps them, so the model's bounds decide (as the engine decides from the LpProblem's).
        if (n > 0) {
          const double lo = mv.col_lower[0], hi = mv.col_upper[0];
          bool uniform = (lo == 0.0 || lo == -INFINITY) && (hi == 0.0 || hi == INFINITY);
          for (int j = 1; uniform && j < n; ++j) {
            uniform = mv.col_lower[j] == lo && mv.col_upper[j] == hi;
          }
          lp.x_uniform = uniform;
          lp.x_lo = lo;
          lp.x_hi = hi;
        }
        rc = Engine::create_from_device(out, lp, opt, err);
      }
    }
  }
  cudaStreamDestroy(s);
  return rc;
}

// An engine for an LpProblem on the host (sg_pdlp_create's arguments) with the row-major copy
// of A built on the device: the input is checked on the host (row indices and values by up to 16
// threads), the column starts (as int32), row indices, values and vectors are uploaded once, and
// the nonzeros are sorted by row with CUB's stable radix sort. The same CSR as the host's counting sort (stable in both), so the
// same bits in every solve; the host keeps only O(m + n) work.
int create_engine_from_lp(Engine** out, int m, int n, const int64_t* colptr,
                          const int32_t* rowidx, const double* val, const double* cost,
                          const double* lower, const double* upper, const Options& opt,
                          std::string* err) {
  *out = nullptr;
  if (m < 0 || n < 0 || colptr == nullptr || cost == nullptr || lower == nullptr ||
      upper == nullptr) {
    if (err) *err = "invalid argument";
    return kErrInvalidArgument;
  }
  const long long nnz = colptr[n];
  if (nnz < 0 || colptr[0] != 0) {
    if (err) *err = "column starts must begin at 0";
    return kErrInvalidArgument;
  }
  if (nnz >= static_cast<long long>(std::numeric_limits<int>::max()) ||
      static_cast<long long>(n) + m >= std::numeric_limits<int>::max()) {
    if (err) *err = "matrix too large for 32-bit offsets";
    return kErrTooLarge;
  }
  if (nnz > 0 && (rowidx == nullptr || val == nullptr)) {
    if (err) *err = "null matrix arrays";
    return kErrInvalidArgument;
  }
  DeviceLp lp;
  lp.m = m;
  lp.n = n;
  lp.nnz = nnz;
  lp.tptr_host.resize(static_cast<size_t>(n) + 1);
  const long long nt = static_cast<long long>(n) + m;
  bool shared_bounds = false;
  {
    const char* why = nullptr;
    if (check_columns(m, n, colptr, cost, lower, upper, lp.tptr_host.data(), &shared_bounds, 16,
                      &why) != 0) {
      if (err) *err = why;
      return kErrInvalidArgument;
    }
  }
  if (nnz > 0) {
    const char* why = nullptr;
    if (check_nonzeros(m, nnz, rowidx, val, 16, &why) != 0) {
      if (err) *err = why;
      return kErrInvalidArgument;
    }
  }
  if (device_info(nullptr, nullptr, nullptr, 0) != kOk) {
    if (err) *err = "no sm_103 GPU";
    return kErrNoDevice;
  }
  cudaStream_t s = nullptr;
  SG_DEV(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  int rc = kOk;
  {
    Buffers t;
    int* tptr = nullptr;
    int32_t* row = nullptr;
    double* v = nullptr;
    double* c = nullptr;
    double* lo = nullptr;
    double* up = nullptr;
    int* col = nullptr;
    int* keys = nullptr;
    int* perm_in = nullptr;
    int* perm = nullptr;
    int* kptr = nullptr;
    int* kidx = nullptr;
    double* kval = nullptr;
    cudaError_t e = cudaSuccess;
    auto step = [&](cudaError_t x) {
      if (e == cudaSuccess) e = x;
    };
    const size_t nb = static_cast<size_t>(nnz);
    step(t.get(&tptr, static_cast<size_t>(n) + 1));
    step(t.get(&row, nb));
    step(t.get(&v, nb));
    step(t.get(&c, static_cast<size_t>(nt)));
    step(t.get(&lo, static_cast<size_t>(nt)));
    step(t.get(&up, static_cast<size_t>(nt)));
    step(t.get(&col, nb));
    step(t.get(&keys, nb));
    step(t.get(&perm_in, nb));
    step(t.get(&perm, nb));
    step(t.get(&kptr, static_cast<size_t>(m) + 1));
    step(t.get(&kidx, nb));
    step(t.get(&kval, nb));
    if (e == cudaSuccess) {
      step(cudaMemcpyAsync(tptr, lp.tptr_host.data(), (static_cast<size_t>(n) + 1) * sizeof(int),
                           cudaMemcpyHostToDevice, s));
      if (nb > 0) {
        step(cudaMemcpyAsync(row, rowidx, nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        step(cudaMemcpyAsync(v, val, nb * sizeof(double), cudaMemcpyHostToDevice, s));
      }
      if (nt > 0) {
        step(cudaMemcpyAsync(c, cost, nt * sizeof(double), cudaMemcpyHostToDevice, s));
        step(cudaMemcpyAsync(lo, lower, nt * sizeof(double), cudaMemcpyHostToDevice, s));
        step(cudaMemcpyAsync(up, upper, nt * sizeof(double), cudaMemcpyHostToDevice, s));
      }
    }
    // The row-major copy: a stable sort of the nonzeros by row.
    if (e == cudaSuccess && rc == kOk && nnz > 0) {
      if (n > 0) column_of_kernel<<<grid_for(n), kT, 0, s>>>(n, tptr, col);
      iota_kernel<<<grid_for(nnz), kT, 0, s>>>(static_cast<int>(nnz), perm_in);
      int bits = 1;
      while (bits < 31 && (1LL << bits) <= m) ++bits;
      size_t temp = 0;
      step(cub::DeviceRadixSort::SortPairs(nullptr, temp, row, keys, perm_in, perm,
                                           static_cast<int>(nnz), 0, bits, s));
      char* tmp = nullptr;
      step(t.get(&tmp, temp));
      step(cub::DeviceRadixSort::SortPairs(tmp, temp, row, keys, perm_in, perm,
                                           static_cast<int>(nnz), 0, bits, s));
      gather_rows_kernel<<<grid_for(nnz), kT, 0, s>>>(static_cast<int>(nnz), perm, col, v, kidx,
                                                      kval);
      step(cudaGetLastError());
    }
    if (e == cudaSuccess && rc == kOk) {
      row_starts_kernel<<<grid_for(static_cast<long long>(m) + 1), kT, 0, s>>>(
          m, static_cast<int>(nnz), keys, kptr);
      step(cudaGetLastError());
      lp.kptr_host.resize(static_cast<size_t>(m) + 1);
      step(cudaMemcpyAsync(lp.kptr_host.data(), kptr, lp.kptr_host.size() * sizeof(int),
                           cudaMemcpyDeviceToHost, s));
      step(cudaStreamSynchronize(s));
    }
    if (e != cudaSuccess) {
      if (err) *err = std::string("device setup: ") + cudaGetErrorString(e);
      rc = e == cudaErrorMemoryAllocation ? kErrOutOfMemory : kErrCuda;
    }
    if (rc == kOk) {
      // Inert rows and shared column bounds from the host's vectors (as Engine::create_from_device
      // expects them).
      lp.row_inert.resize(static_cast<size_t>(m));
      for (int i = 0; i < m; ++i) {
        lp.row_inert[i] = lp.kptr_host[i + 1] == lp.kptr_host[i] && cost[n + i] == 0.0 &&
                          lower[n + i] <= 0.0 && upper[n + i] >= 0.0;
      }
      if (n > 0) {
        const double l0 = lower[0], u0 = upper[0];
        lp.x_uniform = shared_bounds && (l0 == 0.0 || l0 == -INFINITY) &&
                       (u0 == 0.0 || u0 == INFINITY);
        lp.x_lo = l0;
        lp.x_hi = u0;
      }
      lp.kptr = kptr;
      lp.kidx = kidx;
      lp.kval = kval;
      lp.tptr = tptr;
      lp.tidx = row;
      lp.tval = v;
      lp.cost = c;
      lp.lower = lo;
      lp.upper = up;
      rc = Engine::create_from_device(out, lp, opt, err);
    }
  }
  cudaStreamDestroy(s);
  return rc;
}

}  // namespace sg
