// Host side of the batched PDLP engine (see sg_batch.cu).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <limits>
#include <numeric>
#include <random>

#include "../../include/sg_pdlp.h"
#include "sg_batch.cuh"

namespace sg {

template <typename T>
int Batch::alloc(T** p, size_t count) {
  *p = nullptr;
  const cudaError_t e =
      cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? SG_ERR_OUT_OF_MEMORY : SG_ERR_CUDA;
  allocs_.push_back(*p);
  return SG_OK;
}

Batch::~Batch() {
  if (stream_) cudaStreamSynchronize(stream_);
  for (void* p : allocs_) cudaFree(p);
  for (void* p : {static_cast<void*>(u_.ck), static_cast<void*>(u_.mask),
                  const_cast<void*>(static_cast<const void*>(u_.ck_off)),
                  const_cast<void*>(static_cast<const void*>(u_.mask_off))}) {
    if (p) cudaFree(p);
  }
  if (stream_) cudaStreamDestroy(stream_);
}

#define SG_B_TRY(call)                                     \
  do {                                                     \
    const int rc_ = (call);                                \
    if (rc_ != SG_OK) {                                    \
      if (err) *err = std::string("batch: ") + #call;     \
      delete b;                                            \
      return rc_;                                          \
    }                                                      \
  } while (0)

#define SG_B_CUDA(call)                                                              \
  do {                                                                               \
    const cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                         \
      if (err) *err = std::string(#call) + ": " + cudaGetErrorString(e_);           \
      delete b;                                                                      \
      return e_ == cudaErrorMemoryAllocation ? SG_ERR_OUT_OF_MEMORY : SG_ERR_CUDA; \
    }                                                                                \
  } while (0)

int Batch::create(Batch** out, int nmat, const int* mat_m, const int* mat_n,
                  const int64_t* mat_colptr, const int32_t* mat_rowidx, const double* mat_val,
                  int count, const int* inst_mat, const double* cost, const double* lower,
                  const double* upper, double tol, long long max_iter, double time_limit,
                  int precision, int algorithm, std::string* err) {
  *out = nullptr;
  if (nmat <= 0 || count <= 0 || mat_m == nullptr || mat_n == nullptr || mat_colptr == nullptr ||
      inst_mat == nullptr || cost == nullptr || lower == nullptr || upper == nullptr) {
    if (err) *err = "invalid argument";
    return SG_ERR_INVALID_ARGUMENT;
  }
  // Host layout of the matrices.
  std::vector<long long> nnz_off(nmat + 1, 0), kptr_off(nmat + 1, 0), tptr_off(nmat + 1, 0),
      col_off(nmat + 1, 0), row_off(nmat + 1, 0), cp_off(nmat + 1, 0);
  for (int g = 0; g < nmat; ++g) {
    if (mat_m[g] < 0 || mat_n[g] < 0) {
      if (err) *err = "negative dimension";
      return SG_ERR_INVALID_ARGUMENT;
    }
    cp_off[g + 1] = cp_off[g] + mat_n[g] + 1;
    const int64_t* cp = mat_colptr + cp_off[g];
    const long long nnz = cp[mat_n[g]];
    if (cp[0] != 0 || nnz < 0 || nnz >= std::numeric_limits<int>::max()) {
      if (err) *err = "bad column starts";
      return SG_ERR_INVALID_ARGUMENT;
    }
    for (int j = 0; j < mat_n[g]; ++j) {
      if (cp[j + 1] < cp[j]) {
        if (err) *err = "column starts decrease";
        return SG_ERR_INVALID_ARGUMENT;
      }
    }
    nnz_off[g + 1] = nnz_off[g] + nnz;
    kptr_off[g + 1] = kptr_off[g] + mat_m[g] + 1;
    tptr_off[g + 1] = tptr_off[g] + mat_n[g] + 1;
    col_off[g + 1] = col_off[g] + mat_n[g];
    row_off[g + 1] = row_off[g] + mat_m[g];
  }
  const long long total_nnz = nnz_off[nmat];
  if (total_nnz > 0 && (mat_rowidx == nullptr || mat_val == nullptr)) {
    if (err) *err = "null matrix arrays";
    return SG_ERR_INVALID_ARGUMENT;
  }
  std::vector<int> kptr(kptr_off[nmat]), tptr(tptr_off[nmat]), kidx(std::max(total_nnz, 1LL)),
      tidx(std::max(total_nnz, 1LL));
  std::vector<double> kval(std::max(total_nnz, 1LL)), tval(std::max(total_nnz, 1LL));
  int max_m = 0;
  for (int g = 0; g < nmat; ++g) {
    const int m = mat_m[g], n = mat_n[g];
    max_m = std::max(max_m, m);
    const int64_t* cp = mat_colptr + cp_off[g];
    const int32_t* ri = mat_rowidx + nnz_off[g];
    const double* va = mat_val + nnz_off[g];
    int* tp = tptr.data() + tptr_off[g];
    for (int j = 0; j <= n; ++j) tp[j] = static_cast<int>(cp[j]);
    for (long long p = 0; p < cp[n]; ++p) {
      if (ri[p] < 0 || ri[p] >= m || !std::isfinite(va[p])) {
        if (err) *err = "bad matrix entry";
        return SG_ERR_INVALID_ARGUMENT;
      }
      tidx[nnz_off[g] + p] = ri[p];
      tval[nnz_off[g] + p] = va[p];
    }
    int* kp = kptr.data() + kptr_off[g];
    std::fill(kp, kp + m + 1, 0);
    for (long long p = 0; p < cp[n]; ++p) ++kp[ri[p] + 1];
    for (int i = 0; i < m; ++i) kp[i + 1] += kp[i];
    std::vector<int> next(kp, kp + m);
    for (int j = 0; j < n; ++j) {
      for (long long p = cp[j]; p < cp[j + 1]; ++p) {
        const int q = next[ri[p]]++;
        kidx[nnz_off[g] + q] = j;
        kval[nnz_off[g] + q] = va[p];
      }
    }
  }
  // Instances.
  std::vector<long long> vec_off(count + 1, 0), yrow_off(count + 1, 0), state_off(count + 1, 0);
  const size_t tsz = precision == 1 ? sizeof(float) : sizeof(double);
  for (int i = 0; i < count; ++i) {
    const int g = inst_mat[i];
    if (g < 0 || g >= nmat) {
      if (err) *err = "instance matrix out of range";
      return SG_ERR_INVALID_ARGUMENT;
    }
    const long long nt = static_cast<long long>(mat_n[g]) + mat_m[g];
    vec_off[i + 1] = vec_off[i] + nt;
    yrow_off[i + 1] = yrow_off[i] + mat_m[g];
    // Keep every instance's block 16-byte aligned.
    long long elems = 8 * nt + 4 * static_cast<long long>(mat_m[g]);
    const long long align = 16 / static_cast<long long>(tsz);
    elems = (elems + align - 1) / align * align;
    state_off[i + 1] = state_off[i] + elems;
  }
  for (long long k = 0; k < vec_off[count]; ++k) {
    if (!std::isfinite(cost[k]) || std::isnan(lower[k]) || std::isnan(upper[k])) {
      if (err) *err = "cost or bound not valid";
      return SG_ERR_INVALID_ARGUMENT;
    }
  }
  // Largest instances first.
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    const long long wa = nnz_off[inst_mat[a] + 1] - nnz_off[inst_mat[a]] + vec_off[a + 1] - vec_off[a];
    const long long wc = nnz_off[inst_mat[c] + 1] - nnz_off[inst_mat[c]] + vec_off[c + 1] - vec_off[c];
    return wa > wc;
  });
  std::vector<double> u0(std::max(max_m, 1));
  {
    // The reference's power-iteration start (pdlp.cpp:47-51).
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> dist(-1.0, 1.0);
    for (int i = 0; i < max_m; ++i) u0[i] = dist(rng);
  }
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count <= 0) {
    cudaGetLastError();
    if (err) *err = "no GPU";
    return SG_ERR_NO_DEVICE;
  }
  Batch* b = new Batch();
  b->time_limit_ = time_limit;
  b->total_vec_ = vec_off[count];
  b->total_rows_ = yrow_off[count];
  b->vec_off_host_ = vec_off;
  b->inst_nt_host_.resize(count);
  b->inst_m_host_.resize(count);
  for (int i = 0; i < count; ++i) {
    b->inst_nt_host_[i] = static_cast<int>(vec_off[i + 1] - vec_off[i]);
    b->inst_m_host_[i] = mat_m[inst_mat[i]];
  }
  SG_B_CUDA(cudaStreamCreateWithFlags(&b->stream_, cudaStreamNonBlocking));
  BatchView& v = b->v_;
  v.nmat = nmat;
  v.count = count;
  auto up = [&](auto** dst, const auto* src, size_t n) -> int {
    using E = std::remove_const_t<std::remove_reference_t<decltype(*src)>>;
    E* d = nullptr;
    int rc = b->alloc(&d, n);
    if (rc != SG_OK) return rc;
    if (n > 0 && cudaMemcpy(d, src, n * sizeof(E), cudaMemcpyHostToDevice) != cudaSuccess) {
      return SG_ERR_CUDA;
    }
    *dst = d;
    return SG_OK;
  };
  int* d_mm = nullptr;
  int* d_mn = nullptr;
  long long *d_nz = nullptr, *d_kpo = nullptr, *d_tpo = nullptr, *d_co = nullptr, *d_ro = nullptr;
  SG_B_TRY(up(&d_mm, mat_m, nmat));
  SG_B_TRY(up(&d_mn, mat_n, nmat));
  SG_B_TRY(up(&d_nz, nnz_off.data(), nmat + 1));
  SG_B_TRY(up(&d_kpo, kptr_off.data(), nmat + 1));
  SG_B_TRY(up(&d_tpo, tptr_off.data(), nmat + 1));
  SG_B_TRY(up(&d_co, col_off.data(), nmat + 1));
  SG_B_TRY(up(&d_ro, row_off.data(), nmat + 1));
  v.mat_m = d_mm;
  v.mat_n = d_mn;
  v.mat_nnz_off = d_nz;
  v.mat_kptr_off = d_kpo;
  v.mat_tptr_off = d_tpo;
  v.mat_col_off = d_co;
  v.mat_row_off = d_ro;
  int *d_kp = nullptr, *d_ki = nullptr, *d_tp = nullptr, *d_ti = nullptr;
  double *d_kv0 = nullptr, *d_tv0 = nullptr;
  SG_B_TRY(up(&d_kp, kptr.data(), kptr.size()));
  SG_B_TRY(up(&d_ki, kidx.data(), total_nnz));
  SG_B_TRY(up(&d_tp, tptr.data(), tptr.size()));
  SG_B_TRY(up(&d_ti, tidx.data(), total_nnz));
  SG_B_TRY(up(&d_kv0, kval.data(), total_nnz));
  SG_B_TRY(up(&d_tv0, tval.data(), total_nnz));
  v.k_ptr = d_kp;
  v.k_idx = d_ki;
  v.t_ptr = d_tp;
  v.t_idx = d_ti;
  v.k_val0 = d_kv0;
  v.t_val0 = d_tv0;
  SG_B_TRY(b->alloc(&v.k_val, total_nnz));
  SG_B_TRY(b->alloc(&v.t_val, total_nnz));
  v.fp32 = precision == 1 ? 1 : 0;
  if (v.fp32) {
    SG_B_TRY(b->alloc(&v.k_val32, total_nnz));
    SG_B_TRY(b->alloc(&v.t_val32, total_nnz));
  }
  SG_B_TRY(b->alloc(&v.cs, col_off[nmat]));
  SG_B_TRY(b->alloc(&v.rs, row_off[nmat]));
  SG_B_TRY(b->alloc(&v.cn, col_off[nmat]));
  SG_B_TRY(b->alloc(&v.rn, row_off[nmat]));
  SG_B_TRY(b->alloc(&v.pu, row_off[nmat]));
  SG_B_TRY(b->alloc(&v.pv, col_off[nmat]));
  SG_B_TRY(b->alloc(&v.info, nmat));
  const double* d_u0 = nullptr;
  SG_B_TRY(up(&d_u0, u0.data(), u0.size()));
  v.power_start = d_u0;
  int* d_im = nullptr;
  long long *d_vo = nullptr, *d_yo = nullptr, *d_so = nullptr;
  double *d_c = nullptr, *d_l = nullptr, *d_u = nullptr;
  int* d_order = nullptr;
  SG_B_TRY(up(&d_im, inst_mat, count));
  SG_B_TRY(up(&d_vo, vec_off.data(), count + 1));
  SG_B_TRY(up(&d_yo, yrow_off.data(), count + 1));
  SG_B_TRY(up(&d_so, state_off.data(), count + 1));
  SG_B_TRY(up(&d_c, cost, vec_off[count]));
  SG_B_TRY(up(&d_l, lower, vec_off[count]));
  SG_B_TRY(up(&d_u, upper, vec_off[count]));
  SG_B_TRY(up(&d_order, order.data(), count));
  v.inst_mat = d_im;
  v.vec_off = d_vo;
  v.row_off = d_yo;
  v.state_off = d_so;
  v.cost = d_c;
  v.lower = d_l;
  v.upper = d_u;
  v.order = d_order;
  unsigned char* st = nullptr;
  SG_B_TRY(b->alloc(&st, static_cast<size_t>(state_off[count]) * tsz));
  v.state = st;
  SG_B_TRY(b->alloc(&v.x_out, vec_off[count]));
  SG_B_TRY(b->alloc(&v.y_out, yrow_off[count]));
  SG_B_TRY(b->alloc(&v.results, count));
  SG_B_TRY(b->alloc(&v.queue, 1));
  unsigned long long* dl = nullptr;
  SG_B_TRY(b->alloc(&dl, 1));
  v.deadline = dl;
  v.total_nnz = total_nnz;
  v.max_iter = max_iter;
  v.tol = tol;
  v.algorithm = algorithm == 1 || algorithm == 2 ? algorithm : 0;
  // The reference's 0.36 for its own algorithm; the Halpern iteration restarts at 0.1, as the
  // single-LP engine does (the enhanced PDHG keeps 0.36 here: measured no faster at 0.1 on the
  // batched node relaxations).
  v.art_frac = v.algorithm == 2 ? 0.1 : 0.36;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  b->grid_ = std::max(1, std::min(count, 2 * sms));
  *out = b;
  return SG_OK;
}

int Batch::solve(InstResult* results, double* x, double* y, double* device_ms, std::string* err) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, stream_);
  const unsigned long long budget =
      time_limit_ > 0 ? static_cast<unsigned long long>(time_limit_ * 1e9) : 0ull;
  launch_batch(v_, grid_, budget, stream_);
  cudaEventRecord(e1, stream_);
  cudaError_t e = cudaStreamSynchronize(stream_);
  if (e == cudaSuccess) e = cudaGetLastError();
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (device_ms) *device_ms = ms;
  if (e != cudaSuccess) {
    if (err) *err = std::string("batch solve: ") + cudaGetErrorString(e);
    return SG_ERR_CUDA;
  }
  if (results) {
    e = cudaMemcpy(results, v_.results, sizeof(InstResult) * v_.count, cudaMemcpyDeviceToHost);
  }
  if (e == cudaSuccess && x) {
    e = cudaMemcpy(x, v_.x_out, sizeof(double) * total_vec_, cudaMemcpyDeviceToHost);
  }
  if (e == cudaSuccess && y && total_rows_ > 0) {
    e = cudaMemcpy(y, v_.y_out, sizeof(double) * total_rows_, cudaMemcpyDeviceToHost);
  }
  if (e != cudaSuccess) {
    if (err) *err = std::string("batch download: ") + cudaGetErrorString(e);
    return SG_ERR_CUDA;
  }
  return SG_OK;
}

int Batch::unroll(int iterations, int every, double* v_out, std::string* err) {
  if (v_.fp32) {
    if (err) *err = "the unrolled PDHG runs in FP64: create the batch with SG_PRECISION_FP64";
    return SG_ERR_INVALID_ARGUMENT;
  }
  if (iterations <= 0 || every <= 0) {
    if (err) *err = "iterations and checkpoint interval must be positive";
    return SG_ERR_INVALID_ARGUMENT;
  }
  const int count = v_.count;
  const int nck = (iterations + every - 1) / every;
  std::vector<long long> ck_off(count + 1, 0), mask_off(count + 1, 0);
  for (int i = 0; i < count; ++i) {
    const long long nt = inst_nt_host_[i];
    ck_off[i + 1] = ck_off[i] + static_cast<long long>(nck) * (2 * nt + inst_m_host_[i]);
    // Keep every instance's masks 16-byte aligned.
    mask_off[i + 1] = mask_off[i] + (static_cast<long long>(every) * nt + 15) / 16 * 16;
  }
  auto fail = [&](cudaError_t e, const char* what) {
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SG_ERR_OUT_OF_MEMORY : SG_ERR_CUDA;
  };
  if (u_.iterations != iterations || u_.every != every || u_.ck == nullptr) {
    for (void* p : {static_cast<void*>(u_.ck), static_cast<void*>(u_.mask),
                    const_cast<void*>(static_cast<const void*>(u_.ck_off)),
                    const_cast<void*>(static_cast<const void*>(u_.mask_off))}) {
      if (p) cudaFree(p);
    }
    u_.ck = nullptr;
    u_.mask = nullptr;
    u_.ck_off = nullptr;
    u_.mask_off = nullptr;
    double* ck = nullptr;
    unsigned char* mask = nullptr;
    long long *cko = nullptr, *mko = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&ck),
                               std::max<long long>(ck_off[count], 1) * sizeof(double));
    if (e == cudaSuccess) {
      e = cudaMalloc(reinterpret_cast<void**>(&mask), std::max<long long>(mask_off[count], 16));
    }
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&cko), count * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&mko), count * sizeof(long long));
    if (e == cudaSuccess) {
      e = cudaMemcpy(cko, ck_off.data(), count * sizeof(long long), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
      e = cudaMemcpy(mko, mask_off.data(), count * sizeof(long long), cudaMemcpyHostToDevice);
    }
    u_.ck = ck;
    u_.mask = mask;
    u_.ck_off = cko;
    u_.mask_off = mko;
    if (e != cudaSuccess) return fail(e, "unroll buffers");
    if (u_.v_out == nullptr) {
      for (double** p : {&u_.v_out, &u_.grad_cost, &u_.grad_lower, &u_.grad_upper}) {
        const int rc = alloc(p, total_vec_);
        if (rc != SG_OK) {
          if (err) *err = "unroll buffers: out of memory";
          return rc;
        }
      }
      double* gv = nullptr;
      const int rc = alloc(&gv, total_vec_);
      if (rc != SG_OK) {
        if (err) *err = "unroll buffers: out of memory";
        return rc;
      }
      u_.grad_v = gv;
    }
    u_.iterations = iterations;
    u_.every = every;
    u_.nck = nck;
  }
  launch_batch_setup(v_, stream_);
  launch_unroll(v_, u_, 0, grid_, stream_);
  cudaError_t e = cudaStreamSynchronize(stream_);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail(e, "unroll");
  if (v_out) {
    e = cudaMemcpy(v_out, u_.v_out, sizeof(double) * total_vec_, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(e, "unroll download");
  }
  unrolled_ = true;
  return SG_OK;
}

int Batch::unroll_adjoint(const double* grad_v, double* grad_cost, double* grad_lower,
                          double* grad_upper, std::string* err) {
  if (!unrolled_) {
    if (err) *err = "sg_batch_unroll must run before its adjoint";
    return SG_ERR_NOT_READY;
  }
  if (grad_v == nullptr) {
    if (err) *err = "grad_v is required";
    return SG_ERR_INVALID_ARGUMENT;
  }
  auto fail = [&](cudaError_t e, const char* what) {
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return SG_ERR_CUDA;
  };
  cudaError_t e = cudaMemcpy(const_cast<double*>(u_.grad_v), grad_v,
                             sizeof(double) * total_vec_, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(e, "adjoint upload");
  launch_batch_setup(v_, stream_);
  launch_unroll(v_, u_, 1, grid_, stream_);
  e = cudaStreamSynchronize(stream_);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail(e, "adjoint");
  const std::pair<double*, const double*> outs[3] = {
      {grad_cost, u_.grad_cost}, {grad_lower, u_.grad_lower}, {grad_upper, u_.grad_upper}};
  for (const auto& o : outs) {
    if (o.first == nullptr) continue;
    e = cudaMemcpy(o.first, o.second, sizeof(double) * total_vec_, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(e, "adjoint download");
  }
  return SG_OK;
}

}  // namespace sg

struct sg_batch {
  sg::Batch* batch = nullptr;
};

namespace {
thread_local std::string g_batch_error;
}

extern "C" {

int sg_batch_create(sg_batch** handle, int nmat, const int* mat_m, const int* mat_n,
                    const int64_t* mat_colptr, const int32_t* mat_rowidx, const double* mat_val,
                    int count, const int* inst_mat, const double* cost, const double* lower,
                    const double* upper, const sg_pdlp_opts* opts) {
  if (handle == nullptr) return SG_ERR_INVALID_ARGUMENT;
  *handle = nullptr;
  try {
    sg_pdlp_opts d;
    sg_pdlp_default_opts(&d);
    if (opts == nullptr) opts = &d;
    std::string why;
    sg::Batch* b = nullptr;
    const int rc = sg::Batch::create(&b, nmat, mat_m, mat_n, mat_colptr, mat_rowidx, mat_val,
                                     count, inst_mat, cost, lower, upper,
                                     opts->tol > 0 ? opts->tol : 1e-8, opts->max_iterations,
                                     opts->time_limit, opts->precision, opts->algorithm, &why);
    if (rc != SG_OK) {
      g_batch_error = why;
      return rc;
    }
    *handle = new sg_batch{b};
    return SG_OK;
  } catch (...) {
    g_batch_error = "unexpected exception";
    return SG_ERR_INTERNAL;
  }
}

int sg_batch_solve(sg_batch* handle, sg_batch_result* results, double* x, double* y,
                   double* device_ms) {
  if (handle == nullptr || handle->batch == nullptr) return SG_ERR_INVALID_ARGUMENT;
  try {
    std::string why;
    static_assert(sizeof(sg::InstResult) == sizeof(sg_batch_result), "result layout");
    const int rc = handle->batch->solve(reinterpret_cast<sg::InstResult*>(results), x, y,
                                        device_ms, &why);
    if (rc != SG_OK) g_batch_error = why;
    return rc;
  } catch (...) {
    g_batch_error = "unexpected exception";
    return SG_ERR_INTERNAL;
  }
}

void sg_batch_destroy(sg_batch* handle) {
  if (handle == nullptr) return;
  try {
    delete handle->batch;
  } catch (...) {
  }
  delete handle;
}

int sg_batch_unroll(sg_batch* handle, int iterations, int checkpoint_every, double* v_out) {
  if (handle == nullptr || handle->batch == nullptr) return SG_ERR_INVALID_ARGUMENT;
  try {
    std::string why;
    const int rc = handle->batch->unroll(iterations, checkpoint_every, v_out, &why);
    if (rc != SG_OK) g_batch_error = why;
    return rc;
  } catch (...) {
    g_batch_error = "unexpected exception";
    return SG_ERR_INTERNAL;
  }
}

int sg_batch_unroll_adjoint(sg_batch* handle, const double* grad_v, double* grad_cost,
                            double* grad_lower, double* grad_upper) {
  if (handle == nullptr || handle->batch == nullptr) return SG_ERR_INVALID_ARGUMENT;
  try {
    std::string why;
    const int rc =
        handle->batch->unroll_adjoint(grad_v, grad_cost, grad_lower, grad_upper, &why);
    if (rc != SG_OK) g_batch_error = why;
    return rc;
  } catch (...) {
    g_batch_error = "unexpected exception";
    return SG_ERR_INTERNAL;
  }
}

const char* sg_batch_last_error(void) { return g_batch_error.c_str(); }

}  // extern "C"
