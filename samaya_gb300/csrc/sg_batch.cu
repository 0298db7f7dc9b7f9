// Batched PDLP: many LPs in one persistent launch (the engine's own; the reference solves one
// LP at a time). Instances are stored as a segmented concatenated CSR: matrices (each by rows,
// A, and by columns, A') concatenated with offsets, several instances may share one matrix
// (branch-and-bound node relaxations: one A, many bound vectors), and every instance has its
// own cost and bounds.
//
// Two kernels:
//   batch_setup_kernel   one CTA per matrix: the residual-scale norms of A, Ruiz (or the
//                        enhanced preconditioning), A_eq in place, and ||[A_eq -I]|| by power
//                        iteration — shared by every instance of that matrix;
//   batch_solve_kernel   persistent CTAs pull instances from a work queue (largest first) and
//                        run the whole PDLP of one instance inside the CTA: the fused steps, the
//                        evaluation every 64 iterations, the termination test, the restarts and
//                        the primal-weight update of the single-LP engine (the reference's rules,
//                        pdlp.cpp:493-541, 674-713, 1069-1131), per instance.
// Row sums: one thread per row, a warp per row longer than 32 nonzeros (ballot queue), fixed
// order, so a re-run is bit-identical.
#include <math.h>
#include <stdint.h>

#include "sg_batch.cuh"

namespace sg {

namespace {

constexpr int kBT = 512;  // threads per CTA of the batched kernels
constexpr int kBWarps = kBT / 32;

__device__ __forceinline__ double bsum(double v, double* sh) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < kBWarps; ++w) t += sh[w];
    sh[kBWarps] = t;
  }
  __syncthreads();
  return sh[kBWarps];
}

// K sums at once (fixed order), result broadcast to every thread.
template <int K>
__device__ __forceinline__ void bsums(double (&v)[K], double* sh) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < K; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
  }
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) sh[q * kBWarps + warp] = v[q];
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double t = 0.0;
    for (int w = 0; w < kBWarps; ++w) t += sh[threadIdx.x * kBWarps + w];
    sh[K * kBWarps + threadIdx.x] = t;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < K; ++q) v[q] = sh[K * kBWarps + q];
  __syncthreads();
}

__device__ __forceinline__ double bmax(double v, double* sh) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = sh[0];
    for (int w = 1; w < kBWarps; ++w) t = fmax(t, sh[w]);
    sh[kBWarps] = t;
  }
  __syncthreads();
  return sh[kBWarps];
}

// For every row r < rows of a CSR (ptr, idx, val): s = sum_k prod(val_k, idx_k) (or max), then
// f(r, s). Thread per row; rows longer than 32 nonzeros by their warp. The sums are taken in
// prod's result type (FP32 for the FP32 steps: GB300's FP64 pipe is small).
template <bool MAXRED, typename T, typename Prod, typename F>
__device__ __forceinline__ void block_rows(int rows, const int* __restrict__ ptr,
                                           const int* __restrict__ idx, const T* __restrict__ val,
                                           const Prod& prod, F& f) {
  using ACC = decltype(prod(val[0], 0));
  const int lane = threadIdx.x & 31;
  for (int base = 0; base < rows; base += kBT) {
    const int r = base + threadIdx.x;
    const bool valid = r < rows;
    int b = 0, e = 0;
    if (valid) {
      b = ptr[r];
      e = ptr[r + 1];
    }
    const bool shortrow = valid && e - b <= 32;
    if (shortrow) {
      ACC s = ACC(0);
      for (int q = b; q < e; ++q) {
        const ACC p = prod(val[q], idx[q]);
        s = MAXRED ? fmax(s, p) : s + p;
      }
      f(r, s);
    }
    unsigned pending = __ballot_sync(0xffffffffu, valid && !shortrow);
    while (pending != 0u) {
      const int src = __ffs(pending) - 1;
      pending &= pending - 1u;
      const int rb = __shfl_sync(0xffffffffu, b, src);
      const int re = __shfl_sync(0xffffffffu, e, src);
      ACC s = ACC(0);
      for (int q = rb + lane; q < re; q += 32) {
        const ACC p = prod(val[q], idx[q]);
        s = MAXRED ? fmax(s, p) : s + p;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const ACC t = __shfl_down_sync(0xffffffffu, s, o);
        s = MAXRED ? fmax(s, t) : s + t;
      }
      if (lane == 0) f(base + (threadIdx.x & ~31) + src, s);
    }
  }
}

__device__ __forceinline__ double lam_of(double g, double lo, double up) {
  const bool hl = lo > -INFINITY;
  const bool hu = up < INFINITY;
  return hl && hu ? g : hl ? fmax(g, 0.0) : hu ? fmin(g, 0.0) : 0.0;
}

}  // namespace

// ------------------------------------------------------------------------------------------
// Setup: one CTA per matrix.
__global__ void __launch_bounds__(kBT) batch_setup_kernel(BatchView b) {
  __shared__ double sh[32 * (kBWarps + 1)];
  const int g = blockIdx.x;
  if (g >= b.nmat) return;
  const int m = b.mat_m[g];
  const int n = b.mat_n[g];
  const long long nz = b.mat_nnz_off[g];
  const long long nnz = b.mat_nnz_off[g + 1] - nz;
  const int* kp = b.k_ptr + b.mat_kptr_off[g];
  const int* ki = b.k_idx + nz;
  double* kv = b.k_val + nz;
  const double* kv0 = b.k_val0 + nz;
  const int* tp = b.t_ptr + b.mat_tptr_off[g];
  const int* ti = b.t_idx + nz;
  double* tv = b.t_val + nz;
  const double* tv0 = b.t_val0 + nz;
  double* cs = b.cs + b.mat_col_off[g];
  double* rs = b.rs + b.mat_row_off[g];
  double* cn = b.cn + b.mat_col_off[g];
  double* rn = b.rn + b.mat_row_off[g];
  double* pu = b.pu + b.mat_row_off[g];
  double* pv = b.pv + b.mat_col_off[g];
  MatInfo* info = b.info + g;
  for (long long k = threadIdx.x; k < nnz; k += kBT) {
    kv[k] = kv0[k];
    tv[k] = tv0[k];
  }
  for (int j = threadIdx.x; j < n; j += kBT) cs[j] = 1.0;
  for (int i = threadIdx.x; i < m; i += kBT) rs[i] = 1.0;
  __syncthreads();
  // Relative-residual scales of the original matrix (pdlp.cpp:377-394).
  double amc = 0.0, amr = 0.0;
  if (m > 0) {
    struct Sq {
      __device__ double operator()(double a, int) const { return a * a; }
    } sq;
    double loc = 0.0;
    auto colmax = [&](int, double s) { loc = fmax(loc, sqrt(s)); };
    block_rows<false>(n, tp, ti, tv, sq, colmax);
    amc = bmax(loc, sh);
    loc = 0.0;
    auto rowmax = [&](int, double s) { loc = fmax(loc, sqrt(s)); };
    block_rows<false>(m, kp, ki, kv, sq, rowmax);
    amr = bmax(loc, sh);
  }
  // Preconditioning.
  if (m > 0 && n > 0) {
    if (b.algorithm >= 1) {
      for (int pass = 0; pass < 11; ++pass) {
        const bool ruiz = pass < 10;
        struct Abs {
          const double* o;
          __device__ double operator()(double a, int j) const { return fabs(a) * o[j]; }
        };
        Abs pc{rs};
        Abs pr{cs};
        if (ruiz) {
          auto fc = [&](int j, double s) { cn[j] = s * cs[j]; };
          block_rows<true>(n, tp, ti, tv, pc, fc);
          auto fr = [&](int i, double s) { rn[i] = s * rs[i]; };
          block_rows<true>(m, kp, ki, kv, pr, fr);
        } else {
          auto fc = [&](int j, double s) { cn[j] = s * cs[j]; };
          block_rows<false>(n, tp, ti, tv, pc, fc);
          auto fr = [&](int i, double s) { rn[i] = s * rs[i]; };
          block_rows<false>(m, kp, ki, kv, pr, fr);
        }
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += kBT) {
          if (cn[j] > 0.0) cs[j] = cs[j] / sqrt(cn[j]);
        }
        for (int i = threadIdx.x; i < m; i += kBT) {
          if (rn[i] > 0.0) rs[i] = rs[i] / sqrt(rn[i]);
        }
        __syncthreads();
      }
    } else {
      // The reference's L2 Ruiz (pdlp.cpp:109-187).
      for (int pass = 0; pass < 10; ++pass) {
        struct Sq2 {
          const double* o;
          __device__ double operator()(double a, int j) const {
            const double v = a * o[j];
            return v * v;
          }
        };
        Sq2 pc{rs};
        Sq2 pr{cs};
        auto fc = [&](int j, double s) { cn[j] = sqrt(s) * cs[j]; };
        block_rows<false>(n, tp, ti, tv, pc, fc);
        auto fr = [&](int i, double s) { rn[i] = sqrt(s) * rs[i]; };
        block_rows<false>(m, kp, ki, kv, pr, fr);
        __syncthreads();
        double changed = 0.0;
        for (int k = threadIdx.x; k < n + m; k += kBT) {
          double* sc = k < n ? cs + k : rs + (k - n);
          const double nv = k < n ? cn[k] : rn[k - n];
          if (nv > 0) {
            const double old = *sc;
            double s = old / nv;
            s = fmax(1e-8, fmin(1e8, s));
            if (fabs(s - old) / fmax(fabs(old), 1.0) > 0.1) changed = 1.0;
            *sc = s;
          }
        }
        if (bmax(changed, sh) == 0.0) break;
      }
    }
  }
  __syncthreads();
  // A_eq in place: K entries (a rs_i) cs_j, K' entries (a cs_j) rs_i.
  for (int i = threadIdx.x; i < m; i += kBT) {
    for (int q = kp[i]; q < kp[i + 1]; ++q) kv[q] = kv[q] * rs[i] * cs[ki[q]];
  }
  for (int j = threadIdx.x; j < n; j += kBT) {
    for (int q = tp[j]; q < tp[j + 1]; ++q) tv[q] = tv[q] * cs[j] * rs[ti[q]];
  }
  __syncthreads();
  // Power iteration (pdlp.cpp:36-103).
  double L = 1.0;
  if (m > 0) {
    for (int i = threadIdx.x; i < m; i += kBT) pu[i] = b.power_start[i];
    __syncthreads();
    double ss = 0.0;
    for (int i = threadIdx.x; i < m; i += kBT) ss += pu[i] * pu[i];
    double un = sqrt(bsum(ss, sh));
    for (int i = threadIdx.x; i < m; i += kBT) pu[i] = pu[i] / un;
    __syncthreads();
    double sigma = 0.0;
    bool zero = false;
    struct G {
      const double* x;
      __device__ double operator()(double a, int j) const { return a * x[j]; }
    };
    for (int it = 0; it < 20 && !zero; ++it) {
      double acc = 0.0;
      G gu{pu};
      auto fv = [&](int j, double s) { pv[j] = s; acc += s * s; };
      block_rows<false>(n, tp, ti, tv, gu, fv);
      const double vn = sqrt(bsum(acc, sh));
      if (vn == 0.0) {
        zero = true;
        break;
      }
      acc = 0.0;
      G gv{pv};
      auto fu = [&](int i, double s) { pu[i] = s; acc += s * s; };
      block_rows<false>(m, kp, ki, kv, gv, fu);
      un = sqrt(bsum(acc, sh));
      if (un == 0.0) {
        zero = true;
        break;
      }
      sigma = un / vn;
      for (int i = threadIdx.x; i < m; i += kBT) pu[i] = pu[i] / un;
      __syncthreads();
    }
    if (!zero) {
      const double la = sigma * 1.01;
      L = sqrt(la * la + 1.0);
    }
  }
  if (threadIdx.x == 0) {
    info->eta = 0.99 / L;
    info->a_norm_max_col = amc;
    info->at_norm_max_row = amr;
  }
}

// ------------------------------------------------------------------------------------------
// Solve: persistent CTAs, one instance at a time.

namespace {

struct Meas {
  double rp, rd, rg, pobj, dobj;
};

__device__ __forceinline__ Meas finish7(const double* s, double amc, double amr, double cnorm,
                                        int m) {
  Meas r;
  const double ps = 1.0 + amc * sqrt(s[4]) + sqrt(s[5]);
  const double ds = 1.0 + amr * sqrt(s[6]) + cnorm;
  const double gs = 1.0 + fabs(s[2]) + fabs(s[3]);
  r.rp = m > 0 ? sqrt(s[0]) / ps : 0.0;
  r.rd = m > 0 ? sqrt(s[1]) / ds : 0.0;
  r.rg = (s[2] - s[3]) / gs;
  r.pobj = s[2];
  r.dobj = s[3];
  return r;
}

__device__ __forceinline__ double kkt_w(double w, const Meas& e) {
  return sqrt(w * w * e.rp * e.rp + e.rd * e.rd / (w * w) + e.rg * e.rg);
}

template <typename T>
__device__ void solve_instance(const BatchView& b, int inst, double* sh) {
  const int g = b.inst_mat[inst];
  const int m = b.mat_m[g];
  const int n = b.mat_n[g];
  const int nt = n + m;
  const long long nz = b.mat_nnz_off[g];
  const int* kp = b.k_ptr + b.mat_kptr_off[g];
  const int* ki = b.k_idx + nz;
  const int* tp = b.t_ptr + b.mat_tptr_off[g];
  const int* ti = b.t_idx + nz;
  const T* kv = reinterpret_cast<const T*>(b.fp32 ? static_cast<const void*>(b.k_val32 + nz)
                                                  : static_cast<const void*>(b.k_val + nz));
  const T* tv = reinterpret_cast<const T*>(b.fp32 ? static_cast<const void*>(b.t_val32 + nz)
                                                  : static_cast<const void*>(b.t_val + nz));
  const double* cs = b.cs + b.mat_col_off[g];
  const double* rs = b.rs + b.mat_row_off[g];
  const MatInfo mi = b.info[g];
  const long long vo = b.vec_off[inst];
  const long long yo = b.row_off[inst];
  const double* cost0 = b.cost + vo;
  const double* lo0 = b.lower + vo;
  const double* up0 = b.upper + vo;
  T* st = reinterpret_cast<T*>(b.state) + b.state_off[inst];
  // Per-instance state (storage type T): V0 V1 Vbar Verg Vrst c l u (nt each), Y0 Y1 Yerg Yrst
  // (m each).
  // Ping-pong pairs picked by selects (a runtime index into a local array puts it in local
  // memory).
  T* const V0 = st;
  T* const V1 = st + nt;
  T* Vbar = st + 2 * nt;
  T* Verg = st + 3 * nt;
  T* Vrst = st + 4 * nt;
  T* ce = st + 5 * nt;
  T* le = st + 6 * nt;
  T* ue = st + 7 * nt;
  T* const Y0 = st + 8 * nt;
  T* const Y1 = st + 8 * nt + m;
  auto V = [&](int q) { return q ? V1 : V0; };
  auto Y = [&](int q) { return q ? Y1 : Y0; };
  T* Yerg = st + 8 * nt + 2 * m;
  T* Yrst = st + 8 * nt + 3 * m;
  // Scaled problem, zero iterates, ||c||.
  double cc = 0.0, c2 = 0.0, b2 = 0.0;
  for (int k = threadIdx.x; k < nt; k += kBT) {
    double c, l, u;
    if (k < n) {
      c = cost0[k] * cs[k];
      l = lo0[k] / cs[k];
      u = up0[k] / cs[k];
      c2 += c * c;
    } else {
      const double r = rs[k - n];
      c = cost0[k] * r;
      l = lo0[k] * r;
      u = up0[k] * r;
      const double bb = fmax(isfinite(l) ? fabs(l) : 0.0, isfinite(u) ? fabs(u) : 0.0);
      b2 += bb * bb;
    }
    ce[k] = static_cast<T>(c);
    le[k] = static_cast<T>(l);
    ue[k] = static_cast<T>(u);
    cc += cost0[k] * cost0[k];
    V0[k] = V1[k] = Vbar[k] = Verg[k] = Vrst[k] = T(0);
    if (k < m) Y0[k] = Y1[k] = Yerg[k] = Yrst[k] = T(0);
  }
  double nrm[3] = {cc, c2, b2};
  bsums<3>(nrm, sh);
  const double c_norm = sqrt(nrm[0]);
  double omega = 1.0;
  const bool halpern = b.algorithm == 2;
  if (b.algorithm >= 1) {
    const double cn = sqrt(nrm[1]), bn = sqrt(nrm[2]);
    omega = (cn > 1e-10 && bn > 1e-10) ? cn / bn : 1.0;
  }
  const double eta = mi.eta;
  double tau = eta / omega, sigma = eta * omega;
  long long max_iter = b.max_iter;
  if (max_iter <= 0) {
    max_iter = 10000LL * nt / 10;
    if (max_iter < 10000LL) max_iter = 10000LL;
    if (max_iter > 1000000LL) max_iter = 1000000LL;
  }
  double kar = INFINITY, kprev = INFINITY;
  long long t = 0, k_since = 0, restarts = 0;
  int status = kIterationLimit;
  int result_avg = 0;
  Meas final_meas{0, 0, 0, 0, 0};
  __syncthreads();
  while (t < max_iter) {
    const int p = static_cast<int>(t & 1);
    const double alpha = 1.0 / static_cast<double>(k_since + 1);
    const T ta = static_cast<T>(alpha), tb = static_cast<T>(1.0 - alpha);
    const T tsig = static_cast<T>(sigma), ttau = static_cast<T>(tau);
    if (halpern) {
      // The reflected Halpern iteration z+ = N + w (z0 - N), N = 2 T(z) - z, w = 1 / (k + 2)
      // (k: iterations since the restart), T the PDHG map in primal-first order, as the
      // single-LP engine's halpern_primal / halpern_dual kernels compute it; T(z) lands in
      // Verg / Yerg (the point the evaluation, the restarts and the answer use).
      const T tw = static_cast<T>(1.0 / static_cast<double>(k_since + 2));
      {
        struct G {
          const T* y;
          __device__ T operator()(T a, int i) const { return a * y[i]; }
        } gy{Y(p)};
        const T* x = V(p);
        T* xn = V(p ^ 1);
        auto f = [&](int j, T s) {
          const T xo = x[j];
          const T xh = fmin(fmax(xo - ttau * (ce[j] + s), le[j]), ue[j]);
          const T refl = xh + (xh - xo);
          Verg[j] = xh;
          Vbar[j] = refl;
          xn[j] = refl + tw * (Vrst[j] - refl);
        };
        block_rows<false>(n, tp, ti, tv, gy, f);
      }
      __syncthreads();
      {
        struct G {
          const T* x;
          __device__ T operator()(T a, int j) const { return a * x[j]; }
        } gx{Vbar};
        const T* yv = Y(p);
        T* yn = Y(p ^ 1);
        const T* vr = V(p) + n;
        T* vrn = V(p ^ 1) + n;
        auto f = [&](int i, T s) {
          const T y = yv[i];
          const T r = vr[i];
          const T rh = fmin(fmax(r - ttau * (ce[n + i] - y), le[n + i]), ue[n + i]);
          const T rrefl = rh + (rh - r);
          const T yh = y + tsig * (s - rrefl);
          Yerg[i] = yh;
          Verg[n + i] = rh;
          const T yrefl = yh + (yh - y);
          yn[i] = yrefl + tw * (Yrst[i] - yrefl);
          vrn[i] = rrefl + tw * (Vrst[n + i] - rrefl);
        };
        block_rows<false>(m, kp, ki, kv, gx, f);
      }
      __syncthreads();
    } else {
    // Dual step (rows of A_eq) with the logicals' primal update.
    {
      // Products and sums in the storage type.
      struct G {
        const T* x;
        __device__ T operator()(T a, int j) const { return a * x[j]; }
      } gx{Vbar};
      const T* yv = Y(p);
      T* yn = Y(p ^ 1);
      const T* vr = V(p) + n;
      T* vrn = V(p ^ 1) + n;
      T* vbr = Vbar + n;
      auto f = [&](int i, T s) {
        const T res = s - vbr[i];
        const T ynew = yv[i] + tsig * res;
        yn[i] = ynew;
        const T r = vr[i];
        T rn = r - ttau * (ce[n + i] - ynew);
        rn = fmin(fmax(rn, le[n + i]), ue[n + i]);
        vrn[i] = rn;
        vbr[i] = rn + (rn - r);
        Yerg[i] = tb * Yerg[i] + ta * ynew;
        Verg[n + i] = tb * Verg[n + i] + ta * rn;
      };
      block_rows<false>(m, kp, ki, kv, gx, f);
    }
    __syncthreads();
    // Primal step (rows of A_eq').
    {
      struct G {
        const T* y;
        __device__ T operator()(T a, int i) const { return a * y[i]; }
      } gy{Y(p ^ 1)};
      const T* x = V(p);
      T* xn = V(p ^ 1);
      auto f = [&](int j, T s) {
        const T xo = x[j];
        T v = xo - ttau * (ce[j] + s);
        v = fmin(fmax(v, le[j]), ue[j]);
        xn[j] = v;
        Vbar[j] = v + (v - xo);
        Verg[j] = tb * Verg[j] + ta * v;
      };
      block_rows<false>(n, tp, ti, tv, gy, f);
    }
    __syncthreads();
    }
    ++t;
    ++k_since;
    if (t % 64 != 0 && t != max_iter) continue;
    // Evaluation of the current and the average iterate (pdlp.cpp:411-488), original space.
    const int cur = static_cast<int>(t & 1);
    // One iterate's sums (7 evaluation sums, restart distances of v and y) into e with
    // constant indices, so they stay in registers; called for the current and the average
    // iterate.
    struct G2 {
      const T* x;
      __device__ double operator()(T v, int j) const {
        return static_cast<double>(v) * static_cast<double>(x[j]);
      }
    };
    auto eval_one = [&](const T* vv, const T* yy, double (&e)[9]) {
#pragma unroll
      for (int q = 0; q < 9; ++q) e[q] = 0.0;
      G2 gx{vv};
      auto fr = [&](int i, double s) {
        const double r_s = rs[i];
        const double value = static_cast<double>(vv[n + i]) / r_s;
        const double yo2 = static_cast<double>(yy[i]) * r_s;
        const double c = cost0[n + i];
        const double g2 = c - yo2;
        const double ep = s / r_s - value;
        e[0] += ep * ep;
        e[5] += value * value;
        e[6] += yo2 * yo2;
        e[2] += c * value;
        const double lam = lam_of(g2, lo0[n + i], up0[n + i]);
        e[1] += (g2 - lam) * (g2 - lam);
        if (lam > 0.0) e[3] += lam * lo0[n + i];
        if (lam < 0.0) e[3] += lam * up0[n + i];
        const double dv = static_cast<double>(vv[n + i]) - static_cast<double>(Vrst[n + i]);
        const double dy = static_cast<double>(yy[i]) - static_cast<double>(Yrst[i]);
        e[7] += dv * dv;
        e[8] += dy * dy;
      };
      block_rows<false>(m, kp, ki, kv, gx, fr);
      G2 gy{yy};
      auto fc = [&](int j, double s) {
        const double c_s = cs[j];
        const double value = static_cast<double>(vv[j]) * c_s;
        const double c = cost0[j];
        const double g2 = c + (m > 0 ? s / c_s : 0.0);
        e[4] += value * value;
        e[2] += c * value;
        const double lam = lam_of(g2, lo0[j], up0[j]);
        e[1] += (g2 - lam) * (g2 - lam);
        if (lam > 0.0) e[3] += lam * lo0[j];
        if (lam < 0.0) e[3] += lam * up0[j];
        const double dv = static_cast<double>(vv[j]) - static_cast<double>(Vrst[j]);
        e[7] += dv * dv;
      };
      block_rows<false>(n, tp, ti, tv, gy, fc);
    };
    double ec[9], ea[9];
    // Halpern: only T(z) is measured (the Halpern iterate itself can leave the bounds).
    if (halpern) {
#pragma unroll
      for (int q = 0; q < 9; ++q) ec[q] = 0.0;
    } else {
      eval_one(V(cur), Y(cur), ec);
    }
    eval_one(Verg, Yerg, ea);
    // a: the current iterate's 7 sums, the average's 7, then the distances (v, y) of each.
    double a[18];
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      a[q] = ec[q];
      a[7 + q] = ea[q];
    }
    a[14] = ec[7];
    a[15] = ec[8];
    a[16] = ea[7];
    a[17] = ea[8];
    bsums<18>(a, sh);
    const Meas mc = finish7(a, mi.a_norm_max_col, mi.at_norm_max_row, c_norm, m);
    const Meas ma = finish7(a + 7, mi.a_norm_max_col, mi.at_norm_max_row, c_norm, m);
    const double tol = b.tol;
    if (!halpern && mc.rp < tol && mc.rd < tol && fabs(mc.rg) < tol) {
      status = kOptimal;
      final_meas = mc;
      break;
    }
    if (ma.rp < tol && ma.rd < tol && fabs(ma.rg) < tol) {
      status = kOptimal;
      result_avg = 1;
      final_meas = ma;
      break;
    }
    final_meas = halpern ? ma : mc;
    // Restart (pdlp.cpp:1069-1131); the Halpern iteration restarts to T(z).
    const double kc = kkt_w(omega, mc), ka = kkt_w(omega, ma);
    const bool to_avg = halpern || ka < kc;
    const double cand = halpern ? ka : fmin(kc, ka);
    if (!(kar < INFINITY)) kar = cand;
    const bool restart = cand <= 0.2 * kar || (cand <= 0.8 * kar && cand > kprev) ||
                         static_cast<double>(k_since) >= b.art_frac * static_cast<double>(t);
    kprev = cand;
    if (restart) {
      const double dx = sqrt(a[to_avg ? 16 : 14]);
      const double dy = sqrt(a[to_avg ? 17 : 15]);
      if (dx > 1e-10 && dy > 1e-10) {
        omega = exp(0.5 * log(dy / dx) + 0.5 * log(omega));
        tau = eta / omega;
        sigma = eta * omega;
      }
      const T* vc = to_avg ? Verg : V(cur);
      const T* yc = to_avg ? Yerg : Y(cur);
      for (int k = threadIdx.x; k < nt; k += kBT) {
        const T v = vc[k];
        Vrst[k] = v;
        V0[k] = v;
        V1[k] = v;
        Vbar[k] = v;
        if (k < m) {
          const T y = yc[k];
          Yrst[k] = y;
          Y0[k] = y;
          Y1[k] = y;
        }
      }
      __syncthreads();
      k_since = 0;
      kar = cand;
      kprev = INFINITY;
      ++restarts;
    }
    const unsigned long long deadline = *b.deadline;
    if (deadline != 0ull) {
      unsigned long long now;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
      if (now > deadline) {
        status = kTimeLimit;
        break;
      }
    }
  }
  // Answer in the LpProblem's space (Halpern: T(z), within the bounds).
  if (halpern) result_avg = 1;
  const int cur = static_cast<int>(t & 1);
  const T* vv = result_avg ? Verg : V(cur);
  const T* yy = result_avg ? Yerg : Y(cur);
  double* xo = b.x_out + vo;
  double* yo2 = b.y_out + yo;
  for (int k = threadIdx.x; k < nt; k += kBT) {
    xo[k] = k < n ? static_cast<double>(vv[k]) * cs[k] : static_cast<double>(vv[k]) / rs[k - n];
    if (k < m) yo2[k] = static_cast<double>(yy[k]) * rs[k];
  }
  if (threadIdx.x == 0) {
    InstResult& r = b.results[inst];
    r.status = status;
    r.iterations = status == kIterationLimit ? max_iter : t;
    r.rel_primal = final_meas.rp;
    r.rel_dual = final_meas.rd;
    r.rel_gap = final_meas.rg;
    r.primal_obj = final_meas.pobj;
    r.dual_obj = final_meas.dobj;
    r.restarts = restarts;
  }
  __syncthreads();
}

}  // namespace

template <typename T>
__global__ void __launch_bounds__(kBT) batch_solve_kernel(BatchView b) {
  __shared__ double sh[32 * (kBWarps + 1)];
  __shared__ int next;
  for (;;) {
    if (threadIdx.x == 0) next = static_cast<int>(atomicAdd(b.queue, 1u));
    __syncthreads();
    const int q = next;
    __syncthreads();
    if (q >= b.count) break;
    solve_instance<T>(b, b.order[q], sh);
  }
}

// ------------------------------------------------------------------------------------------
// Unrolled PDHG and its adjoint (the differentiable layer). Per instance (one CTA), K iterations
// of the fixed-step PDHG — tau = sigma = eta, primal weight 1, no restarts and no averaging —
// from zero on the equilibrated problem (the reference's step, pdlp.cpp:574-641):
//   y+ = y + sigma (A x_bar - r_bar);  v+ = P(v - tau (c + [A -I]' y+));  v_bar+ = 2 v+ - v
// with v = (x, r) and P the projection on [l, u]. The state (v, v_bar, y) is saved every
// `every` iterations. The adjoint recomputes each segment forward from its checkpoint, keeping
// for every projection which bound it met, then runs the transposed recurrences backwards:
//   V = v_hat + 2 b_hat;  z_hat = [l < z < u] V;  l_hat += [z <= l] V;  u_hat += [z >= u] V
//   v_hat' = z_hat - b_hat;  g_hat = -tau z_hat;  c_hat += g_hat
//   y_hat' = y_hat + [A -I] g_hat;  b_hat' = [A -I]' (sigma y_hat')
// (the costs, bounds and iterates map to the LpProblem's space by the column and row scales).

namespace {

struct UnrollPtrs {
  int m, n, nt;
  const int* kp;
  const int* ki;
  const double* kv;
  const int* tp;
  const int* ti;
  const double* tv;
  const double* cs;
  const double* rs;
  double eta;
  double* st;  // the instance's state storage (8 (n+m) + 4 m doubles)
  long long vo;
};

__device__ __forceinline__ UnrollPtrs unroll_ptrs(const BatchView& b, int inst) {
  UnrollPtrs p;
  const int g = b.inst_mat[inst];
  p.m = b.mat_m[g];
  p.n = b.mat_n[g];
  p.nt = p.n + p.m;
  const long long nz = b.mat_nnz_off[g];
  p.kp = b.k_ptr + b.mat_kptr_off[g];
  p.ki = b.k_idx + nz;
  p.kv = b.k_val + nz;
  p.tp = b.t_ptr + b.mat_tptr_off[g];
  p.ti = b.t_idx + nz;
  p.tv = b.t_val + nz;
  p.cs = b.cs + b.mat_col_off[g];
  p.rs = b.rs + b.mat_row_off[g];
  p.eta = b.info[g].eta;
  p.st = reinterpret_cast<double*>(b.state) + b.state_off[inst];
  p.vo = b.vec_off[inst];
  return p;
}

// The equilibrated cost and bounds of an instance into ce, le, ue.
__device__ void unroll_problem(const BatchView& b, const UnrollPtrs& p, double* ce, double* le,
                               double* ue) {
  const double* c0 = b.cost + p.vo;
  const double* l0 = b.lower + p.vo;
  const double* u0 = b.upper + p.vo;
  for (int k = threadIdx.x; k < p.nt; k += kBT) {
    if (k < p.n) {
      ce[k] = c0[k] * p.cs[k];
      le[k] = l0[k] / p.cs[k];
      ue[k] = u0[k] / p.cs[k];
    } else {
      const double r = p.rs[k - p.n];
      ce[k] = c0[k] * r;
      le[k] = l0[k] * r;
      ue[k] = u0[k] * r;
    }
  }
}

__device__ __forceinline__ unsigned char project(double z, double lo, double up, double* out) {
  if (z <= lo) {
    *out = lo;
    return 1;
  }
  if (z >= up) {
    *out = up;
    return 2;
  }
  *out = z;
  return 0;
}

// One fixed-step iteration on (v, vbar, y); `mask` (n+m bytes) records the projections when
// given.
__device__ void unroll_step(const UnrollPtrs& p, double* v, double* vbar, double* y,
                            const double* ce, const double* le, const double* ue,
                            unsigned char* mask) {
  const double tau = p.eta, sigma = p.eta;
  const int n = p.n;
  struct G {
    const double* x;
    __device__ double operator()(double a, int j) const { return a * x[j]; }
  };
  {
    G gx{vbar};
    auto f = [&](int i, double s) {
      const double yn = y[i] + sigma * (s - vbar[n + i]);
      y[i] = yn;
      const double r = v[n + i];
      double rn;
      const unsigned char c = project(r - tau * (ce[n + i] - yn), le[n + i], ue[n + i], &rn);
      if (mask != nullptr) mask[n + i] = c;
      v[n + i] = rn;
      vbar[n + i] = 2.0 * rn - r;
    };
    block_rows<false>(p.m, p.kp, p.ki, p.kv, gx, f);
  }
  __syncthreads();
  {
    G gy{y};
    auto f = [&](int j, double s) {
      const double x = v[j];
      double xn;
      const unsigned char c = project(x - tau * (ce[j] + s), le[j], ue[j], &xn);
      if (mask != nullptr) mask[j] = c;
      v[j] = xn;
      vbar[j] = 2.0 * xn - x;
    };
    block_rows<false>(n, p.tp, p.ti, p.tv, gy, f);
  }
  __syncthreads();
}

}  // namespace

__global__ void __launch_bounds__(kBT) unroll_forward_kernel(BatchView b, UnrollView u) {
  for (int inst = blockIdx.x; inst < b.count; inst += gridDim.x) {
    const UnrollPtrs p = unroll_ptrs(b, inst);
    const int nt = p.nt, m = p.m, n = p.n;
    double* v = p.st;
    double* vbar = p.st + 2 * nt;
    double* ce = p.st + 5 * nt;
    double* le = p.st + 6 * nt;
    double* ue = p.st + 7 * nt;
    double* y = p.st + 8 * nt;
    unroll_problem(b, p, ce, le, ue);
    for (int k = threadIdx.x; k < nt; k += kBT) {
      v[k] = 0.0;
      vbar[k] = 0.0;
      if (k < m) y[k] = 0.0;
    }
    __syncthreads();
    double* ck = u.ck + u.ck_off[inst];
    const int stride = 2 * nt + m;
    for (int it = 0; it < u.iterations; ++it) {
      if (it % u.every == 0) {
        double* c = ck + static_cast<long long>(it / u.every) * stride;
        for (int k = threadIdx.x; k < nt; k += kBT) {
          c[k] = v[k];
          c[nt + k] = vbar[k];
          if (k < m) c[2 * nt + k] = y[k];
        }
      }
      unroll_step(p, v, vbar, y, ce, le, ue, nullptr);
    }
    double* vo = u.v_out + p.vo;
    for (int k = threadIdx.x; k < nt; k += kBT) {
      vo[k] = k < n ? v[k] * p.cs[k] : v[k] / p.rs[k - n];
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kBT) unroll_adjoint_kernel(BatchView b, UnrollView u) {
  for (int inst = blockIdx.x; inst < b.count; inst += gridDim.x) {
    const UnrollPtrs p = unroll_ptrs(b, inst);
    const int nt = p.nt, m = p.m, n = p.n;
    const double tau = p.eta, sigma = p.eta;
    // Forward working state, the problem, and the adjoint state in the instance's storage.
    double* v = p.st;
    double* vh = p.st + nt;
    double* vbar = p.st + 2 * nt;
    double* bh = p.st + 3 * nt;
    double* gh = p.st + 4 * nt;
    double* ce = p.st + 5 * nt;
    double* le = p.st + 6 * nt;
    double* ue = p.st + 7 * nt;
    double* y = p.st + 8 * nt;
    double* yh = p.st + 8 * nt + m;
    double* shat = p.st + 8 * nt + 2 * m;
    double* gc = u.grad_cost + p.vo;
    double* gl = u.grad_lower + p.vo;
    double* gu = u.grad_upper + p.vo;
    const double* gv = u.grad_v + p.vo;
    unroll_problem(b, p, ce, le, ue);
    // Adjoint of v_K in the equilibrated space: x = x_eq cs, r = r_eq / rs.
    for (int k = threadIdx.x; k < nt; k += kBT) {
      vh[k] = k < n ? gv[k] * p.cs[k] : gv[k] / p.rs[k - n];
      bh[k] = 0.0;
      gc[k] = 0.0;
      gl[k] = 0.0;
      gu[k] = 0.0;
      if (k < m) yh[k] = 0.0;
    }
    __syncthreads();
    const double* ck = u.ck + u.ck_off[inst];
    unsigned char* mask = u.mask + u.mask_off[inst];
    const int stride = 2 * nt + m;
    struct G {
      const double* x;
      __device__ double operator()(double a, int j) const { return a * x[j]; }
    };
    for (int seg = u.nck - 1; seg >= 0; --seg) {
      const int k0 = seg * u.every;
      const int len = min(u.every, u.iterations - k0);
      const double* c = ck + static_cast<long long>(seg) * stride;
      for (int k = threadIdx.x; k < nt; k += kBT) {
        v[k] = c[k];
        vbar[k] = c[nt + k];
        if (k < m) y[k] = c[2 * nt + k];
      }
      __syncthreads();
      for (int t = 0; t < len; ++t) {
        unroll_step(p, v, vbar, y, ce, le, ue, mask + static_cast<long long>(t) * nt);
      }
      for (int t = len - 1; t >= 0; --t) {
        const unsigned char* mk = mask + static_cast<long long>(t) * nt;
        for (int k = threadIdx.x; k < nt; k += kBT) {
          const double V = vh[k] + 2.0 * bh[k];
          const unsigned char code = mk[k];
          const double zh = code == 0 ? V : 0.0;
          if (code == 1) gl[k] += V;
          if (code == 2) gu[k] += V;
          vh[k] = zh - bh[k];
          const double g = -tau * zh;
          gc[k] += g;
          gh[k] = g;
        }
        __syncthreads();
        {
          G gg{gh};
          auto f = [&](int i, double s) {
            const double yt = yh[i] + (s - gh[n + i]);
            yh[i] = yt;
            shat[i] = sigma * yt;
          };
          block_rows<false>(m, p.kp, p.ki, p.kv, gg, f);
        }
        __syncthreads();
        {
          G gs{shat};
          auto f = [&](int j, double s) { bh[j] = s; };
          block_rows<false>(n, p.tp, p.ti, p.tv, gs, f);
          for (int i = threadIdx.x; i < m; i += kBT) bh[n + i] = -shat[i];
        }
        __syncthreads();
      }
    }
    // Gradients in the LpProblem's space: c_eq = c s, l_eq = l / cs (columns), l rs (rows).
    for (int k = threadIdx.x; k < nt; k += kBT) {
      if (k < n) {
        const double s = p.cs[k];
        gc[k] *= s;
        gl[k] /= s;
        gu[k] /= s;
      } else {
        const double r = p.rs[k - n];
        gc[k] *= r;
        gl[k] *= r;
        gu[k] *= r;
      }
    }
    __syncthreads();
  }
}

__global__ void to_fp32_kernel(const double* a, float* o, long long count) {
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < count;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    o[k] = static_cast<float>(a[k]);
  }
}

__global__ void batch_deadline_kernel(unsigned long long* word, unsigned long long budget_ns) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long now;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
  *word = budget_ns == 0ull ? 0ull : now + budget_ns;
}

void launch_batch(const BatchView& b, int solve_grid, unsigned long long budget_ns,
                  cudaStream_t s) {
  batch_deadline_kernel<<<1, 32, 0, s>>>(const_cast<unsigned long long*>(b.deadline), budget_ns);
  cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
  batch_setup_kernel<<<b.nmat, kBT, 0, s>>>(b);
  if (b.fp32) {
    const long long nnz = b.total_nnz;
    const int g = static_cast<int>(nnz / 256 + 1 < 4096 ? nnz / 256 + 1 : 4096);
    to_fp32_kernel<<<g, 256, 0, s>>>(b.k_val, b.k_val32, nnz);
    to_fp32_kernel<<<g, 256, 0, s>>>(b.t_val, b.t_val32, nnz);
    batch_solve_kernel<float><<<solve_grid, kBT, 0, s>>>(b);
  } else {
    batch_solve_kernel<double><<<solve_grid, kBT, 0, s>>>(b);
  }
}

void launch_batch_setup(const BatchView& b, cudaStream_t s) {
  batch_setup_kernel<<<b.nmat, kBT, 0, s>>>(b);
}

void launch_unroll(const BatchView& b, const UnrollView& u, int adjoint, int grid,
                   cudaStream_t s) {
  if (adjoint) {
    unroll_adjoint_kernel<<<grid, kBT, 0, s>>>(b, u);
  } else {
    unroll_forward_kernel<<<grid, kBT, 0, s>>>(b, u);
  }
}

int batch_threads() { return kBT; }

}  // namespace sg
