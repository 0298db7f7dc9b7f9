// Kernels of the GB300 PDLP engine: the two fused PDHG step kernels, the evaluation kernels, the
// single-CTA decision kernels, restarts, infeasibility/unboundedness detection and the
// device-side setup (Ruiz, power iteration, norms).
//
// Reference algorithm: src/lp/pdlp.cpp (CPU loop and decisions) and src/gpu/pdhg_core.cu (its
// GPU arithmetic). Here every decision of the loop runs on the device, so a chunk of
// kCheckFrequency iterations plus its evaluation replays from one CUDA graph.
#include <math.h>

#include <type_traits>

#include "sg_kernels.cuh"
#include "sg_tile.cuh"

namespace sg {

namespace {

template <typename T>
__device__ __forceinline__ T clampv(T v, T lo, T hi) {
  return fmin(fmax(v, lo), hi);
}

// Doubles compared through their bit patterns mapped to a signed integer order, on the integer
// pipe (GB300's FP64 pipe is small): the same as fmin(fmax(v, lo), hi) for numbers (with
// -0 ordered below +0).
__device__ __forceinline__ long long order_key(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

template <>
__device__ __forceinline__ double clampv<double>(double v, double lo, double hi) {
  const double r = order_key(v) < order_key(lo) ? lo : v;
  return order_key(r) > order_key(hi) ? hi : r;
}

// The extrapolated point 2 v+ - v (one fused operation in FP64).
template <typename T>
__device__ __forceinline__ T extrapolate(T vn, T v) {
  return vn + (vn - v);
}

template <>
__device__ __forceinline__ double extrapolate<double>(double vn, double v) {
  return fma(2.0, vn, -v);
}

// lambda of the reduced cost g for a variable with bounds [lo, up] (pdlp.cpp:455-465).
__device__ __forceinline__ double bound_part(double g, double lo, double up) {
  const bool hl = lo > -INFINITY;
  const bool hu = up < INFINITY;
  return hl && hu ? g : hl ? fmax(g, 0.0) : hu ? fmin(g, 0.0) : 0.0;
}

template <typename T, typename ACC>
struct Gather1 {
  const T* x;
  __device__ __forceinline__ ACC operator()(int, T a, int j) const {
    return static_cast<ACC>(a) * static_cast<ACC>(ldg(x + j));
  }
};

template <typename T>
struct Gather2 {
  const T* x0;
  const T* x1;
  __device__ __forceinline__ double operator()(int v, T a, int j) const {
    return static_cast<double>(a) * static_cast<double>(ldg((v == 0 ? x0 : x1) + j));
  }
};

// ------------------------------------------------------------------------------------------
// Step kernels. One PDHG iteration (pdlp.cpp:574-641; pdhg_core.cu:23-50) is two launches:
//   dual   (rows of K):  y+ = y + sigma (K xbar - rbar - q); r+ = proj(r - tau (c_r - y+));
//                        rbar' = r+ + (r+ - r); averages of y and r
//   primal (rows of K'): x+ = proj(x - tau (c_x + K' y+)); xbar' = x+ + (x+ - x); average of x
// The extrapolation of the reference's first kernel is produced by the previous step's
// epilogue (xbar'), so the SpMV gathers one vector.

template <typename T, typename ACC>
struct DualEpi {
  const T* y;
  T* y_new;
  const T* vr;   // r (n offset applied)
  T* vr_new;
  T* vbar_r;
  const T* c;
  const T* l;
  const T* u;
  const T* q;
  T* yerg;
  T* verg_r;
  ACC sigma, tau, alpha, beta;
  struct Pre {
    ACC rbar, q, y, r, c, l, u, yerg, rerg;
  };
  __device__ __forceinline__ Pre load(int i) const {
    Pre p;
    p.rbar = static_cast<ACC>(vbar_r[i]);
    p.q = q != nullptr ? static_cast<ACC>(q[i]) : ACC(0);
    p.y = static_cast<ACC>(y[i]);
    p.r = static_cast<ACC>(vr[i]);
    p.c = static_cast<ACC>(c[i]);
    p.l = static_cast<ACC>(l[i]);
    p.u = static_cast<ACC>(u[i]);
    p.yerg = static_cast<ACC>(yerg[i]);
    p.rerg = static_cast<ACC>(verg_r[i]);
    return p;
  }
  __device__ __forceinline__ void row(int i, const ACC (&s)[1], const Pre& p) {
    ACC res = s[0] - p.rbar;
    if (q != nullptr) res -= p.q;
    const ACC yn = p.y + sigma * res;
    y_new[i] = static_cast<T>(yn);
    ACC rn = p.r - tau * (p.c - yn);
    rn = clampv<ACC>(rn, p.l, p.u);
    vr_new[i] = static_cast<T>(rn);
    vbar_r[i] = static_cast<T>(extrapolate<ACC>(rn, p.r));
    yerg[i] = static_cast<T>(beta * p.yerg + alpha * yn);
    verg_r[i] = static_cast<T>(beta * p.rerg + alpha * rn);
  }
  __device__ __forceinline__ void row(int i, const ACC (&s)[1]) { row(i, s, load(i)); }
  __device__ __forceinline__ void long_row(int, int i, const ACC (&s)[1]) { row(i, s); }
};

// The bounds of column j: the shared pair when every column has it (no loads), else the
// vectors.
template <typename T, typename ACC>
struct ColBounds {
  const T* l;
  const T* u;
  int uniform;
  ACC lo, hi;
  __device__ __forceinline__ void load(int j, ACC& pl, ACC& pu) const {
    if (uniform) {
      pl = lo;
      pu = hi;
    } else {
      pl = static_cast<ACC>(l[j]);
      pu = static_cast<ACC>(u[j]);
    }
  }
};

template <typename T, typename ACC>
__device__ __forceinline__ ColBounds<T, ACC> col_bounds(const IterView<T>& it) {
  return ColBounds<T, ACC>{it.lower, it.upper, it.xb_uniform, static_cast<ACC>(it.xb_lo),
                           static_cast<ACC>(it.xb_hi)};
}

template <typename T, typename ACC>
struct PrimalEpi {
  const T* x;
  T* x_new;
  T* xbar;
  const T* c;
  ColBounds<T, ACC> b;
  T* xerg;
  ACC tau, alpha, beta;
  struct Pre {
    ACC x, c, l, u, xerg;
  };
  __device__ __forceinline__ Pre load(int j) const {
    Pre p;
    p.x = static_cast<ACC>(x[j]);
    p.c = static_cast<ACC>(c[j]);
    b.load(j, p.l, p.u);
    p.xerg = static_cast<ACC>(xerg[j]);
    return p;
  }
  __device__ __forceinline__ void row(int j, const ACC (&s)[1], const Pre& p) {
    ACC xn = p.x - tau * (p.c + s[0]);
    xn = clampv<ACC>(xn, p.l, p.u);
    x_new[j] = static_cast<T>(xn);
    xbar[j] = static_cast<T>(extrapolate<ACC>(xn, p.x));
    xerg[j] = static_cast<T>(beta * p.xerg + alpha * xn);
  }
  __device__ __forceinline__ void row(int j, const ACC (&s)[1]) { row(j, s, load(j)); }
  __device__ __forceinline__ void long_row(int, int j, const ACC (&s)[1]) { row(j, s); }
};

template <typename T>
using Acc = T;  // FP64 storage accumulates in FP64, FP32 storage in FP32.

// The scalars of one step launch. FP64 kernels compute them once per CTA (thread 0) and share
// them: an FP64 division in every thread of thousands of CTAs kept GB300's small FP64 pipe
// busy. FP32 kernels compute the average weight in FP32 per thread.
template <typename ACC>
struct StepScalars {
  ACC sigma, tau, alpha, beta;
};

template <typename ACC>
__device__ __forceinline__ StepScalars<ACC> step_scalars(const Ctl* __restrict__ ctl,
                                                         long long k) {
  if constexpr (std::is_same<ACC, double>::value) {
    __shared__ StepScalars<double> sh;
    if (threadIdx.x == 0) {
      const double alpha = 1.0 / static_cast<double>(k + 1);
      sh.sigma = ctl->sigma;
      sh.tau = ctl->tau;
      sh.alpha = alpha;
      sh.beta = 1.0 - alpha;
    }
    __syncthreads();
    return sh;
  } else {
    // FP32: lane 0 of each warp converts and divides, the warp shuffles the results (the
    // shared-memory broadcast above put a dependent load and a barrier in front of every CTA's
    // first load: slower; per thread, the FP64 -> FP32 and 64-bit integer conversions ran on
    // the FP64 pipe in every thread). Every lane is active at kernel entry.
    StepScalars<ACC> s{};
    if ((threadIdx.x & 31) == 0) {
      s.sigma = static_cast<ACC>(ctl->sigma);
      s.tau = static_cast<ACC>(ctl->tau);
      s.alpha = ACC(1) / static_cast<ACC>(k + 1);
      s.beta = ACC(1) - s.alpha;
    }
    s.sigma = __shfl_sync(0xffffffffu, s.sigma, 0);
    s.tau = __shfl_sync(0xffffffffu, s.tau, 0);
    s.alpha = __shfl_sync(0xffffffffu, s.alpha, 0);
    s.beta = __shfl_sync(0xffffffffu, s.beta, 0);
    return s;
  }
}

// Two variants of each step kernel (TileSet::variant, one per operator, picked by the tile
// tuner or the built-in rule):
//   0: many CTAs per SM resident (operators of short rows, where occupancy hides the latency),
//      as many as fit without spills: the primal step 6 (40 registers) in FP32 and 5 (48) in
//      FP64; the dual step, whose epilogue preloads eight or nine row values, 5 in FP32 and 4
//      (64) in FP64 (a few bytes spill; at 3 per SM, spill-free, the power-law LP's FP64 dual
//      step took 108 us instead of 92);
//   1: 128 registers, the warp-per-row and segment loops unrolled twice as deep (operators of
//      long rows, whose few CTAs need more loads in flight each; at 3 CTAs per SM, 80
//      registers, no faster on the transportation LP);
//   2 (dual steps only): variant 0 plus the kind-3 row groups and the staged kind-1 segments
//      of a tile set that has them.
// (Measured and not kept: a third variant loading a short row's first three pairs of
// nonzeros together at 4 CTAs per SM; no faster on the transportation or power-law LPs.)
template <typename T>
constexpr int step_min_blocks(int variant, bool dual) {
  if (variant == 1) return 2;
  if (variant == 2) return sizeof(T) == 8 ? 3 : 4;
  if (sizeof(T) == 8) return dual ? 4 : 5;
  return dual ? 5 : 6;
}

template <typename T, int VAR>
__global__ void __launch_bounds__(kBlock, step_min_blocks<T>(VAR, true)) dual_step_kernel(
    const Ctl* __restrict__ ctl, OpView<T> K, IterView<T> it, int j) {
  if (ctl->done) return;
  const long long t = ctl->t + j;
  if (t >= ctl->max_iter) return;
  using ACC = Acc<T>;
  const int p = static_cast<int>(t & 1);
  const long long k = ctl->k + j;
  const StepScalars<ACC> sc = step_scalars<ACC>(ctl, k);
  DualEpi<T, ACC> epi;
  const int n = it.n;
  epi.y = it.y(p);
  epi.y_new = it.y(p ^ 1);
  epi.vr = it.v(p) + n;
  epi.vr_new = it.v(p ^ 1) + n;
  epi.vbar_r = it.Vbar + n;
  epi.c = it.cost + n;
  epi.l = it.lower + n;
  epi.u = it.upper + n;
  epi.q = it.rhs;
  epi.yerg = it.Yerg;
  epi.verg_r = it.Verg + n;
  epi.sigma = sc.sigma;
  epi.tau = sc.tau;
  epi.alpha = sc.alpha;
  epi.beta = sc.beta;
  Gather1<T, ACC> g{it.Vbar};
  run_tiles<T, ACC, 1, Gather1<T, ACC>, DualEpi<T, ACC>, false, VAR == 1, VAR == 2>(
      K.ts, K.ptr, K.idx, K.val, g, epi);
}

template <typename T, int VAR>
__global__ void __launch_bounds__(kBlock, step_min_blocks<T>(VAR, false)) primal_step_kernel(
    const Ctl* __restrict__ ctl, OpView<T> Kt, IterView<T> it, int j) {
  if (ctl->done) return;
  const long long t = ctl->t + j;
  if (t >= ctl->max_iter) return;
  using ACC = Acc<T>;
  const int p = static_cast<int>(t & 1);
  const long long k = ctl->k + j;
  const StepScalars<ACC> sc = step_scalars<ACC>(ctl, k);
  PrimalEpi<T, ACC> epi;
  epi.x = it.v(p);
  epi.x_new = it.v(p ^ 1);
  epi.xbar = it.Vbar;
  epi.c = it.cost;
  epi.b = col_bounds<T, ACC>(it);
  epi.xerg = it.Verg;
  epi.tau = sc.tau;
  epi.alpha = sc.alpha;
  epi.beta = sc.beta;
  Gather1<T, ACC> g{it.y(p ^ 1)};
  run_tiles<T, ACC, 1, Gather1<T, ACC>, PrimalEpi<T, ACC>, false, VAR == 1>(
      Kt.ts, Kt.ptr, Kt.idx, Kt.val, g, epi);
}

// ------------------------------------------------------------------------------------------
// Reflected Halpern PDHG (the engine's SG_ALGORITHM_HALPERN; no reference counterpart). With
// T the PDHG map z = (v, y) -> (v^, y^) (primal first: v^ = proj(v - tau (c - K'y)),
// y^ = y + sigma (K (2 v^ - v) - q)) and z0 the point of the last restart, one iteration is
//   z+ = lambda (2 T(z) - z) + (1 - lambda) z0,  lambda = (k + 1) / (k + 2)
// (Halpern's iteration on the reflected map 2T - I, nonexpansive, so z -> a fixed point of T).
// The primal launch runs first: x^ and the reflected 2 x^ - x (written to Vbar, the dual
// launch's SpMV input) and x+ from y; then the dual launch: the logicals' r^ from the old y,
// y^, and r+, y+. T(z) lands in Verg / Yerg, the evaluation's second iterate and the answer.

// z+ = N + w (z0 - N) with N = 2 z^ - z the reflected point and w = 1 - lambda = 1 / (k + 2).
template <typename ACC>
__device__ __forceinline__ ACC halpern_mix(ACC reflected, ACC z0, ACC w) {
  return reflected + w * (z0 - reflected);
}

template <>
__device__ __forceinline__ double halpern_mix<double>(double reflected, double z0, double w) {
  return fma(w, z0 - reflected, reflected);
}

// T(z) is read only by the evaluation after a chunk's last step (and by the restart, the
// precision switch and the answer, all after an evaluation), so only that step writes it: the
// chunk's last launch, or the step that reaches max_iter. Saves one vector write per
// iteration (8 MB of the 104 MB an FP32 primal step of the transportation LP moves).
__device__ __forceinline__ bool halpern_writes_hat(const Ctl* ctl, long long t, int j) {
  return j == kCheckFrequency - 1 || t + 1 >= ctl->max_iter;
}

template <typename T, typename ACC>
struct HalpernPrimalEpi {
  const T* x;
  T* x_new;
  T* xbar;   // 2 x^ - x, the dual launch's SpMV input
  T* xhat;   // x^ (T(z)'s primal part), written only when `hat`
  const T* x0;
  const T* c;
  ColBounds<T, ACC> b;
  ACC tau, w;
  bool hat;
  struct Pre {
    ACC x, c, l, u, x0;
  };
  __device__ __forceinline__ Pre load(int j) const {
    Pre p;
    p.x = static_cast<ACC>(x[j]);
    p.c = static_cast<ACC>(c[j]);
    b.load(j, p.l, p.u);
    p.x0 = static_cast<ACC>(x0[j]);
    return p;
  }
  __device__ __forceinline__ void row(int j, const ACC (&s)[1], const Pre& p) {
    const ACC xh = clampv<ACC>(p.x - tau * (p.c + s[0]), p.l, p.u);
    const ACC refl = extrapolate<ACC>(xh, p.x);
    if (hat) xhat[j] = static_cast<T>(xh);
    xbar[j] = static_cast<T>(refl);
    x_new[j] = static_cast<T>(halpern_mix<ACC>(refl, p.x0, w));
  }
  __device__ __forceinline__ void row(int j, const ACC (&s)[1]) { row(j, s, load(j)); }
  __device__ __forceinline__ void long_row(int, int j, const ACC (&s)[1]) { row(j, s); }
};

template <typename T, typename ACC>
struct HalpernDualEpi {
  const T* y;
  T* y_new;
  T* yhat;
  const T* y0;
  const T* vr;   // r (n offset applied)
  T* vr_new;
  T* vr_hat;
  const T* r0;
  const T* c;
  const T* l;
  const T* u;
  const T* q;
  ACC sigma, tau, w;
  bool hat;  // write T(z) (y^, r^)
  struct Pre {
    ACC y, r, c, l, u, q, y0, r0;
  };
  __device__ __forceinline__ Pre load(int i) const {
    Pre p;
    p.y = static_cast<ACC>(y[i]);
    p.r = static_cast<ACC>(vr[i]);
    p.c = static_cast<ACC>(c[i]);
    p.l = static_cast<ACC>(l[i]);
    p.u = static_cast<ACC>(u[i]);
    p.q = q != nullptr ? static_cast<ACC>(q[i]) : ACC(0);
    p.y0 = static_cast<ACC>(y0[i]);
    p.r0 = static_cast<ACC>(r0[i]);
    return p;
  }
  __device__ __forceinline__ void row(int i, const ACC (&s)[1], const Pre& p) {
    // The logical's primal step uses the old dual (primal first), then the dual step sees the
    // row's reflected logical: K (2 v^ - v) = A (2 x^ - x) - (2 r^ - r).
    const ACC rh = clampv<ACC>(p.r - tau * (p.c - p.y), p.l, p.u);
    const ACC rrefl = extrapolate<ACC>(rh, p.r);
    ACC res = s[0] - rrefl;
    if (q != nullptr) res -= p.q;
    const ACC yh = p.y + sigma * res;
    if (hat) {
      yhat[i] = static_cast<T>(yh);
      vr_hat[i] = static_cast<T>(rh);
    }
    y_new[i] = static_cast<T>(halpern_mix<ACC>(extrapolate<ACC>(yh, p.y), p.y0, w));
    vr_new[i] = static_cast<T>(halpern_mix<ACC>(rrefl, p.r0, w));
  }
  __device__ __forceinline__ void row(int i, const ACC (&s)[1]) { row(i, s, load(i)); }
  __device__ __forceinline__ void long_row(int, int i, const ACC (&s)[1]) { row(i, s); }
};

template <typename T, int VAR>
__global__ void __launch_bounds__(kBlock, step_min_blocks<T>(VAR, false)) halpern_primal_kernel(
    const Ctl* __restrict__ ctl, OpView<T> Kt, IterView<T> it, int j) {
  if (ctl->done) return;
  const long long t = ctl->t + j;
  if (t >= ctl->max_iter) return;
  using ACC = Acc<T>;
  const int p = static_cast<int>(t & 1);
  // alpha = 1 / (k' + 1) with k' = k + 1: the Halpern weight 1 / (k + 2).
  const StepScalars<ACC> sc = step_scalars<ACC>(ctl, ctl->k + j + 1);
  HalpernPrimalEpi<T, ACC> epi;
  epi.x = it.v(p);
  epi.x_new = it.v(p ^ 1);
  epi.xbar = it.Vbar;
  epi.xhat = it.Verg;
  epi.x0 = it.Vrst;
  epi.c = it.cost;
  epi.b = col_bounds<T, ACC>(it);
  epi.tau = sc.tau;
  epi.w = sc.alpha;
  epi.hat = halpern_writes_hat(ctl, t, j);
  Gather1<T, ACC> g{it.y(p)};
  run_tiles<T, ACC, 1, Gather1<T, ACC>, HalpernPrimalEpi<T, ACC>, false, VAR == 1>(
      Kt.ts, Kt.ptr, Kt.idx, Kt.val, g, epi);
}

template <typename T, int VAR>
__global__ void __launch_bounds__(kBlock, step_min_blocks<T>(VAR, true)) halpern_dual_kernel(
    const Ctl* __restrict__ ctl, OpView<T> K, IterView<T> it, int j) {
  if (ctl->done) return;
  const long long t = ctl->t + j;
  if (t >= ctl->max_iter) return;
  using ACC = Acc<T>;
  const int p = static_cast<int>(t & 1);
  const StepScalars<ACC> sc = step_scalars<ACC>(ctl, ctl->k + j + 1);
  HalpernDualEpi<T, ACC> epi;
  const int n = it.n;
  epi.y = it.y(p);
  epi.y_new = it.y(p ^ 1);
  epi.yhat = it.Yerg;
  epi.y0 = it.Yrst;
  epi.vr = it.v(p) + n;
  epi.vr_new = it.v(p ^ 1) + n;
  epi.vr_hat = it.Verg + n;
  epi.r0 = it.Vrst + n;
  epi.c = it.cost + n;
  epi.l = it.lower + n;
  epi.u = it.upper + n;
  epi.q = it.rhs;
  epi.sigma = sc.sigma;
  epi.tau = sc.tau;
  epi.w = sc.alpha;
  epi.hat = halpern_writes_hat(ctl, t, j);
  Gather1<T, ACC> g{it.Vbar};
  run_tiles<T, ACC, 1, Gather1<T, ACC>, HalpernDualEpi<T, ACC>, false, VAR == 1, VAR == 2>(
      K.ts, K.ptr, K.idx, K.val, g, epi);
}

// ------------------------------------------------------------------------------------------
// Evaluation (pdhg_core.cu:102-144 / pdlp.cpp:411-488): the seven sums of the current and the
// average iterate in the space before equilibration, plus the restart distances, from one
// pass over each operator (both iterates share the matrix read). W0 = 1 measures the second
// slot alone (the Halpern solves decide on T(z) only; the current iterate's sums stay 0).

template <typename T, int W0 = 0>
struct EvalRowEpi {
  // rows of K: logicals r and duals y
  const T* vr[2];
  const T* y[2];
  const T* vr_rst;
  const T* y_rst;
  EvalView ev;
  int n;
  double acc[kEvalSums];
  double* long_terms;
  __device__ __forceinline__ void terms(int i, const double (&s)[2 - W0],
                                        double (&a)[kEvalSums]) {
    const double rs = ev.rs[i];
    const double irs = ev.inv_rs[i];
    const double c = ev.cost[n + i];
    const double lo = ev.lower[n + i];
    const double up = ev.upper[n + i];
    const double q = ev.rhs != nullptr ? ev.rhs[i] : 0.0;
#pragma unroll
    for (int w = W0; w < 2; ++w) {
      const double vrv = static_cast<double>(vr[w][i]);
      const double yv = static_cast<double>(y[w][i]);
      const double value = vrv * irs;
      const double yo = yv * rs;
      const double g = c - yo;
      const double e = s[w - W0] * irs - value - q;
      a[w * 7 + 0] += e * e;
      a[w * 7 + 5] += value * value;
      a[w * 7 + 6] += yo * yo;
      a[w * 7 + 2] += c * value;
      const double lam = bound_part(g, lo, up);
      a[w * 7 + 1] += (g - lam) * (g - lam);
      if (lam > 0.0) a[w * 7 + 3] += lam * lo;
      if (lam < 0.0) a[w * 7 + 3] += lam * up;
      // With a right-hand side ([A -I] v = q) the dual objective carries -y'q.
      if (q != 0.0) a[w * 7 + 3] -= yo * q;
      const double dv = vrv - static_cast<double>(vr_rst[i]);
      const double dy = yv - static_cast<double>(y_rst[i]);
      a[14 + 2 * w] += dv * dv;
      a[15 + 2 * w] += dy * dy;
    }
  }
  __device__ __forceinline__ void row(int i, const double (&s)[2 - W0]) { terms(i, s, acc); }
  __device__ __forceinline__ void long_row(int lrow, int i, const double (&s)[2 - W0]) {
    double a[kEvalSums];
#pragma unroll
    for (int q = 0; q < kEvalSums; ++q) a[q] = 0.0;
    terms(i, s, a);
#pragma unroll
    for (int q = 0; q < kEvalSums; ++q) long_terms[lrow * kMaxSums + q] = a[q];
  }
};

template <typename T, int W0 = 0>
struct EvalColEpi {
  // rows of K': structurals x
  const T* x[2];
  const T* x_rst;
  EvalView ev;
  int m;
  double acc[kEvalSums];
  double* long_terms;
  __device__ __forceinline__ void terms(int j, const double (&s)[2 - W0],
                                        double (&a)[kEvalSums]) {
    const double cs = ev.cs[j];
    const double ics = ev.inv_cs[j];
    const double c = ev.cost[j];
    const double lo = ev.lower[j];
    const double up = ev.upper[j];
#pragma unroll
    for (int w = W0; w < 2; ++w) {
      const double xv = static_cast<double>(x[w][j]);
      const double value = xv * cs;
      const double g = c + (m > 0 ? s[w - W0] * ics : 0.0);
      a[w * 7 + 4] += value * value;
      a[w * 7 + 2] += c * value;
      const double lam = bound_part(g, lo, up);
      a[w * 7 + 1] += (g - lam) * (g - lam);
      if (lam > 0.0) a[w * 7 + 3] += lam * lo;
      if (lam < 0.0) a[w * 7 + 3] += lam * up;
      const double dv = xv - static_cast<double>(x_rst[j]);
      a[14 + 2 * w] += dv * dv;
    }
  }
  __device__ __forceinline__ void row(int j, const double (&s)[2 - W0]) { terms(j, s, acc); }
  __device__ __forceinline__ void long_row(int lrow, int j, const double (&s)[2 - W0]) {
    double a[kEvalSums];
#pragma unroll
    for (int q = 0; q < kEvalSums; ++q) a[q] = 0.0;
    terms(j, s, a);
#pragma unroll
    for (int q = 0; q < kEvalSums; ++q) long_terms[lrow * kMaxSums + q] = a[q];
  }
};

// Stores the grid totals (the split rows' terms are added by grid_reduce).
struct EvalFin {
  double* out;
  __device__ __forceinline__ void operator()(const double (&tot)[kEvalSums]) const {
    for (int q = 0; q < kEvalSums; ++q) out[q] = tot[q];
  }
};

__device__ __forceinline__ int eval_parity(const Ctl* ctl, int fixed_parity) {
  if (fixed_parity >= 0) return fixed_parity;
  long long steps = ctl->max_iter - ctl->t;
  if (steps > kCheckFrequency) steps = kCheckFrequency;
  return static_cast<int>((ctl->t + steps) & 1);
}

template <typename T, int W0>
__global__ void __launch_bounds__(kBlock) eval_rows_kernel(Ctl* ctl, OpView<T> K, IterView<T> it,
                                                           EvalView ev, RedView red,
                                                           int fixed_parity) {
  if (fixed_parity < 0 && ctl->done) return;
  const int cur = eval_parity(ctl, fixed_parity);
  EvalRowEpi<T, W0> epi;
  const int n = it.n;
  epi.vr[0] = it.v(cur) + n;
  epi.vr[1] = it.Verg + n;
  epi.y[0] = it.y(cur);
  epi.y[1] = it.Yerg;
  epi.vr_rst = it.Vrst + n;
  epi.y_rst = it.Yrst;
  epi.ev = ev;
  epi.n = n;
  epi.long_terms = red.long_terms;
#pragma unroll
  for (int q = 0; q < kEvalSums; ++q) epi.acc[q] = 0.0;
  if constexpr (W0 == 0) {
    Gather2<T> g{it.v(cur), it.Verg};
    run_tiles<T, double, 2>(K.ts, K.ptr, K.idx, K.val, g, epi);
  } else {
    Gather1<T, double> g{it.Verg};
    run_tiles<T, double, 1>(K.ts, K.ptr, K.idx, K.val, g, epi);
  }
  EvalFin fin{ctl->eval_r};
  grid_reduce<kEvalSums>(epi.acc, red.partial, red.counter, smem_red(), fin, red.long_terms,
                         K.ts.nlong);
}

template <typename T, int W0>
__global__ void __launch_bounds__(kBlock) eval_cols_kernel(Ctl* ctl, OpView<T> Kt, IterView<T> it,
                                                           EvalView ev, RedView red,
                                                           int fixed_parity) {
  if (fixed_parity < 0 && ctl->done) return;
  const int cur = eval_parity(ctl, fixed_parity);
  EvalColEpi<T, W0> epi;
  epi.x[0] = it.v(cur);
  epi.x[1] = it.Verg;
  epi.x_rst = it.Vrst;
  epi.ev = ev;
  epi.m = it.m;
  epi.long_terms = red.long_terms;
#pragma unroll
  for (int q = 0; q < kEvalSums; ++q) epi.acc[q] = 0.0;
  if constexpr (W0 == 0) {
    Gather2<T> g{it.y(cur), it.Yerg};
    run_tiles<T, double, 2>(Kt.ts, Kt.ptr, Kt.idx, Kt.val, g, epi);
  } else {
    Gather1<T, double> g{it.Yerg};
    run_tiles<T, double, 1>(Kt.ts, Kt.ptr, Kt.idx, Kt.val, g, epi);
  }
  EvalFin fin{ctl->eval_c};
  grid_reduce<kEvalSums>(epi.acc, red.partial, red.counter, smem_red(), fin, red.long_terms,
                         Kt.ts.nlong);
}

// The same sums for an FP32 operator, which is always an inner problem already in its own
// equilibrated space (unit scales) with its own FP32 cost, bounds and right-hand side: FP32
// products, row sums and terms (GB300's FP64 rate is a small fraction of its FP32 rate, and FP64
// terms made these kernels arithmetic-bound), FP64 grid totals. Precision ~1e-6 relative is
// ample for the inner tolerance; the refined point is assessed by the FP64 evaluation above.

__device__ __forceinline__ float bound_part32(float g, float lo, float up) {
  const bool hl = lo > -INFINITY;
  const bool hu = up < INFINITY;
  return hl && hu ? g : hl ? fmaxf(g, 0.0f) : hu ? fminf(g, 0.0f) : 0.0f;
}

struct Gather2f {
  const float* x0;
  const float* x1;
  __device__ __forceinline__ float operator()(int v, float a, int j) const {
    return a * ldg((v == 0 ? x0 : x1) + j);
  }
};

template <int W0 = 0>
struct EvalRowEpi32 {
  const float* vr[2];
  const float* y[2];
  const float* vr_rst;
  const float* y_rst;
  const float* c;  // row parts (n offset applied)
  const float* l;
  const float* u;
  const float* q;
  float acc[kEvalSums];
  double* long_terms;
  __device__ __forceinline__ void terms(int i, const float (&s)[2 - W0], float (&a)[kEvalSums]) {
    const float c_i = c[i];
    const float lo = l[i];
    const float up = u[i];
    const float q_i = q != nullptr ? q[i] : 0.0f;
#pragma unroll
    for (int w = W0; w < 2; ++w) {
      const float value = vr[w][i];
      const float yv = y[w][i];
      const float g = c_i - yv;
      const float e = s[w - W0] - value - q_i;
      a[w * 7 + 0] += e * e;
      a[w * 7 + 5] += value * value;
      a[w * 7 + 6] += yv * yv;
      a[w * 7 + 2] += c_i * value;
      const float lam = bound_part32(g, lo, up);
      a[w * 7 + 1] += (g - lam) * (g - lam);
      if (lam > 0.0f) a[w * 7 + 3] += lam * lo;
      if (lam < 0.0f) a[w * 7 + 3] += lam * up;
      a[w * 7 + 3] -= yv * q_i;
      const float dv = value - vr_rst[i];
      const float dy = yv - y_rst[i];
      a[14 + 2 * w] += dv * dv;
      a[15 + 2 * w] += dy * dy;
    }
  }
  __device__ __forceinline__ void row(int i, const float (&s)[2 - W0]) { terms(i, s, acc); }
  __device__ __forceinline__ void long_row(int lrow, int i, const float (&s)[2 - W0]) {
    float a[kEvalSums];
#pragma unroll
    for (int q2 = 0; q2 < kEvalSums; ++q2) a[q2] = 0.0f;
    terms(i, s, a);
#pragma unroll
    for (int q2 = 0; q2 < kEvalSums; ++q2) long_terms[lrow * kMaxSums + q2] = a[q2];
  }
};

template <int W0 = 0>
struct EvalColEpi32 {
  const float* x[2];
  const float* x_rst;
  const float* c;
  const float* l;
  const float* u;
  int m;
  float acc[kEvalSums];
  double* long_terms;
  __device__ __forceinline__ void terms(int j, const float (&s)[2 - W0], float (&a)[kEvalSums]) {
    const float c_j = c[j];
    const float lo = l[j];
    const float up = u[j];
#pragma unroll
    for (int w = W0; w < 2; ++w) {
      const float value = x[w][j];
      const float g = c_j + (m > 0 ? s[w - W0] : 0.0f);
      a[w * 7 + 4] += value * value;
      a[w * 7 + 2] += c_j * value;
      const float lam = bound_part32(g, lo, up);
      a[w * 7 + 1] += (g - lam) * (g - lam);
      if (lam > 0.0f) a[w * 7 + 3] += lam * lo;
      if (lam < 0.0f) a[w * 7 + 3] += lam * up;
      const float dv = value - x_rst[j];
      a[14 + 2 * w] += dv * dv;
    }
  }
  __device__ __forceinline__ void row(int j, const float (&s)[2 - W0]) { terms(j, s, acc); }
  __device__ __forceinline__ void long_row(int lrow, int j, const float (&s)[2 - W0]) {
    float a[kEvalSums];
#pragma unroll
    for (int q2 = 0; q2 < kEvalSums; ++q2) a[q2] = 0.0f;
    terms(j, s, a);
#pragma unroll
    for (int q2 = 0; q2 < kEvalSums; ++q2) long_terms[lrow * kMaxSums + q2] = a[q2];
  }
};

template <int W0>
__global__ void __launch_bounds__(kBlock) eval_rows32_kernel(Ctl* ctl, OpView<float> K,
                                                             IterView<float> it, RedView red,
                                                             int fixed_parity) {
  if (fixed_parity < 0 && ctl->done) return;
  const int cur = eval_parity(ctl, fixed_parity);
  const int n = it.n;
  EvalRowEpi32<W0> epi;
  epi.vr[0] = it.v(cur) + n;
  epi.vr[1] = it.Verg + n;
  epi.y[0] = it.y(cur);
  epi.y[1] = it.Yerg;
  epi.vr_rst = it.Vrst + n;
  epi.y_rst = it.Yrst;
  epi.c = it.cost + n;
  epi.l = it.lower + n;
  epi.u = it.upper + n;
  epi.q = it.rhs;
  epi.long_terms = red.long_terms;
#pragma unroll
  for (int q = 0; q < kEvalSums; ++q) epi.acc[q] = 0.0f;
  if constexpr (W0 == 0) {
    Gather2f g{it.v(cur), it.Verg};
    run_tiles<float, float, 2>(K.ts, K.ptr, K.idx, K.val, g, epi);
  } else {
    Gather1<float, float> g{it.Verg};
    run_tiles<float, float, 1>(K.ts, K.ptr, K.idx, K.val, g, epi);
  }
  double acc[kEvalSums];
#pragma unroll
  for (int q = 0; q < kEvalSums; ++q) acc[q] = epi.acc[q];
  EvalFin fin{ctl->eval_r};
  grid_reduce<kEvalSums>(acc, red.partial, red.counter, smem_red(), fin, red.long_terms,
                         K.ts.nlong);
}

template <int W0>
__global__ void __launch_bounds__(kBlock) eval_cols32_kernel(Ctl* ctl, OpView<float> Kt,
                                                             IterView<float> it, RedView red,
                                                             int fixed_parity) {
  if (fixed_parity < 0 && ctl->done) return;
  const int cur = eval_parity(ctl, fixed_parity);
  EvalColEpi32<W0> epi;
  epi.x[0] = it.v(cur);
  epi.x[1] = it.Verg;
  epi.x_rst = it.Vrst;
  epi.c = it.cost;
  epi.l = it.lower;
  epi.u = it.upper;
  epi.m = it.m;
  epi.long_terms = red.long_terms;
#pragma unroll
  for (int q = 0; q < kEvalSums; ++q) epi.acc[q] = 0.0f;
  if constexpr (W0 == 0) {
    Gather2f g{it.y(cur), it.Yerg};
    run_tiles<float, float, 2>(Kt.ts, Kt.ptr, Kt.idx, Kt.val, g, epi);
  } else {
    Gather1<float, float> g{it.Yerg};
    run_tiles<float, float, 1>(Kt.ts, Kt.ptr, Kt.idx, Kt.val, g, epi);
  }
  double acc[kEvalSums];
#pragma unroll
  for (int q = 0; q < kEvalSums; ++q) acc[q] = epi.acc[q];
  EvalFin fin{ctl->eval_c};
  grid_reduce<kEvalSums>(acc, red.partial, red.counter, smem_red(), fin, red.long_terms,
                         Kt.ts.nlong);
}

// ------------------------------------------------------------------------------------------
// Decisions (pdlp.cpp:493-541, 674-713, 1069-1131), one thread.

struct Meas {
  double rp, rd, rg, pobj, dobj;
};

__device__ Meas finish_sums(const Ctl* c, const double* s) {
  // s = (primal_sq, dual_sq, primal_obj, dual_obj, x_sq, r_sq, y_sq)
  Meas r;
  const double primal_res = sqrt(s[0]);
  const double dual_res = sqrt(s[1]);
  const double gap = s[2] - s[3];
  const double primal_scale = 1.0 + c->a_norm_max_col * sqrt(s[4]) + sqrt(s[5]) + c->q_norm;
  const double dual_scale = 1.0 + c->at_norm_max_row * sqrt(s[6]) + c->c_norm;
  const double gap_scale = 1.0 + fabs(s[2]) + fabs(s[3]);
  r.rp = c->m > 0 ? primal_res / primal_scale : 0.0;
  r.rd = c->m > 0 ? dual_res / dual_scale : 0.0;
  r.rg = gap / gap_scale;
  r.pobj = s[2];
  r.dobj = s[3];
  return r;
}

__device__ __forceinline__ double kkt_weighted(double omega, const Meas& e) {
  return sqrt(omega * omega * e.rp * e.rp + e.rd * e.rd / (omega * omega) + e.rg * e.rg);
}

__device__ __forceinline__ bool converged(const Meas& e, double tol) {
  return e.rp < tol && e.rd < tol && fabs(e.rg) < tol;
}

__device__ void set_answer(Ctl* c, int status, const Meas& e, long long iterations, int avg) {
  c->status = status;
  c->res[0] = e.rp;
  c->res[1] = e.rd;
  c->res[2] = e.rg;
  c->pobj = e.pobj;
  c->dobj = e.dobj;
  c->iterations = iterations;
  c->result_average = avg;
  c->done = 1;
}

// Termination test after the evaluation; schedules the detection checks.
__global__ void decide_a_kernel(Ctl* c) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  c->restart_pending = 0;
  c->detect_pending = 0;
  if (c->done) return;
  long long steps = c->max_iter - c->t;
  if (steps > kCheckFrequency) steps = kCheckFrequency;
  const long long t_new = c->t + steps;
  const long long iter = t_new - 1;
  double s_cur[7], s_avg[7];
  for (int q = 0; q < 7; ++q) {
    s_cur[q] = c->eval_c[q] + c->eval_r[q];
    s_avg[q] = c->eval_c[7 + q] + c->eval_r[7 + q];
  }
  const Meas cur = finish_sums(c, s_cur);
  const Meas avg = finish_sums(c, s_avg);
  c->evaluations += 1;
  const double wc[5] = {cur.rp, cur.rd, cur.rg, cur.pobj, cur.dobj};
  const double wa[5] = {avg.rp, avg.rd, avg.rg, avg.pobj, avg.dobj};
  for (int q = 0; q < 5; ++q) {
    c->meas[0][q] = wc[q];
    c->meas[1][q] = wa[q];
  }
  if (!c->halpern && converged(cur, c->tol)) {
    set_answer(c, kOptimal, cur, t_new, 0);
    c->t = t_new;
    return;
  }
  if (converged(avg, c->tol)) {
    set_answer(c, kOptimal, avg, t_new, 1);
    c->t = t_new;
    return;
  }
  if (c->stall_limit > 0) {
    const double ec = fmax(fmax(cur.rp, cur.rd), fabs(cur.rg));
    const double ea = fmax(fmax(avg.rp, avg.rd), fabs(avg.rg));
    const bool use_avg = c->halpern || ea < ec;
    const double e = use_avg ? ea : ec;
    if (e < 0.8 * c->stall_best) {
      c->stall_best = e;
      c->stall_evals = 0;
    } else if (++c->stall_evals >= (e < c->stall_floor ? c->stall_limit : 8 * c->stall_limit)) {
      set_answer(c, kIterationLimit, use_avg ? avg : cur, t_new, use_avg ? 1 : 0);
      c->t = t_new;
      return;
    }
  }
  c->detect_pending =
      (!c->no_detect && iter > 1000 && c->m > 0 && ((iter + 1) / kCheckFrequency) % 8 == 0) ? 1
                                                                                              : 0;
  for (int q = 0; q < 8; ++q) c->det_flags[q] = 0;
}

// Detection verdict, then PDLP's adaptive restart and primal-weight update; advances the
// iteration counters and applies the iteration and time limits.
__global__ void decide_b_kernel(Ctl* c) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (c->done) return;
  long long steps = c->max_iter - c->t;
  if (steps > kCheckFrequency) steps = kCheckFrequency;
  const long long t_new = c->t + steps;
  const long long iter = t_new - 1;
  Meas cur{c->meas[0][0], c->meas[0][1], c->meas[0][2], c->meas[0][3], c->meas[0][4]};
  Meas avg{c->meas[1][0], c->meas[1][1], c->meas[1][2], c->meas[1][3], c->meas[1][4]};
  if (c->detect_pending) {
    if (c->det_flags[0]) {
      set_answer(c, kInfeasible, cur, t_new, 0);
      c->t = t_new;
      return;
    }
    if (c->det_flags[1]) {
      set_answer(c, kUnbounded, cur, t_new, 0);
      c->t = t_new;
      return;
    }
  }
  const long long k_new = c->k + steps;
  const double omega = c->omega;
  const double kkt_cur = kkt_weighted(omega, cur);
  const double kkt_avg = kkt_weighted(omega, avg);
  const bool to_average = c->halpern || kkt_avg < kkt_cur;
  const double cand = to_average ? kkt_avg : kkt_cur;
  if (!(c->kkt_at_restart < INFINITY)) c->kkt_at_restart = cand;
  const bool restart = cand <= 0.2 * c->kkt_at_restart ||
                       (cand <= 0.8 * c->kkt_at_restart && cand > c->kkt_previous) ||
                       static_cast<double>(k_new) >= c->art_frac * static_cast<double>(iter + 1);
  c->kkt_previous = cand;
  c->last_kkt = cand;
  if (restart) {
    const double dx = sqrt(c->eval_c[to_average ? 16 : 14] + c->eval_r[to_average ? 16 : 14]);
    const double dy = sqrt(c->eval_r[to_average ? 17 : 15]);
    if (dx > 1e-10 && dy > 1e-10) {
      const double w = exp(0.5 * log(dy / dx) + 0.5 * log(omega));
      c->omega = w;
      c->tau = c->eta / w;
      c->sigma = c->eta * w;
    }
    c->restart_pending = 1;
    c->restart_to_avg = to_average ? 1 : 0;
    c->k = 0;
    c->kkt_at_restart = cand;
    c->kkt_previous = INFINITY;
    c->restarts += 1;
  } else {
    c->k = k_new;
  }
  c->t = t_new;
  // Halpern: the answer is T(z) (within the bounds), not the Halpern iterate.
  const int ans = c->halpern ? 1 : 0;
  if (c->t >= c->max_iter) {
    set_answer(c, kIterationLimit, ans ? avg : cur, c->max_iter, ans);
    return;
  }
  if (c->deadline_ns != 0ull && globaltimer_ns() > c->deadline_ns) {
    set_answer(c, kTimeLimit, ans ? avg : cur, c->t, ans);
  }
}

// Restart at the candidate (pdhg_core.cu:362-380 + advance()): it becomes the current point
// (both ping-pong buffers), the extrapolated point (no momentum) and the restart point.
template <typename T>
__global__ void restart_kernel(const Ctl* __restrict__ ctl, IterView<T> it) {
  if (!ctl->restart_pending) return;
  const int cur = static_cast<int>(ctl->t & 1);
  const bool avg = ctl->restart_to_avg != 0;
  const int nt = it.n + it.m;
  const T* vc = avg ? it.Verg : it.v(cur);
  const T* yc = avg ? it.Yerg : it.y(cur);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
    const T val = vc[k];
    it.Vrst[k] = val;
    it.V[0][k] = val;
    it.V[1][k] = val;
    it.Vbar[k] = val;
    if (k < it.m) {
      const T yv = yc[k];
      it.Yrst[k] = yv;
      it.Y[0][k] = yv;
      it.Y[1][k] = yv;
    }
  }
}

__global__ void set_deadline_kernel(Ctl* c, unsigned long long budget_ns) {
  if (threadIdx.x == 0 && blockIdx.x == 0) c->deadline_ns = globaltimer_ns() + budget_ns;
}

// The answer in the LpProblem's space (pdlp.cpp:1167-1189): x = v cs, r = v / rs, y = y rs.
template <typename T>
__global__ void extract_kernel(const Ctl* __restrict__ ctl, IterView<T> it, EvalView ev,
                               double* x_out, double* y_out, double* dual_ray) {
  const int cur = static_cast<int>(ctl->t & 1);
  const bool avg = ctl->result_average != 0;
  const T* v = avg ? it.Verg : it.v(cur);
  const T* y = avg ? it.Yerg : it.y(cur);
  const int n = it.n;
  const int nt = n + it.m;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
    if (k < n) {
      x_out[k] = static_cast<double>(v[k]) * ev.cs[k];
    } else {
      x_out[k] = static_cast<double>(v[k]) / ev.rs[k - n];
    }
    if (k < it.m) {
      y_out[k] = static_cast<double>(y[k]) * ev.rs[k];
      if (dual_ray != nullptr) dual_ray[k] = static_cast<double>(it.Yerg[k]);
    }
  }
}

// ------------------------------------------------------------------------------------------
// Infeasibility and unboundedness detection (pdlp.cpp:715-1043), on the device: Farkas
// certificate from the average dual, improving ray from the difference of consecutive
// iterates. Gated by Ctl::detect_pending; scalars land in Ctl::det / det_flags.

template <typename T>
__global__ void __launch_bounds__(kBlock) det_farkas_rows_kernel(Ctl* c, IterView<T> it,
                                                                 EvalView ev, RedView red) {
  if (c->done || !c->detect_pending) return;
  __shared__ double scratch[kMaxSums * (kBlock / 32)];
  double a[2] = {0.0, 0.0};  // max |yf|, sum |yf|
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < it.m; i += gridDim.x * blockDim.x) {
    const double yf = fabs(static_cast<double>(it.Yerg[i]) * ev.rs[i]);
    a[0] = fmax(a[0], yf);
    a[1] += yf;
  }
  grid_reduce<2, 1u>(a, red.partial, red.counter, scratch, [c](const double (&t)[2]) {
    c->det[0] = t[0];
    c->det[1] = t[1];
  });
}

// A'yf by columns: aty_j = (K' yerg)_j / cs_j, stored, and sum |aty_j|.
template <typename T>
struct FarkasColEpi {
  double* aty;
  const double* cs;
  double acc[1];
  __device__ __forceinline__ void row(int j, const double (&s)[1]) {
    const double a = s[0] / cs[j];
    aty[j] = a;
    acc[0] += fabs(a);
  }
  __device__ __forceinline__ void long_row(int lrow, int j, const double (&s)[1]) {
    const double a = s[0] / cs[j];
    aty[j] = a;
    long_abs[lrow * kMaxSums] = fabs(a);
  }
  double* long_abs;
};

template <typename T>
__global__ void __launch_bounds__(kBlock) det_farkas_cols_kernel(Ctl* c, OpView<T> Kt,
                                                                 IterView<T> it, EvalView ev,
                                                                 RedView red, double* aty) {
  if (c->done || !c->detect_pending) return;
  FarkasColEpi<T> epi;
  epi.aty = aty;
  epi.cs = ev.cs;
  epi.acc[0] = 0.0;
  epi.long_abs = red.long_terms;
  struct G {
    const T* y;
    __device__ __forceinline__ double operator()(int, T a, int i) const {
      return static_cast<double>(a) * static_cast<double>(ldg(y + i));
    }
  } g{it.Yerg};
  run_tiles<T, double, 1>(Kt.ts, Kt.ptr, Kt.idx, Kt.val, g, epi);
  grid_reduce<1>(epi.acc, red.partial, red.counter, smem_red(), [c](const double (&t)[1]) {
    // w_scale: columns first, then the logicals' |yf| (pdlp.cpp:761-767).
    c->det[1] = t[0] + c->det[1];
  }, red.long_terms, Kt.ts.nlong);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) det_farkas_bounds_kernel(Ctl* c, IterView<T> it,
                                                                   EvalView ev, RedView red,
                                                                   const double* aty) {
  if (c->done || !c->detect_pending) return;
  __shared__ double scratch[kMaxSums * (kBlock / 32)];
  const double y_max = c->det[0];
  const double tol = 1e-9 * c->det[1];
  const int n = it.n;
  const int nt = n + it.m;
  // min_f finite part, max_f finite part, min_f has -inf, max_f has +inf, scale
  double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
    const double raw = k < n ? aty[k] : -(static_cast<double>(it.Yerg[k - n]) * ev.rs[k - n]);
    const double lo = ev.lower[k];
    const double up = ev.upper[k];
    const double coef = fabs(raw) <= tol ? 0.0 : raw;
    if (coef > 0) {
      if (lo > -INFINITY) a[0] += coef * lo; else a[2] = 1.0;
      if (up < INFINITY) a[1] += coef * up; else a[3] = 1.0;
    } else if (coef < 0) {
      if (up < INFINITY) a[0] += coef * up; else a[2] = 1.0;
      if (lo > -INFINITY) a[1] += coef * lo; else a[3] = 1.0;
    }
    const double w = k < n ? raw / y_max : -raw / y_max;
    if (fabs(w) > 1e-9) {
      if (lo > -INFINITY) a[4] = fmax(a[4], fabs(w * lo));
      if (up < INFINITY) a[4] = fmax(a[4], fabs(w * up));
    }
  }
  grid_reduce<5, 0x1Cu>(a, red.partial, red.counter, scratch, [c](const double (&t)[5]) {
    const double min_f = t[2] > 0.0 ? -INFINITY : t[0];
    const double max_f = t[3] > 0.0 ? INFINITY : t[1];
    double scale = t[4];
    if (!isfinite(scale)) scale = 0.0;
    const double margin = 1e-8 * (1.0 + scale);
    c->det[2] = min_f;
    c->det[3] = max_f;
    c->det[4] = scale;
    const bool found = c->det[0] > 1e-6 && ((isfinite(min_f) && min_f > margin) ||
                                            (isfinite(max_f) && max_f < -margin));
    c->det_flags[0] = found ? 1 : 0;
  });
}

// Ray candidate d = v_new - v: v_max = max |d|.
template <typename T>
__global__ void __launch_bounds__(kBlock) det_ray_max_kernel(Ctl* c, IterView<T> it, RedView red) {
  if (c->done || !c->detect_pending || c->det_flags[0]) return;
  __shared__ double scratch[kMaxSums * (kBlock / 32)];
  const int cur = static_cast<int>(((c->t + (c->max_iter - c->t < kCheckFrequency
                                                  ? c->max_iter - c->t
                                                  : kCheckFrequency))) & 1);
  const T* vn = it.v(cur);
  const T* vo = it.v(cur ^ 1);
  const int nt = it.n + it.m;
  double a[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
    a[0] = fmax(a[0], fabs(static_cast<double>(vn[k]) - static_cast<double>(vo[k])));
  }
  grid_reduce<1, 1u>(a, red.partial, red.counter, scratch,
                     [c](const double (&t)[1]) { c->det[5] = t[0]; });
}

// Columns of the ray: cost_dir (structural part), bound checks and the polished ray x
// (pdlp.cpp:887-964). ray_x (n) in the LpProblem's space.
template <typename T>
__global__ void __launch_bounds__(kBlock) det_ray_cols_kernel(Ctl* c, IterView<T> it, EvalView ev,
                                                              RedView red, double* ray_x) {
  if (c->done || !c->detect_pending || c->det_flags[0]) return;
  __shared__ double scratch[kMaxSums * (kBlock / 32)];
  const int cur = static_cast<int>(((c->t + (c->max_iter - c->t < kCheckFrequency
                                                  ? c->max_iter - c->t
                                                  : kCheckFrequency))) & 1);
  const T* vn = it.v(cur);
  const T* vo = it.v(cur ^ 1);
  const double v_max = c->det[5];
  double a[2] = {0.0, 0.0};  // cost_dir (cols), bound failure
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < it.n; j += gridDim.x * blockDim.x) {
    const double d = (static_cast<double>(vn[j]) - static_cast<double>(vo[j])) / v_max;
    double xj = d * ev.cs[j];
    a[0] += ev.cost[j] * xj;
    const double lo = ev.lower[j];
    const double up = ev.upper[j];
    const bool lb = lo > -INFINITY / 2;
    const bool ub = up < INFINITY / 2;
    const bool fixed = lb && ub && (up - lo <= 1e-10 * (1.0 + fabs(lo)));
    if (lb && ub) {
      if (fabs(xj) > (fixed ? 1e-3 : 1e-4)) a[1] = 1.0;
      xj = 0.0;
    } else if (lb) {
      if (xj < -1e-4) a[1] = 1.0;
      xj = fmax(xj, 0.0);
    } else if (ub) {
      if (xj > 1e-4) a[1] = 1.0;
      xj = fmin(xj, 0.0);
    }
    ray_x[j] = xj;
  }
  grid_reduce<2, 2u>(a, red.partial, red.counter, scratch, [c](const double (&t)[2]) {
    c->det[7] = t[0];
    c->det_flags[4] = t[1] > 0.0 ? 0 : 1;
  });
}

// Rows of the ray: primal feasibility of the raw direction and cost_dir of the logicals
// (NV 0: K d_x), and the row bounds of the polished ray (NV 1: K (ray_x / cs)).
template <typename T>
struct RayRowEpi {
  const T* vn;
  const T* vo;
  double inv_vmax;
  EvalView ev;
  int n;
  double acc[3];  // primal_feas^2, cost_dir (rows), row failure
  double* long_terms;
  __device__ __forceinline__ void terms(int i, const double (&s)[2], double (&a)[3]) {
    const double rs = ev.rs[i];
    const double dr = (static_cast<double>(vn[n + i]) - static_cast<double>(vo[n + i])) * inv_vmax;
    const double res = s[0] / rs - dr / rs;
    a[0] += res * res;
    a[1] += ev.cost[n + i] * (dr / rs);
    const double av = s[1] / rs;
    const double lo = ev.lower[n + i];
    const double up = ev.upper[n + i];
    const bool lb = lo > -INFINITY / 2;
    const bool ub = up < INFINITY / 2;
    const bool fixed = lb && ub && (up - lo <= 1e-10 * (1.0 + fabs(lo)));
    if (lb && ub) {
      if (fabs(av) > (fixed ? 1e-3 : 1e-4)) a[2] = 1.0;
    } else if (lb) {
      if (av < -1e-4) a[2] = 1.0;
    } else if (ub) {
      if (av > 1e-4) a[2] = 1.0;
    }
  }
  __device__ __forceinline__ void row(int i, const double (&s)[2]) { terms(i, s, acc); }
  __device__ __forceinline__ void long_row(int lrow, int i, const double (&s)[2]) {
    double a[3] = {0.0, 0.0, 0.0};
    terms(i, s, a);
    for (int q = 0; q < 3; ++q) long_terms[lrow * kMaxSums + q] = a[q];
  }
};

template <typename T>
__global__ void __launch_bounds__(kBlock) det_ray_rows_kernel(Ctl* c, OpView<T> K, IterView<T> it,
                                                              EvalView ev, RedView red,
                                                              const double* ray_x) {
  if (c->done || !c->detect_pending || c->det_flags[0]) return;
  const int cur = static_cast<int>(((c->t + (c->max_iter - c->t < kCheckFrequency
                                                  ? c->max_iter - c->t
                                                  : kCheckFrequency))) & 1);
  RayRowEpi<T> epi;
  epi.vn = it.v(cur);
  epi.vo = it.v(cur ^ 1);
  epi.inv_vmax = 1.0;
  const double v_max = c->det[5];
  epi.ev = ev;
  epi.n = it.n;
  epi.acc[0] = epi.acc[1] = epi.acc[2] = 0.0;
  epi.long_terms = red.long_terms;
  struct G {
    const T* vn;
    const T* vo;
    const double* ray_x;
    const double* cs;
    double v_max;
    __device__ __forceinline__ double operator()(int v, T a, int j) const {
      if (v == 0) {
        const double d = (static_cast<double>(vn[j]) - static_cast<double>(vo[j])) / v_max;
        return static_cast<double>(a) * d;
      }
      return static_cast<double>(a) * (ray_x[j] / cs[j]);
    }
  } g{epi.vn, epi.vo, ray_x, ev.cs, v_max};
  epi.inv_vmax = 1.0 / v_max;
  run_tiles<T, double, 2>(K.ts, K.ptr, K.idx, K.val, g, epi);
  grid_reduce<3, 4u>(epi.acc, red.partial, red.counter, smem_red(),
                     [c](const double (&t)[3]) {
    const double cd = t[1];
    const double fail = t[2];
    const double primal_feas = sqrt(t[0]);
    const double cost_dir = c->det[7] + cd;
    c->det[6] = primal_feas;
    c->det[7] = cost_dir;
    const bool ok = c->det_flags[4] != 0 && !(fail > 0.0);
    c->det_flags[1] = (c->det[5] > 1e-6 && primal_feas < 1e-6 && cost_dir < -1e-8 && ok) ? 1 : 0;
  }, red.long_terms, K.ts.nlong);
}

// ------------------------------------------------------------------------------------------
// Setup on the device (pdlp.cpp:36-187, 289-299, 377-394, 490-492), FP64.

struct MaxNormEpi {
  double acc[1];
  __device__ __forceinline__ void row(int, const double (&s)[1]) { acc[0] = fmax(acc[0], sqrt(s[0])); }
  __device__ __forceinline__ void long_row(int, int, const double (&s)[1]) {
    acc[0] = fmax(acc[0], sqrt(s[0]));
  }
};

struct SqProd {
  __device__ __forceinline__ double operator()(int, double a, int) const { return a * a; }
};

__global__ void __launch_bounds__(kBlock) max_norm_kernel(OpView<double> A, RedView red,
                                                          double* out) {
  MaxNormEpi epi;
  epi.acc[0] = 0.0;
  run_tiles<double, double, 1>(A.ts, A.ptr, A.idx, A.val, SqProd{}, epi);
  grid_reduce<1, 1u>(epi.acc, red.partial, red.counter, smem_red(),
                     [out](const double (&t)[1]) { *out = t[0]; });
}

__global__ void __launch_bounds__(kBlock) sum_sq_kernel(const double* x, int len, RedView red,
                                                        double* out_sqrt) {
  __shared__ double scratch[kMaxSums * (kBlock / 32)];
  double a[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < len; k += gridDim.x * blockDim.x) {
    a[0] += x[k] * x[k];
  }
  grid_reduce<1>(a, red.partial, red.counter, scratch,
                 [out_sqrt](const double (&t)[1]) { *out_sqrt = sqrt(t[0]); });
}

// Ruiz norms of D_r A D_c: product (a * scale[col])^2, row norm = rowscale * sqrt(sum).
struct RuizProd {
  const double* other;
  __device__ __forceinline__ double operator()(int, double a, int j) const {
    const double v = a * other[j];
    return v * v;
  }
};

struct RuizEpi {
  const double* own;
  double* norm;
  __device__ __forceinline__ void row(int r, const double (&s)[1]) { norm[r] = sqrt(s[0]) * own[r]; }
  __device__ __forceinline__ void long_row(int, int r, const double (&s)[1]) { row(r, s); }
};

__global__ void __launch_bounds__(kBlock) ruiz_norm_kernel(const Ctl* c, OpView<double> A,
                                                           const double* own, const double* other,
                                                           double* norm) {
  if (c->ruiz_done) return;
  RuizEpi epi{own, norm};
  run_tiles<double, double, 1>(A.ts, A.ptr, A.idx, A.val, RuizProd{other}, epi);
}

// Scale update of one Ruiz pass (pdlp.cpp:154-178) over columns then rows.
__global__ void __launch_bounds__(kBlock) ruiz_update_kernel(Ctl* c, int n, int m, double* cs,
                                                             const double* cn, double* rs,
                                                             const double* rn, RedView red) {
  if (c->ruiz_done) return;
  __shared__ double scratch[kMaxSums * (kBlock / 32)];
  double a[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n + m; k += gridDim.x * blockDim.x) {
    double* sc = k < n ? cs + k : rs + (k - n);
    const double nv = k < n ? cn[k] : rn[k - n];
    if (nv > 0) {
      const double old = *sc;
      double s = old / nv;
      s = fmax(1e-8, fmin(1e8, s));
      if (fabs(s - old) / fmax(fabs(old), 1.0) > 0.1) a[0] = 1.0;
      *sc = s;
    }
  }
  grid_reduce<1, 1u>(a, red.partial, red.counter, scratch,
                     [c](const double (&t)[1]) { c->ruiz_done = t[0] > 0.0 ? 0 : 1; });
}

// A_eq = D_r A D_c on both operators: K entries (a rs_i) cs_j, K' entries (a cs_j) rs_i, the
// association of apply_equilibration for A and A' (pdlp.cpp:204, 265-266). Rows by binary
// search in the row starts.
__device__ __forceinline__ int row_of(const int* ptr, int rows, int k) {
  int lo = 0, hi = rows;  // ptr[lo] <= k < ptr[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (ptr[mid] <= k) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void apply_scaling_kernel(OpView<double> K, OpView<double> Kt, const double* rs,
                                     const double* cs, long long nnz) {
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nnz;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int kk = static_cast<int>(k);
    const int i = row_of(K.ptr, K.rows, kk);
    const int j = K.idx[kk];
    K.val[kk] = K.val[kk] * rs[i] * cs[j];
    const int jj = row_of(Kt.ptr, Kt.rows, kk);
    const int ii = Kt.idx[kk];
    Kt.val[kk] = Kt.val[kk] * cs[jj] * rs[ii];
  }
}

__global__ void scale_vectors_kernel(int n, int m, const double* cs, const double* rs,
                                     const double* cost, const double* lower, const double* upper,
                                     const double* rhs, double* cost_eq, double* lower_eq,
                                     double* upper_eq, double* rhs_eq) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n + m; k += gridDim.x * blockDim.x) {
    if (k < n) {
      cost_eq[k] = cost[k] * cs[k];
      lower_eq[k] = lower[k] / cs[k];
      upper_eq[k] = upper[k] / cs[k];
    } else {
      const double r = rs[k - n];
      cost_eq[k] = cost[k] * r;
      lower_eq[k] = lower[k] * r;
      upper_eq[k] = upper[k] * r;
      if (rhs != nullptr) rhs_eq[k - n] = rhs[k - n] * r;
    }
  }
}

// Power iteration (pdlp.cpp:36-103) on A_eq: v = A' u, u = A v, sigma = |u| / |v|.
struct StoreSqEpi {
  double* out;
  double acc[1];
  double* long_terms;
  __device__ __forceinline__ void row(int r, const double (&s)[1]) {
    out[r] = s[0];
    acc[0] += s[0] * s[0];
  }
  __device__ __forceinline__ void long_row(int lrow, int r, const double (&s)[1]) {
    out[r] = s[0];
    long_terms[lrow * kMaxSums] = s[0] * s[0];
  }
};

__global__ void __launch_bounds__(kBlock) power_spmv_kernel(Ctl* c, OpView<double> A,
                                                            const double* x, double* y,
                                                            RedView red, int which) {
  if (c->power_done) return;
  StoreSqEpi epi;
  epi.out = y;
  epi.acc[0] = 0.0;
  epi.long_terms = red.long_terms;
  run_tiles<double, double, 1>(A.ts, A.ptr, A.idx, A.val, Gather1<double, double>{x}, epi);
  grid_reduce<1>(epi.acc, red.partial, red.counter, smem_red(),
                 [c, which](const double (&t)[1]) {
    const double nrm = sqrt(t[0]);
    if (which == 0) {
      c->power_vnorm = nrm;
      if (nrm == 0.0) c->power_done = 1;
    } else {
      c->power_unorm = nrm;
      if (nrm == 0.0) {
        c->power_done = 1;
      } else {
        c->power_sigma = nrm / c->power_vnorm;
      }
    }
  }, red.long_terms, A.ts.nlong);
}

__global__ void scale_by_norm_kernel(const Ctl* c, double* u, int m, int first) {
  if (!first && c->power_done) return;
  const double nrm = c->power_unorm;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    u[i] = u[i] / nrm;
  }
}

__global__ void power_finish_kernel(Ctl* c) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double L = 1.0;
  if (c->m > 0 && !c->power_done) {
    const double la = c->power_sigma * 1.01;
    L = sqrt(la * la + 1.0);
  } else if (c->m > 0 && c->power_done && c->power_sigma > 0.0) {
    // A zero vector after some iterations: the reference returns 1 (pdlp.cpp:74, 92).
    L = 1.0;
  }
  c->op_norm = L;
  c->eta = 0.99 / L;
  c->omega = 1.0;
  c->tau = c->eta;
  c->sigma = c->eta;
}

__global__ void init_state_kernel(Ctl* c) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  c->t = 0;
  c->k = 0;
  c->kkt_at_restart = INFINITY;
  c->kkt_previous = INFINITY;
  c->status = kRunning;
  c->done = 0;
  c->result_average = 0;
  c->restart_pending = 0;
  c->detect_pending = 0;
  c->iterations = 0;
  c->restarts = 0;
  c->evaluations = 0;
  c->res[0] = c->res[1] = c->res[2] = 0.0;
}

template <typename Src, typename Dst>
__global__ void convert_kernel(const Src* src, Dst* dst, long long count) {
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < count;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    dst[k] = static_cast<Dst>(src[k]);
  }
}

struct StoreEpi {
  double* out;
  __device__ __forceinline__ void row(int r, const double (&s)[1]) { out[r] = s[0]; }
  __device__ __forceinline__ void long_row(int, int r, const double (&s)[1]) { out[r] = s[0]; }
};

__global__ void __launch_bounds__(kBlock) spmv_kernel(OpView<double> A, const double* x,
                                                      double* y) {
  StoreEpi epi{y};
  run_tiles<double, double, 1>(A.ts, A.ptr, A.idx, A.val, Gather1<double, double>{x}, epi);
}

// ------------------------------------------------------------------------------------------
// Enhanced preconditioning (the engine's own, not the reference's): Ruiz equilibration in the
// infinity norm (10 passes: every row and column divided by the square root of its largest
// scaled magnitude) followed by Pock-Chambolle scaling with alpha = 1 (divide by the square
// root of the scaled absolute row / column sums), both updating rows and columns from the same
// matrix. Statistics by the tile kernel: products |a| * scale[other], max (Ruiz) or sum (PC).

struct AbsProd {
  const double* other;
  __device__ __forceinline__ double operator()(int, double a, int j) const {
    return fabs(a) * other[j];
  }
};

struct StatEpi {
  const double* own;
  double* stat;
  __device__ __forceinline__ void row(int r, const double (&s)[1]) { stat[r] = s[0] * own[r]; }
  __device__ __forceinline__ void long_row(int, int r, const double (&s)[1]) { row(r, s); }
};

template <bool MAXRED>
__global__ void __launch_bounds__(kBlock) abs_stat_kernel(OpView<double> A, const double* own,
                                                          const double* other, double* stat) {
  StatEpi epi{own, stat};
  run_tiles<double, double, 1, AbsProd, StatEpi, MAXRED>(A.ts, A.ptr, A.idx, A.val,
                                                         AbsProd{other}, epi);
}

// scale /= sqrt(stat) where stat > 0, columns then rows.
__global__ void sqrt_rescale_kernel(int n, int m, double* cs, const double* cn, double* rs,
                                    const double* rn) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n + m; k += gridDim.x * blockDim.x) {
    if (k < n) {
      if (cn[k] > 0.0) cs[k] = cs[k] / sqrt(cn[k]);
    } else {
      if (rn[k - n] > 0.0) rs[k - n] = rs[k - n] / sqrt(rn[k - n]);
    }
  }
}

// Initial primal weight |c| / |b| of the equilibrated problem (b: each row's largest finite
// bound magnitude), 1 when either is ~0.
__global__ void __launch_bounds__(kBlock) primal_weight_init_kernel(Ctl* c, int n, int m,
                                                                    const double* cost_eq,
                                                                    const double* lower_eq,
                                                                    const double* upper_eq,
                                                                    RedView red) {
  __shared__ double scratch[kMaxSums * (kBlock / 32)];
  double a[2] = {0.0, 0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n + m; k += gridDim.x * blockDim.x) {
    if (k < n) {
      a[0] += cost_eq[k] * cost_eq[k];
    } else {
      const double lo = lower_eq[k];
      const double up = upper_eq[k];
      const double b = fmax(isfinite(lo) ? fabs(lo) : 0.0, isfinite(up) ? fabs(up) : 0.0);
      a[1] += b * b;
    }
  }
  grid_reduce<2>(a, red.partial, red.counter, scratch, [c](const double (&t)[2]) {
    const double cn = sqrt(t[0]);
    const double bn = sqrt(t[1]);
    const double w = (cn > 1e-10 && bn > 1e-10) ? cn / bn : 1.0;
    c->omega = w;
    c->tau = c->eta / w;
    c->sigma = c->eta * w;
  });
}

int vec_grid(long long len) {
  long long g = (len + kBlock - 1) / kBlock;
  if (g < 1) g = 1;
  if (g > 4096) g = 4096;
  return static_cast<int>(g);
}

}  // namespace

size_t tile_smem_bytes(const TileSet& ts, int nv, size_t acc_bytes) {
  return tile_smem_size(nv, acc_bytes, ts.cap_nnz, ts.cap_rows);
}

namespace {

// The dual step launches: the kind-3 staging or the staged segments' chunk buffers when the
// tile set has them (both in the variant-2 kernels).
template <typename T>
bool dual_variant2(const TileSet& ts) {
  return ts.groups > 0 || ts.staged;
}
template <typename T>
size_t dual_smem_bytes(const TileSet& ts) {
  if (!dual_variant2<T>(ts)) return tile_smem_bytes(ts, 1, sizeof(T));
  const size_t g = group_smem_size<T, Acc<T>>();
  const size_t c = staged_smem_size<T>();
  return g > c ? g : c;
}

}  // namespace

void configure_kernels() {
  // Opt in to large dynamic shared memory; the launch sizes themselves follow each operator's
  // tile capacity, so occupancy is set by the actual size.
  const int big = 200 * 1024;
  cudaFuncSetAttribute(eval_rows_kernel<double, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(eval_rows_kernel<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(eval_cols_kernel<double, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(eval_cols_kernel<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(eval_rows_kernel<float, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(eval_rows_kernel<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(eval_cols_kernel<float, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(eval_cols_kernel<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(det_ray_rows_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(det_ray_rows_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(dual_step_kernel<double, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(primal_step_kernel<double, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(dual_step_kernel<float, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(primal_step_kernel<float, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(dual_step_kernel<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(dual_step_kernel<double, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(primal_step_kernel<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(dual_step_kernel<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(dual_step_kernel<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(primal_step_kernel<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_dual_kernel<double, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_primal_kernel<double, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_dual_kernel<float, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_primal_kernel<float, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_dual_kernel<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_dual_kernel<double, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_primal_kernel<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_dual_kernel<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_dual_kernel<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(halpern_primal_kernel<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(det_farkas_cols_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(det_farkas_cols_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(max_norm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(ruiz_norm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(power_spmv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(spmv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(abs_stat_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(abs_stat_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
}

template <typename T>
void launch_dual_step(const Ctl* ctl, const OpView<T>& K, const IterView<T>& it, int j, int grid,
                      cudaStream_t s) {
  if (K.ts.ntiles == 0) return;
  const size_t sm = dual_smem_bytes<T>(K.ts);
  if (dual_variant2<T>(K.ts)) {
    dual_step_kernel<T, 2><<<grid, kBlock, sm, s>>>(ctl, K, it, j);
  } else if (K.ts.variant == 1) {
    dual_step_kernel<T, 1><<<grid, kBlock, sm, s>>>(ctl, K, it, j);
  } else {
    dual_step_kernel<T, 0><<<grid, kBlock, sm, s>>>(ctl, K, it, j);
  }
}

template <typename T>
void launch_primal_step(const Ctl* ctl, const OpView<T>& Kt, const IterView<T>& it, int j,
                        int grid, cudaStream_t s) {
  if (Kt.ts.ntiles == 0) return;
  const size_t sm = tile_smem_bytes(Kt.ts, 1, sizeof(T));
  if (Kt.ts.variant == 1) {
    primal_step_kernel<T, 1><<<grid, kBlock, sm, s>>>(ctl, Kt, it, j);
  } else {
    primal_step_kernel<T, 0><<<grid, kBlock, sm, s>>>(ctl, Kt, it, j);
  }
}

template <typename T>
void launch_halpern_primal(const Ctl* ctl, const OpView<T>& Kt, const IterView<T>& it, int j,
                           int grid, cudaStream_t s) {
  if (Kt.ts.ntiles == 0) return;
  const size_t sm = tile_smem_bytes(Kt.ts, 1, sizeof(T));
  if (Kt.ts.variant == 1) {
    halpern_primal_kernel<T, 1><<<grid, kBlock, sm, s>>>(ctl, Kt, it, j);
  } else {
    halpern_primal_kernel<T, 0><<<grid, kBlock, sm, s>>>(ctl, Kt, it, j);
  }
}

template <typename T>
void launch_halpern_dual(const Ctl* ctl, const OpView<T>& K, const IterView<T>& it, int j,
                         int grid, cudaStream_t s) {
  if (K.ts.ntiles == 0) return;
  const size_t sm = dual_smem_bytes<T>(K.ts);
  if (dual_variant2<T>(K.ts)) {
    halpern_dual_kernel<T, 2><<<grid, kBlock, sm, s>>>(ctl, K, it, j);
  } else if (K.ts.variant == 1) {
    halpern_dual_kernel<T, 1><<<grid, kBlock, sm, s>>>(ctl, K, it, j);
  } else {
    halpern_dual_kernel<T, 0><<<grid, kBlock, sm, s>>>(ctl, K, it, j);
  }
}

template <typename T>
void launch_eval(Ctl* ctl, const OpView<T>& K, const OpView<T>& Kt, const IterView<T>& it,
                 const EvalView& ev, const RedView& red, int grid_k, int grid_t,
                 int fixed_parity, cudaStream_t s, bool second_only) {
  const size_t smk = tile_smem_bytes(K.ts, 2, 8);
  const size_t smt = tile_smem_bytes(Kt.ts, 2, 8);
  if constexpr (std::is_same<T, float>::value) {
    // FP32 operators carry their own (equilibrated) data: `ev` is not used.
    (void)ev;
    if (second_only) {
      eval_rows32_kernel<1><<<grid_k, kBlock, smk, s>>>(ctl, K, it, red, fixed_parity);
      eval_cols32_kernel<1><<<grid_t, kBlock, smt, s>>>(ctl, Kt, it, red, fixed_parity);
    } else {
      eval_rows32_kernel<0><<<grid_k, kBlock, smk, s>>>(ctl, K, it, red, fixed_parity);
      eval_cols32_kernel<0><<<grid_t, kBlock, smt, s>>>(ctl, Kt, it, red, fixed_parity);
    }
  } else {
    if (second_only) {
      eval_rows_kernel<T, 1><<<grid_k, kBlock, smk, s>>>(ctl, K, it, ev, red, fixed_parity);
      eval_cols_kernel<T, 1><<<grid_t, kBlock, smt, s>>>(ctl, Kt, it, ev, red, fixed_parity);
    } else {
      eval_rows_kernel<T, 0><<<grid_k, kBlock, smk, s>>>(ctl, K, it, ev, red, fixed_parity);
      eval_cols_kernel<T, 0><<<grid_t, kBlock, smt, s>>>(ctl, Kt, it, ev, red, fixed_parity);
    }
  }
}

void launch_decide_a(Ctl* ctl, cudaStream_t s) { decide_a_kernel<<<1, 32, 0, s>>>(ctl); }
void launch_decide_b(Ctl* ctl, cudaStream_t s) { decide_b_kernel<<<1, 32, 0, s>>>(ctl); }

template <typename T>
void launch_restart(const Ctl* ctl, const IterView<T>& it, cudaStream_t s) {
  restart_kernel<T><<<vec_grid(it.n + it.m), kBlock, 0, s>>>(ctl, it);
}

template <typename T>
void launch_detect(Ctl* ctl, const OpView<T>& K, const OpView<T>& Kt, const IterView<T>& it,
                   const EvalView& ev, const RedView& red, double* scratch_n, double* scratch_nt,
                   int grid_k, int grid_t, cudaStream_t s) {
  (void)scratch_nt;
  const int gm = vec_grid(it.m) < 1024 ? vec_grid(it.m) : 1024;
  const int gn = vec_grid(it.n) < 1024 ? vec_grid(it.n) : 1024;
  const int gnt = vec_grid(it.n + it.m) < 1024 ? vec_grid(it.n + it.m) : 1024;
  det_farkas_rows_kernel<T><<<gm, kBlock, 0, s>>>(ctl, it, ev, red);
  det_farkas_cols_kernel<T><<<grid_t, kBlock, tile_smem_bytes(Kt.ts, 1, 8), s>>>(ctl, Kt, it, ev,
                                                                                red, scratch_n);
  det_farkas_bounds_kernel<T><<<gnt, kBlock, 0, s>>>(ctl, it, ev, red, scratch_n);
  det_ray_max_kernel<T><<<gnt, kBlock, 0, s>>>(ctl, it, red);
  det_ray_cols_kernel<T><<<gn, kBlock, 0, s>>>(ctl, it, ev, red, scratch_n);
  det_ray_rows_kernel<T><<<grid_k, kBlock, tile_smem_bytes(K.ts, 2, 8), s>>>(ctl, K, it, ev, red,
                                                                             scratch_n);
}

template <typename T>
void launch_extract(const Ctl* ctl, const IterView<T>& it, const EvalView& ev, double* x_out,
                    double* y_out, double* dual_ray, double* primal_ray_src, cudaStream_t s) {
  (void)primal_ray_src;
  extract_kernel<T><<<vec_grid(it.n + it.m), kBlock, 0, s>>>(ctl, it, ev, x_out, y_out, dual_ray);
}

void launch_setup_norms(Ctl* ctl, const OpView<double>& K, const OpView<double>& Kt,
                        const double* cost, const RedView& red, int grid_k, int grid_t,
                        cudaStream_t s) {
  if (K.rows > 0) {
    if (Kt.ts.ntiles > 0) {
      max_norm_kernel<<<grid_t, kBlock, tile_smem_bytes(Kt.ts, 1, 8), s>>>(Kt, red,
                                                                         &ctl->a_norm_max_col);
    }
    if (K.ts.ntiles > 0) {
      max_norm_kernel<<<grid_k, kBlock, tile_smem_bytes(K.ts, 1, 8), s>>>(K, red,
                                                                        &ctl->at_norm_max_row);
    }
  }
  const int nt = K.rows + Kt.rows;
  sum_sq_kernel<<<vec_grid(nt) < 1024 ? vec_grid(nt) : 1024, kBlock, 0, s>>>(cost, nt, red,
                                                                          &ctl->c_norm);
}

__global__ void reciprocal_kernel(const double* a, double* out, int count) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    out[k] = 1.0 / a[k];
  }
}

// Gather neighbours: rows i and i + 1, each of more than 32 nonzeros, whose k-th nonzeros lie
// 1 to 4 columns apart at 7 of 8 sampled positions k (the rows of a 2-D variable array x[k][j]
// summed over k: the candidates of the kind-3 row groups).
__global__ void row_neighbours_kernel(int m, const int* __restrict__ ptr,
                                      const int* __restrict__ idx, unsigned char* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    unsigned char a = 0;
    if (i + 1 < m) {
      const int b0 = ptr[i];
      const int b1 = ptr[i + 1];
      const int len = min(b1 - b0, ptr[i + 2] - b1);
      if (len > 32) {
        int hits = 0;
        for (int q = 0; q < 8; ++q) {
          const int k = static_cast<int>(static_cast<long long>(q) * len / 8);
          const int d = idx[b1 + k] - idx[b0 + k];
          hits += d != 0 && d >= -4 && d <= 4;
        }
        a = hits >= 7;
      }
    }
    out[i] = a;
  }
}

void launch_row_neighbours(int m, const int* ptr, const int* idx, unsigned char* out,
                           cudaStream_t s) {
  if (m <= 0) return;
  row_neighbours_kernel<<<vec_grid(m) < 1024 ? vec_grid(m) : 1024, kBlock, 0, s>>>(m, ptr, idx,
                                                                                  out);
}

void launch_reciprocals(const double* a, double* out, int count, cudaStream_t s) {
  if (count <= 0) return;
  reciprocal_kernel<<<vec_grid(count) < 1024 ? vec_grid(count) : 1024, kBlock, 0, s>>>(a, out,
                                                                                     count);
}

void launch_ruiz_pass(Ctl* ctl, const OpView<double>& K, const OpView<double>& Kt, double* rs,
                      double* cs, double* rn, double* cn, const RedView& red, int grid_k,
                      int grid_t, cudaStream_t s) {
  // Column norms (rows of K'), then row norms (rows of K), both with the old scales.
  ruiz_norm_kernel<<<grid_t, kBlock, tile_smem_bytes(Kt.ts, 1, 8), s>>>(ctl, Kt, cs, rs, cn);
  ruiz_norm_kernel<<<grid_k, kBlock, tile_smem_bytes(K.ts, 1, 8), s>>>(ctl, K, rs, cs, rn);
  const int nt = K.rows + Kt.rows;
  ruiz_update_kernel<<<vec_grid(nt) < 1024 ? vec_grid(nt) : 1024, kBlock, 0, s>>>(
      ctl, Kt.rows, K.rows, cs, cn, rs, rn, red);
}

void launch_enhanced_scaling(const OpView<double>& K, const OpView<double>& Kt, double* rs,
                             double* cs, double* rn, double* cn, int grid_k, int grid_t,
                             cudaStream_t s) {
  const int n = Kt.rows;
  const int m = K.rows;
  const int g = vec_grid(n + m);
  for (int pass = 0; pass < 10; ++pass) {
    if (Kt.ts.ntiles > 0) {
      abs_stat_kernel<true><<<grid_t, kBlock, tile_smem_bytes(Kt.ts, 1, 8), s>>>(Kt, cs, rs, cn);
    }
    if (K.ts.ntiles > 0) {
      abs_stat_kernel<true><<<grid_k, kBlock, tile_smem_bytes(K.ts, 1, 8), s>>>(K, rs, cs, rn);
    }
    sqrt_rescale_kernel<<<g, kBlock, 0, s>>>(n, m, cs, cn, rs, rn);
  }
  if (Kt.ts.ntiles > 0) {
    abs_stat_kernel<false><<<grid_t, kBlock, tile_smem_bytes(Kt.ts, 1, 8), s>>>(Kt, cs, rs, cn);
  }
  if (K.ts.ntiles > 0) {
    abs_stat_kernel<false><<<grid_k, kBlock, tile_smem_bytes(K.ts, 1, 8), s>>>(K, rs, cs, rn);
  }
  sqrt_rescale_kernel<<<g, kBlock, 0, s>>>(n, m, cs, cn, rs, rn);
}

void launch_primal_weight_init(Ctl* ctl, int n, int m, const double* cost_eq,
                               const double* lower_eq, const double* upper_eq,
                               const RedView& red, cudaStream_t s) {
  const int g = vec_grid(n + m) < 1024 ? vec_grid(n + m) : 1024;
  primal_weight_init_kernel<<<g, kBlock, 0, s>>>(ctl, n, m, cost_eq, lower_eq, upper_eq, red);
}

void launch_apply_scaling(const OpView<double>& K, const OpView<double>& Kt, const double* rs,
                          const double* cs, long long nnz, cudaStream_t s) {
  if (nnz == 0) return;
  apply_scaling_kernel<<<vec_grid(nnz), kBlock, 0, s>>>(K, Kt, rs, cs, nnz);
}

void launch_scale_vectors(int n, int m, const double* cs, const double* rs, const double* cost,
                          const double* lower, const double* upper, const double* rhs,
                          double* cost_eq, double* lower_eq, double* upper_eq, double* rhs_eq,
                          cudaStream_t s) {
  scale_vectors_kernel<<<vec_grid(n + m), kBlock, 0, s>>>(n, m, cs, rs, cost, lower, upper, rhs,
                                                          cost_eq, lower_eq, upper_eq, rhs_eq);
}

void launch_power_iteration(Ctl* ctl, const OpView<double>& K, const OpView<double>& Kt,
                            double* u, double* v, const RedView& red, int iters, int grid_k,
                            int grid_t, cudaStream_t s) {
  const int m = K.rows;
  if (m > 0) {
    const int gm = vec_grid(m) < 1024 ? vec_grid(m) : 1024;
    sum_sq_kernel<<<gm, kBlock, 0, s>>>(u, m, red, &ctl->power_unorm);
    scale_by_norm_kernel<<<gm, kBlock, 0, s>>>(ctl, u, m, 1);
    for (int it = 0; it < iters; ++it) {
      if (Kt.ts.ntiles > 0) {
        power_spmv_kernel<<<grid_t, kBlock, tile_smem_bytes(Kt.ts, 1, 8), s>>>(ctl, Kt, u, v, red, 0);
      }
      if (K.ts.ntiles > 0) {
        power_spmv_kernel<<<grid_k, kBlock, tile_smem_bytes(K.ts, 1, 8), s>>>(ctl, K, v, u, red, 1);
      }
      scale_by_norm_kernel<<<gm, kBlock, 0, s>>>(ctl, u, m, 0);
    }
  }
  power_finish_kernel<<<1, 32, 0, s>>>(ctl);
}

void launch_init_state(Ctl* ctl, cudaStream_t s) { init_state_kernel<<<1, 32, 0, s>>>(ctl); }

void launch_set_deadline(Ctl* ctl, double seconds, cudaStream_t s) {
  const double ns = seconds * 1e9;
  const unsigned long long budget = ns > 1.8e19 ? 18000000000000000000ull
                                                : static_cast<unsigned long long>(ns);
  set_deadline_kernel<<<1, 32, 0, s>>>(ctl, budget);
}

template <typename Src, typename Dst>
void launch_convert(const Src* src, Dst* dst, long long count, cudaStream_t s) {
  if (count <= 0) return;
  convert_kernel<Src, Dst><<<vec_grid(count), kBlock, 0, s>>>(src, dst, count);
}

void launch_spmv(const OpView<double>& A, const double* x, double* y, int grid, cudaStream_t s) {
  if (A.ts.ntiles == 0) return;
  spmv_kernel<<<grid, kBlock, tile_smem_bytes(A.ts, 1, 8), s>>>(A, x, y);
}

// Explicit instantiations.
template void launch_dual_step<double>(const Ctl*, const OpView<double>&, const IterView<double>&,
                                       int, int, cudaStream_t);
template void launch_dual_step<float>(const Ctl*, const OpView<float>&, const IterView<float>&, int,
                                      int, cudaStream_t);
template void launch_primal_step<double>(const Ctl*, const OpView<double>&,
                                         const IterView<double>&, int, int, cudaStream_t);
template void launch_primal_step<float>(const Ctl*, const OpView<float>&, const IterView<float>&,
                                        int, int, cudaStream_t);
template void launch_halpern_primal<double>(const Ctl*, const OpView<double>&,
                                            const IterView<double>&, int, int, cudaStream_t);
template void launch_halpern_primal<float>(const Ctl*, const OpView<float>&,
                                           const IterView<float>&, int, int, cudaStream_t);
template void launch_halpern_dual<double>(const Ctl*, const OpView<double>&,
                                          const IterView<double>&, int, int, cudaStream_t);
template void launch_halpern_dual<float>(const Ctl*, const OpView<float>&,
                                         const IterView<float>&, int, int, cudaStream_t);
template void launch_eval<double>(Ctl*, const OpView<double>&, const OpView<double>&,
                                  const IterView<double>&, const EvalView&, const RedView&, int,
                                  int, int, cudaStream_t, bool);
template void launch_eval<float>(Ctl*, const OpView<float>&, const OpView<float>&,
                                 const IterView<float>&, const EvalView&, const RedView&, int, int,
                                 int, cudaStream_t, bool);
template void launch_restart<double>(const Ctl*, const IterView<double>&, cudaStream_t);
template void launch_restart<float>(const Ctl*, const IterView<float>&, cudaStream_t);
template void launch_detect<double>(Ctl*, const OpView<double>&, const OpView<double>&,
                                    const IterView<double>&, const EvalView&, const RedView&,
                                    double*, double*, int, int, cudaStream_t);
template void launch_detect<float>(Ctl*, const OpView<float>&, const OpView<float>&,
                                   const IterView<float>&, const EvalView&, const RedView&, double*,
                                   double*, int, int, cudaStream_t);
template void launch_extract<double>(const Ctl*, const IterView<double>&, const EvalView&, double*,
                                     double*, double*, double*, cudaStream_t);
template void launch_extract<float>(const Ctl*, const IterView<float>&, const EvalView&, double*,
                                    double*, double*, double*, cudaStream_t);
template void launch_convert<double, float>(const double*, float*, long long, cudaStream_t);
template void launch_convert<float, double>(const float*, double*, long long, cudaStream_t);

}  // namespace sg
