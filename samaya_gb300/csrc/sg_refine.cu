// Mixed precision with iterative refinement (the engine's own addition; the reference is FP64
// only). The FP64 point (v*, y*) of the equilibrated problem is refined by FP32 PDHG solves of
// scaled correction problems (Gleixner, Steffy & Wolter's LP iterative refinement applied to
// PDLP's computational form):
//   correction:  min (dd d)'w  s.t.  [A_eq -I] w = dp b,  dp (l - v*) <= w <= dp (u - v*),
//   with b = -[A_eq -I] v* (primal residual) and d = c + [A_eq -I]' y* (reduced costs), both in
//   FP64 from the FP64 matrix; then v* += w / dp and y* += z / dd for the correction's duals z.
// dp and dd are the inverse largest primal and dual violations (growth capped per round), so
// every correction problem is well scaled for FP32 arithmetic.
#include <math.h>

#include "sg_kernels.cuh"
#include "sg_refine.cuh"
#include "sg_tile.cuh"

namespace sg {

namespace {

// Dual violation of a reduced cost g at a point v in [lo, up]: the part of g that the point's
// active bounds cannot absorb (a positive g needs v at its lower bound, a negative g v at its
// upper bound). This covers dual infeasibility and complementarity, so a correction problem is
// scaled to what is still wrong even when every variable is boxed.
__device__ __forceinline__ double dual_violation(double g, double v, double lo, double up) {
  const bool at_lo = lo > -INFINITY && v <= lo;
  const bool at_up = up < INFINITY && v >= up;
  if (g > 0.0) return at_lo ? 0.0 : g;
  if (g < 0.0) return at_up ? 0.0 : -g;
  return 0.0;
}

struct Gather64 {
  const double* x;
  __device__ __forceinline__ double operator()(int, double a, int j) const { return a * x[j]; }
};

// Rows: b_i = -(A_eq x* - r*)_i, the logicals' reduced cost d_{n+i} = c_{n+i} - y*_i and its
// dual violation; max |b| and max violation.
struct ResRowEpi {
  const double* v;  // v* (n + m)
  const double* y;
  const double* cost;
  const double* lower;
  const double* upper;
  double* bh;
  double* d;
  int n;
  double acc[2];
  double* long_terms;
  __device__ __forceinline__ void terms(int i, double s, double (&a)[2]) {
    const double b = -(s - v[n + i]);
    bh[i] = b;
    const double g = cost[n + i] - y[i];
    d[n + i] = g;
    const double viol = dual_violation(g, v[n + i], lower[n + i], upper[n + i]);
    a[0] = fmax(a[0], fabs(b));
    a[1] = fmax(a[1], viol);
  }
  __device__ __forceinline__ void row(int i, const double (&s)[1]) { terms(i, s[0], acc); }
  __device__ __forceinline__ void long_row(int lrow, int i, const double (&s)[1]) {
    double a[2] = {0.0, 0.0};
    terms(i, s[0], a);
    long_terms[lrow * kMaxSums + 0] = a[0];
    long_terms[lrow * kMaxSums + 1] = a[1];
  }
};

// Columns: d_j = c_j + (A_eq' y*)_j and its dual violation.
struct ResColEpi {
  const double* v;
  const double* cost;
  const double* lower;
  const double* upper;
  double* d;
  double acc[2];
  double* long_terms;
  __device__ __forceinline__ void terms(int j, double s, double (&a)[2]) {
    const double g = cost[j] + s;
    d[j] = g;
    a[1] = fmax(a[1], dual_violation(g, v[j], lower[j], upper[j]));
  }
  __device__ __forceinline__ void row(int j, const double (&s)[1]) { terms(j, s[0], acc); }
  __device__ __forceinline__ void long_row(int lrow, int j, const double (&s)[1]) {
    double a[2] = {0.0, 0.0};
    terms(j, s[0], a);
    long_terms[lrow * kMaxSums + 0] = a[0];
    long_terms[lrow * kMaxSums + 1] = a[1];
  }
};

__global__ void __launch_bounds__(kBlock) ir_rows_kernel(Ctl* c, OpView<double> K, IrView v) {
  ResRowEpi epi;
  epi.v = v.v;
  epi.y = v.y;
  epi.cost = v.cost_eq;
  epi.lower = v.lower_eq;
  epi.upper = v.upper_eq;
  epi.bh = v.bh;
  epi.d = v.d;
  epi.n = v.n;
  epi.acc[0] = epi.acc[1] = 0.0;
  epi.long_terms = v.red.long_terms;
  run_tiles<double, double, 1>(K.ts, K.ptr, K.idx, K.val, Gather64{v.v}, epi);
  grid_reduce<2, 3u>(epi.acc, v.red.partial, v.red.counter, smem_red(),
                     [c](const double (&t)[2]) {
    c->ir_pmax = t[0];
    c->ir_dmax = t[1];
  }, v.red.long_terms, K.ts.nlong);
}

__global__ void __launch_bounds__(kBlock) ir_cols_kernel(Ctl* c, OpView<double> Kt, IrView v) {
  ResColEpi epi;
  epi.v = v.v;
  epi.cost = v.cost_eq;
  epi.lower = v.lower_eq;
  epi.upper = v.upper_eq;
  epi.d = v.d;
  epi.acc[0] = epi.acc[1] = 0.0;
  epi.long_terms = v.red.long_terms;
  run_tiles<double, double, 1>(Kt.ts, Kt.ptr, Kt.idx, Kt.val, Gather64{v.y}, epi);
  grid_reduce<2, 3u>(epi.acc, v.red.partial, v.red.counter, smem_red(),
                     [c](const double (&t)[2]) {
    c->ir_dmax = fmax(c->ir_dmax, t[1]);
  }, v.red.long_terms, Kt.ts.nlong);
}

// Scale factors of the correction problem and its starting primal weight.
__global__ void ir_scales_kernel(Ctl* c, int round, double growth) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (round == 0) {
    c->ir_dp_prev = 1.0;
    c->ir_dd_prev = 1.0;
    c->ir_dp = 1.0;
    c->ir_dd = 1.0;
    c->omega = c->ir_omega0;
  } else {
    const double pm = fmax(c->ir_pmax, 1e-300);
    const double dm = fmax(c->ir_dmax, 1e-300);
    const double dp_prev = c->ir_dp;
    const double dd_prev = c->ir_dd;
    const double dp = fmin(1.0 / pm, dp_prev * growth);
    const double dd = fmin(1.0 / dm, dd_prev * growth);
    c->ir_dp_prev = dp_prev;
    c->ir_dd_prev = dd_prev;
    c->ir_dp = dp;
    c->ir_dd = dd;
    // The correction scales primal by dp and dual by dd: carry the weight over accordingly,
    // within four orders of magnitude of the first round's.
    const double w = c->omega * (dd / dd_prev) / (dp / dp_prev);
    c->omega = fmin(fmax(w, 1e-4 * c->ir_omega0), 1e4 * c->ir_omega0);
  }
  c->tau = c->eta / c->omega;
  c->sigma = c->eta * c->omega;
}

// Builds the correction problem (FP64 evaluation copy and FP32 iteration copy) and zeroes the
// FP32 iterates.
__global__ void ir_build_kernel(const Ctl* __restrict__ c, IrView v, int round) {
  const double dp = c->ir_dp;
  const double dd = c->ir_dd;
  const int n = v.n;
  const int nt = n + v.m;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
    double cc, lo, up;
    if (round == 0) {
      cc = v.cost_eq[k];
      lo = v.lower_eq[k];
      up = v.upper_eq[k];
    } else {
      cc = dd * v.d[k];
      lo = dp * (v.lower_eq[k] - v.v[k]);
      up = dp * (v.upper_eq[k] - v.v[k]);
    }
    v.cost_in[k] = cc;
    v.lower_in[k] = lo;
    v.upper_in[k] = up;
    v.cost32[k] = static_cast<float>(cc);
    v.lower32[k] = static_cast<float>(lo);
    v.upper32[k] = static_cast<float>(up);
    if (k >= n) {
      const int i = k - n;
      const double q = round == 0 ? 0.0 : dp * v.bh[i];
      v.rhs_in[i] = q;
      v.rhs32[i] = static_cast<float>(q);
    }
  }
}

// v* += w / dp, y* += z / dd from the FP32 answer (current or average iterate), then v* back
// inside its bounds; round 0 takes the FP32 answer as the point.
__global__ void ir_update_kernel(const Ctl* __restrict__ c32, IterView<float> it, IrView v,
                                 int round) {
  const int cur = static_cast<int>(c32->t & 1);
  const bool avg = c32->result_average != 0;
  const float* w = avg ? it.Verg : it.v(cur);
  const float* z = avg ? it.Yerg : it.y(cur);
  const double dp = c32->ir_dp;
  const double dd = c32->ir_dd;
  const int nt = v.n + v.m;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
    double nv = round == 0 ? static_cast<double>(w[k]) : v.v[k] + static_cast<double>(w[k]) / dp;
    nv = fmin(fmax(nv, v.lower_eq[k]), v.upper_eq[k]);
    v.v[k] = nv;
    if (k < v.m) {
      v.y[k] = round == 0 ? static_cast<double>(z[k]) : v.y[k] + static_cast<double>(z[k]) / dd;
    }
  }
}

// Resets the inner solve's control block for a new correction problem.
__global__ void ir_reset_kernel(Ctl* c, double tol, long long max_iter, int stall_limit) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  c->stall_best = INFINITY;
  c->stall_floor = fmin(1e-4, 100.0 * tol);
  c->stall_evals = 0;
  c->stall_limit = stall_limit;
  c->t = 0;
  c->k = 0;
  c->max_iter = max_iter;
  c->tol = tol;
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
  c->no_detect = 1;
}

// Precision switch: the whole FP32 state as doubles (both ping-pong iterates, the
// extrapolated point, the averages and the restart point), so the FP64 PDLP continues the same
// run rather than restarting at its answer.
__global__ void continue_vectors_kernel(IterView<float> a, IterView<double> b) {
  const int nt = b.n + b.m;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
    b.V[0][k] = static_cast<double>(a.V[0][k]);
    b.V[1][k] = static_cast<double>(a.V[1][k]);
    b.Vbar[k] = static_cast<double>(a.Vbar[k]);
    b.Verg[k] = static_cast<double>(a.Verg[k]);
    b.Vrst[k] = static_cast<double>(a.Vrst[k]);
    if (k < b.m) {
      b.Y[0][k] = static_cast<double>(a.Y[0][k]);
      b.Y[1][k] = static_cast<double>(a.Y[1][k]);
      b.Yerg[k] = static_cast<double>(a.Yerg[k]);
      b.Yrst[k] = static_cast<double>(a.Yrst[k]);
    }
  }
}

// The FP64 control block continues the FP32 one: iteration counters (parity and the averages'
// weights), primal weight and steps; the restart references start afresh because the FP64
// evaluation measures the original problem and the FP32 one the equilibrated problem.
__global__ void continue_ctl_kernel(Ctl* c, const Ctl* __restrict__ c32) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  c->t = c32->t;
  c->k = c32->k;
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
  c->omega = c32->omega;
  c->tau = c->eta / c->omega;
  c->sigma = c->eta * c->omega;
}

// The FP64 iterates, average and restart point = the FP64 point V[0], Y[0].
__global__ void point_vectors_kernel(IterView<double> it) {
  const int nt = it.n + it.m;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
    const double v = it.V[0][k];
    it.V[1][k] = v;
    it.Vbar[k] = v;
    it.Verg[k] = v;
    it.Vrst[k] = v;
    if (k < it.m) {
      const double yv = it.Y[0][k];
      it.Y[1][k] = yv;
      it.Yerg[k] = yv;
      it.Yrst[k] = yv;
    }
  }
}

// Restarted FP64 control block; the primal weight from c32 when given, else `omega`.
__global__ void switch_ctl_kernel(Ctl* c, const Ctl* __restrict__ c32, double omega,
                                  long long max_iter) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  c->t = 0;
  c->k = 0;
  c->max_iter = max_iter > 0 ? max_iter : 1;
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
  c->omega = c32 != nullptr ? c32->omega : omega;
  c->tau = c->eta / c->omega;
  c->sigma = c->eta * c->omega;
}

__global__ void __launch_bounds__(kBlock) norm_into_kernel(const double* x, int len, RedView red,
                                                           double* out) {
  __shared__ double scratch[kMaxSums * (kBlock / 32)];
  double a[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < len; k += gridDim.x * blockDim.x) {
    a[0] += x[k] * x[k];
  }
  grid_reduce<1>(a, red.partial, red.counter, scratch,
                 [out](const double (&t)[1]) { *out = sqrt(t[0]); });
}

int grid_for(long long len, int cap) {
  long long g = (len + kBlock - 1) / kBlock;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return static_cast<int>(g);
}

}  // namespace

void configure_refine_kernels() {
  const int big = 200 * 1024;
  cudaFuncSetAttribute(ir_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(ir_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
}

void launch_ir_residual(Ctl* c32, const OpView<double>& K, const OpView<double>& Kt,
                        const IrView& v, int grid_k, int grid_t, cudaStream_t s) {
  ir_rows_kernel<<<grid_k, kBlock, tile_smem_bytes(K.ts, 1, 8), s>>>(c32, K, v);
  ir_cols_kernel<<<grid_t, kBlock, tile_smem_bytes(Kt.ts, 1, 8), s>>>(c32, Kt, v);
}

void launch_ir_scales(Ctl* c32, int round, double growth, cudaStream_t s) {
  ir_scales_kernel<<<1, 32, 0, s>>>(c32, round, growth);
}

void launch_ir_build(const Ctl* c32, const IrView& v, int round, cudaStream_t s) {
  ir_build_kernel<<<grid_for(v.n + v.m, 4096), kBlock, 0, s>>>(c32, v, round);
}

void launch_ir_update(const Ctl* c32, const IterView<float>& it, const IrView& v, int round,
                      cudaStream_t s) {
  ir_update_kernel<<<grid_for(v.n + v.m, 4096), kBlock, 0, s>>>(c32, it, v, round);
}

void launch_ir_reset(Ctl* c32, double tol, long long max_iter, int stall_limit,
                     cudaStream_t s) {
  ir_reset_kernel<<<1, 32, 0, s>>>(c32, tol, max_iter, stall_limit);
}

void launch_continue(Ctl* c64, const Ctl* c32, const IterView<float>& it32,
                     const IterView<double>& it64, cudaStream_t s) {
  continue_vectors_kernel<<<grid_for(static_cast<long long>(it64.n) + it64.m, 4096), kBlock, 0,
                            s>>>(it32, it64);
  continue_ctl_kernel<<<1, 32, 0, s>>>(c64, c32);
}

void launch_restart_at_point(Ctl* c64, double omega, const IterView<double>& it64,
                             long long max_iter, cudaStream_t s) {
  point_vectors_kernel<<<grid_for(static_cast<long long>(it64.n) + it64.m, 4096), kBlock, 0,
                         s>>>(it64);
  switch_ctl_kernel<<<1, 32, 0, s>>>(c64, nullptr, omega, max_iter);
}

void launch_norm_into(const double* x, long long len, const RedView& red, double* out,
                      cudaStream_t s) {
  norm_into_kernel<<<grid_for(len, 1024), kBlock, 0, s>>>(x, static_cast<int>(len), red, out);
}

}  // namespace sg
