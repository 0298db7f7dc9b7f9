// Shared device-side definitions of the GB300 PDLP engine.
//
// Layout in HBM (one LP, computational form min c'v s.t. [A -I] v = 0, l <= v <= u, v = (x, r)):
//   K   = A_eq (m x n) by rows   : kptr int32[m+1], kidx int32[nnz], kval T[nnz]
//   Kt  = A_eq^T (n x m) by rows : tptr int32[n+1], tidx int32[nnz], tval T[nnz]
//   iterates (T)                  : V[2][n+m] (ping-pong by step parity), Vbar[n+m],
//                                   Y[2][m], Verg[n+m], Yerg[m], Vrst[n+m], Yrst[m]
//   problem vectors (T)           : cost/lower/upper after equilibration (n+m)
//   evaluation data (FP64)        : col/row scales, cost/lower/upper before equilibration
//   control block (FP64 scalars)  : step sizes, counters, status, restart state (Ctl)
// Both operators are split into tiles of at most kTileNnz nonzeros (rows longer than that are
// cut into segments whose partial sums are combined in a fixed order), so every CTA streams a
// similar number of bytes whatever the row-length distribution (power-law rows included).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sg {

constexpr int kBlock = 256;          // threads per CTA in the tile kernels
constexpr int kTileNnz = 4096;       // nonzeros staged per tile
constexpr int kTileRows = 1024;      // rows per tile at most
constexpr int kMaxSums = 24;         // FP64 sums reduced by one evaluation kernel
constexpr int kCheckFrequency = 64;  // iterations between evaluations (pdlp.cpp:25)

// One CTA's share of an operator. kind 0: rows [r0, r1) whole, nonzeros [k0, k1);
// kind 1: one segment [k0, k1) of long row r0 (r1 = r0 + 1), segment `seg` of `nseg`, long
// row id `lrow` (its partials are combined by the last segment to finish); kind 2: rows
// [r0, r1) of medium length, `team` warps each; kind 3 (dual step tile sets only): a group of
// up to 32 consecutive rows [r0, r1) whose k-th nonzeros lie in neighbouring columns, nonzero
// positions [k0, k1) within each row (segment `seg` of `nseg`; counter `lrow` when nseg > 1).
struct Tile {
  int r0, r1;
  int k0, k1;
  int kind;
  int team;  // kind 2: warps per row (1, 2, 4 or 8); 1 otherwise
  int seg, nseg;
  int lrow;
  int pad[3];
};

struct TileSet {
  const Tile* tiles;
  int ntiles;
  int nlong;        // number of split rows
  double* seg_part; // [ntiles * kMaxVec] partial sums of long-row segments
  unsigned* lcount; // [nlong] arrival counters (reset by the last arrival)
  int cap_nnz;      // nonzeros per tile at most (shared-memory staging capacity)
  int cap_rows;     // rows per tile at most
  int variant;      // step kernels: 0 high occupancy, 1 deep unroll of medium and long rows
  // Null: the tiles' rows are the operator's rows. Otherwise the tiles cover a subsequence of
  // the rows (rows that are left out are empty, so every nonzero position is unchanged), and
  // a tile's row index v stands for rows[v].
  const int* rows;
  int groups;         // kind-3 tiles in the set (0: none; only the dual step kernels take them)
  double* grp_part;   // [ntiles * 32] partial sums of kind-3 segments (when groups > 0)
  // L > 0: every row of the operator has exactly L nonzeros (row r starts at r L), so the
  // short-row tiles read no row starts (the columns of a transportation or network-flow LP:
  // two nonzeros each); 0 otherwise.
  int uniform_len;
  // 1: the kind-1 segments are streamed through shared memory by bulk copies (dual step tile
  // sets only; the operator's index and value arrays then carry kSegPad elements of padding).
  int staged;
  int* wait_error;  // set to 1 when a bounded wait for a bulk copy gave up (staged sets)
};

constexpr int kSegChunk = 2048;  // nonzeros per bulk-copied chunk of a staged segment
constexpr int kSegPad = 4;       // padding elements after an operator's nonzeros

constexpr int kGroupRows = 32;  // rows of a kind-3 tile at most (a warp's lanes)
constexpr int kGroupPos = 16;   // nonzero positions per row staged per warp and round

__device__ __forceinline__ int tile_row(const TileSet& ts, int v) {
  return ts.rows != nullptr ? __ldg(ts.rows + v) : v;
}

constexpr int kMaxVec = 2;
constexpr int kWarpRowMin = 128;             // rows longer than this get a warp (tile kind 2)
constexpr int kWarpsPerTile = kBlock / 32;   // rows of a kind-2 tile

// Status values (the reference's SimplexStatus, src/lp/simplex.hpp:28-35) plus "running".
enum : int {
  kOptimal = 0,
  kInfeasible = 1,
  kUnbounded = 2,
  kIterationLimit = 3,
  kTimeLimit = 4,
  kNumericalError = 5,
  kRunning = -1,
};

// Control block: written by the single-CTA decision kernels, read by every other kernel, so the
// whole iteration loop runs from a CUDA graph without the host.
struct Ctl {
  // Step sizes (pdlp.cpp:311-315, 1105-1109).
  double eta, omega, tau, sigma;
  // Iteration counters: t = iterations done (the reference's `iter` + 1 at an evaluation),
  // k = iterations since the last restart.
  long long t, k, max_iter;
  // Restart state (pdlp.cpp:397-398).
  double kkt_at_restart, kkt_previous;
  // Constants of the relative residuals (pdlp.cpp:377-394, 490-492).
  double a_norm_max_col, at_norm_max_row, c_norm;
  // Evaluation sums of the row kernel and the column kernel: [w * 7 + q] for w = current (0) /
  // average (1) and q = primal_sq, dual_sq, primal_obj, dual_obj, x_sq, r_sq, y_sq; then the
  // restart distances [14] |v_cur - v_rst|^2, [15] |y_cur - y_rst|^2, [16] |v_avg - v_rst|^2,
  // [17] |y_avg - y_rst|^2.
  double eval_r[kMaxSums];
  double eval_c[kMaxSums];
  // The measures of the last evaluation: [w][rel_primal, rel_dual, rel_gap, pobj, dobj].
  double meas[2][5];
  // Outcome.
  int status;           // kRunning while iterating
  int done;             // every iteration kernel returns at once when set
  int result_average;   // 1: the answer is the average iterate
  int restart_pending;  // 1: restart_kernel copies the candidate
  int restart_to_avg;   // candidate of the pending restart
  int detect_pending;   // 1: detection kernels run at this evaluation
  int ruiz_done;        // setup: Ruiz converged
  int power_done;       // setup: power iteration met a zero vector
  long long iterations; // iteration count of the answer
  double res[3];        // relative primal, dual, gap of the answer
  double pobj, dobj;    // objectives of the answer (LpProblem space)
  long long restarts, evaluations;
  unsigned long long deadline_ns;  // %globaltimer deadline, 0 = none
  int m, n;
  double tol;
  // Setup scalars.
  double power_sigma, power_unorm, power_vnorm, op_norm;
  // Detection scalars: [0] y_max, [1] w_scale, [2] min_f, [3] max_f, [4] scale, [5] v_max,
  // [6] primal_feas, [7] cost_dir; flags: [0] infeasible found, [1] unbounded found,
  // [2] min_f infinite, [3] max_f infinite, [4] ray bounds ok, [5] stage.
  double det[8];
  int det_flags[8];
  double last_kkt;
  // Iterative refinement (FP32 path): |q| of the inner problem's right-hand side (added to the
  // primal scale; 0 for the reference problem), the residual maxima of the FP64 point, and the
  // primal / dual scale factors of the current and previous correction problems.
  double q_norm;
  double ir_pmax, ir_dmax;
  double ir_dp, ir_dd, ir_dp_prev, ir_dd_prev;
  double ir_omega0;
  int no_detect;  // 1: no infeasibility/unboundedness checks (the refinement's inner solves)
  int halpern;    // 1: reflected Halpern PDHG (the answer and restarts use T(z), the second
                  // evaluated iterate; the Halpern iterate itself may leave the bounds)
  // Stall test of the FP32 solves: stop when the better iterate's largest relative residual has
  // not fallen below 0.8 x its best for stall_limit evaluations (0: off) while below
  // stall_floor, or for 8 x stall_limit evaluations above it (there a slow stretch is more
  // often the method's own, which FP64 would crawl through too, than FP32's precision floor).
  double stall_best;
  double stall_floor;
  int stall_evals;
  int stall_limit;
  // Artificial restart: a restart is forced once the iterations since the last one reach this
  // fraction of all iterations (the reference's 0.36, pdlp.cpp:1075-1131; the engine's own
  // algorithms default to 0.1).
  double art_frac;
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}

// Deterministic block reduction of K sums (fixed shuffle tree, then fixed tree over warps).
// Every thread passes its K values; thread 0 receives the totals in `out`. `scratch` holds
// K * (kBlock / 32) doubles.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* scratch, double (&out)[K]) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int kWarps = kBlock / 32;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    double s = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) scratch[q * kWarps + warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      double s = scratch[q * kWarps];
      for (int w = 1; w < kWarps; ++w) s += scratch[q * kWarps + w];
      out[q] = s;
    }
  }
  __syncthreads();
}

template <int K>
__device__ __forceinline__ void block_max(double (&v)[K], double* scratch, double (&out)[K]) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int kWarps = kBlock / 32;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    double s = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_down_sync(0xffffffffu, s, o));
    if (lane == 0) scratch[q * kWarps + warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      double s = scratch[q * kWarps];
      for (int w = 1; w < kWarps; ++w) s = fmax(s, scratch[q * kWarps + w]);
      out[q] = s;
    }
  }
  __syncthreads();
}

// Deterministic block reduction with a per-entry choice of sum or max (bit q of MAXMASK).
template <int K, unsigned MAXMASK>
__device__ __forceinline__ void block_reduce(double (&v)[K], double* scratch, double (&out)[K]) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int kWarps = kBlock / 32;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    const bool mx = (MAXMASK >> q) & 1u;
    double s = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_down_sync(0xffffffffu, s, o);
      s = mx ? fmax(s, t) : s + t;
    }
    if (lane == 0) scratch[q * kWarps + warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      const bool mx = (MAXMASK >> q) & 1u;
      double s = scratch[q * kWarps];
      for (int w = 1; w < kWarps; ++w) s = mx ? fmax(s, scratch[q * kWarps + w]) : s + scratch[q * kWarps + w];
      out[q] = s;
    }
  }
  __syncthreads();
}

// Grid-level deterministic reduction: each CTA reduces its threads' K values (fixed tree) and
// stores them in partial[b * K + q]; the last CTA to arrive (counter) combines the CTAs in a
// fixed order (thread t takes CTAs t, t + 256, ... in order, then the fixed block tree) and
// calls `fin(totals)` from thread 0. The counter is reset by the last CTA so the kernel can be
// replayed from a CUDA graph. Must be reached by every thread of every CTA.
// `extra` (nextra records of stride kMaxSums, e.g. the terms of rows split over several CTAs)
// is added by the last CTA too, spread over its threads in a fixed order.
template <int K, unsigned MAXMASK = 0u, typename Fin>
__device__ __forceinline__ void grid_reduce(double (&mine)[K], double* partial,
                                            unsigned* counter, double* scratch, Fin fin,
                                            const double* extra = nullptr, int nextra = 0) {
  __shared__ bool last;
  double blk[K];
  block_reduce<K, MAXMASK>(mine, scratch, blk);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) partial[blockIdx.x * K + q] = blk[q];
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc[K];
#pragma unroll
  for (int q = 0; q < K; ++q) acc[q] = ((MAXMASK >> q) & 1u) ? -INFINITY : 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      const double p = __ldcg(&partial[b * K + q]);
      acc[q] = ((MAXMASK >> q) & 1u) ? fmax(acc[q], p) : acc[q] + p;
    }
  }
  for (int l = threadIdx.x; l < nextra; l += blockDim.x) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      const double p = __ldcg(&extra[l * kMaxSums + q]);
      acc[q] = ((MAXMASK >> q) & 1u) ? fmax(acc[q], p) : acc[q] + p;
    }
  }
  double tot[K];
  block_reduce<K, MAXMASK>(acc, scratch, tot);
  if (threadIdx.x == 0) {
    *counter = 0u;
    fin(tot);
  }
}

}  // namespace sg
