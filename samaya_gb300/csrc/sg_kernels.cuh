// Kernel interfaces of the GB300 PDLP engine (see sg_common.cuh for the HBM layout).
#pragma once

#include "sg_common.cuh"

namespace sg {

// An operator stored by rows (CSR) with its tile partition.
template <typename T>
struct OpView {
  const int* ptr;
  const int* idx;
  T* val;
  int rows;
  TileSet ts;
};

// Iterates and the equilibrated problem vectors, in storage type T.
template <typename T>
struct IterView {
  T* V[2];     // (x, r) ping-pong by step parity, n + m
  T* Vbar;     // extrapolated point of the next step, n + m
  T* Y[2];     // duals ping-pong, m
  T* Verg;     // running average since the last restart, n + m
  T* Yerg;     // m
  T* Vrst;     // restart point, n + m
  T* Yrst;     // m
  const T* cost;   // n + m
  const T* lower;  // n + m
  const T* upper;  // n + m
  const T* rhs;    // m right-hand side q of [A -I] v = q (null: zero)
  int n, m;
  // 1: every structural column has the bounds [xb_lo, xb_hi] (0 or infinite, so equilibration
  // keeps them), and the primal steps read no bound vectors (16 MB an FP32 primal step of the
  // transportation LP); 0: lower[j], upper[j].
  int xb_uniform;
  T xb_lo, xb_hi;
  // V[p], Y[p] by a select: indexing a kernel parameter's array with a runtime index makes
  // the compiler copy the whole view to local memory first.
  __host__ __device__ __forceinline__ T* v(int p) const { return p ? V[1] : V[0]; }
  __host__ __device__ __forceinline__ T* y(int p) const { return p ? Y[1] : Y[0]; }
};

// The data the evaluation maps iterates back with (FP64): equilibration factors and the
// problem before equilibration.
struct EvalView {
  const double* cs;      // n
  const double* rs;      // m
  const double* cost;    // n + m
  const double* lower;   // n + m
  const double* upper;   // n + m
  const double* rhs;     // m (null: zero)
  const double* inv_cs;  // 1 / cs and 1 / rs (the evaluation multiplies: divisions would load
  const double* inv_rs;  // GB300's small FP64 pipe)
};

// Scratch of the grid reductions.
struct RedView {
  double* partial;       // [max CTAs * kMaxSums]
  unsigned* counter;     // [8]
  double* long_terms;    // [nlong * kMaxSums]
};

constexpr int kEvalSums = 18;

template <typename T>
void launch_dual_step(const Ctl* ctl, const OpView<T>& K, const IterView<T>& it, int j,
                      int grid, cudaStream_t s);
template <typename T>
void launch_primal_step(const Ctl* ctl, const OpView<T>& Kt, const IterView<T>& it, int j,
                        int grid, cudaStream_t s);
// Reflected Halpern PDHG steps (primal launch first, then dual; see sg_kernels.cu).
template <typename T>
void launch_halpern_primal(const Ctl* ctl, const OpView<T>& Kt, const IterView<T>& it, int j,
                           int grid, cudaStream_t s);
template <typename T>
void launch_halpern_dual(const Ctl* ctl, const OpView<T>& K, const IterView<T>& it, int j,
                         int grid, cudaStream_t s);
template <typename T>
// second_only: measure the second slot (Verg, Yerg) alone; the first slot's sums are 0 (the
// Halpern solves decide on T(z) only).
void launch_eval(Ctl* ctl, const OpView<T>& K, const OpView<T>& Kt, const IterView<T>& it,
                 const EvalView& ev, const RedView& red, int grid_k, int grid_t,
                 int fixed_parity, cudaStream_t s, bool second_only = false);
void launch_decide_a(Ctl* ctl, cudaStream_t s);
void launch_decide_b(Ctl* ctl, cudaStream_t s);
template <typename T>
void launch_restart(const Ctl* ctl, const IterView<T>& it, cudaStream_t s);
template <typename T>
void launch_detect(Ctl* ctl, const OpView<T>& K, const OpView<T>& Kt, const IterView<T>& it,
                   const EvalView& ev, const RedView& red, double* scratch_n, double* scratch_nt,
                   int grid_k, int grid_t, cudaStream_t s);
template <typename T>
void launch_extract(const Ctl* ctl, const IterView<T>& it, const EvalView& ev, double* x_out,
                    double* y_out, double* dual_ray, double* primal_ray_src, cudaStream_t s);

// Setup on the device (FP64 master copy).
void launch_setup_norms(Ctl* ctl, const OpView<double>& K, const OpView<double>& Kt,
                        const double* cost, const RedView& red, int grid_k, int grid_t,
                        cudaStream_t s);
// out[k] = 1 / a[k] for k < count.
void launch_reciprocals(const double* a, double* out, int count, cudaStream_t s);
void launch_row_neighbours(int m, const int* ptr, const int* idx, unsigned char* out,
                           cudaStream_t s);
void launch_ruiz_pass(Ctl* ctl, const OpView<double>& K, const OpView<double>& Kt, double* rs,
                      double* cs, double* rn, double* cn, const RedView& red, int grid_k,
                      int grid_t, cudaStream_t s);
// Enhanced preconditioning: 10 passes of infinity-norm Ruiz, then Pock-Chambolle (alpha = 1).
void launch_enhanced_scaling(const OpView<double>& K, const OpView<double>& Kt, double* rs,
                             double* cs, double* rn, double* cn, int grid_k, int grid_t,
                             cudaStream_t s);
// Initial primal weight |c_eq| / |b_eq| (sets omega, tau, sigma; needs eta).
void launch_primal_weight_init(Ctl* ctl, int n, int m, const double* cost_eq,
                               const double* lower_eq, const double* upper_eq,
                               const RedView& red, cudaStream_t s);
void launch_apply_scaling(const OpView<double>& K, const OpView<double>& Kt, const double* rs,
                          const double* cs, long long nnz, cudaStream_t s);
void launch_scale_vectors(int n, int m, const double* cs, const double* rs, const double* cost,
                          const double* lower, const double* upper, const double* rhs,
                          double* cost_eq, double* lower_eq, double* upper_eq, double* rhs_eq,
                          cudaStream_t s);
void launch_power_iteration(Ctl* ctl, const OpView<double>& K, const OpView<double>& Kt,
                            double* u, double* v, const RedView& red, int iters, int grid_k,
                            int grid_t, cudaStream_t s);
void launch_init_state(Ctl* ctl, cudaStream_t s);
void launch_set_deadline(Ctl* ctl, double seconds, cudaStream_t s);

template <typename Src, typename Dst>
void launch_convert(const Src* src, Dst* dst, long long count, cudaStream_t s);

// Plain y = A x by rows through the tile kernel (diagnostics and the SpMV parity test).
void launch_spmv(const OpView<double>& A, const double* x, double* y, int grid, cudaStream_t s);

// Sizes of dynamic shared memory of the tile kernels.
size_t tile_smem_bytes(const TileSet& ts, int nv, size_t acc_bytes);
void configure_kernels();

}  // namespace sg
