// Iterative-refinement kernels of the FP32 path (see sg_refine.cu).
#pragma once

#include "sg_kernels.cuh"

namespace sg {

// Arrays of the refinement (equilibrated space).
struct IrView {
  double* v;               // FP64 point v* (n + m)
  double* y;               // FP64 duals y* (m)
  const double* cost_eq;   // equilibrated problem (n + m)
  const double* lower_eq;
  const double* upper_eq;
  double* bh;              // primal residual -[A_eq -I] v* (m)
  double* d;               // reduced costs c + [A_eq -I]' y* (n + m)
  double* cost_in;         // correction problem, FP64 (evaluation) copy
  double* lower_in;
  double* upper_in;
  double* rhs_in;          // m
  float* cost32;           // correction problem, FP32 (iteration) copy
  float* lower32;
  float* upper32;
  float* rhs32;
  RedView red;
  int n, m;
};

void configure_refine_kernels();
void launch_ir_residual(Ctl* c32, const OpView<double>& K, const OpView<double>& Kt,
                        const IrView& v, int grid_k, int grid_t, cudaStream_t s);
void launch_ir_scales(Ctl* c32, int round, double growth, cudaStream_t s);
void launch_ir_build(const Ctl* c32, const IrView& v, int round, cudaStream_t s);
void launch_ir_update(const Ctl* c32, const IterView<float>& it, const IrView& v, int round,
                      cudaStream_t s);
// Restarts the FP32 control block for a solve to `tol` within `max_iter` iterations, with the
// stall test after `stall_limit` evaluations without progress (0: off).
void launch_ir_reset(Ctl* c32, double tol, long long max_iter, int stall_limit,
                     cudaStream_t s);
constexpr int kStallEvaluations = 64;
void launch_norm_into(const double* x, long long len, const RedView& red, double* out,
                      cudaStream_t s);
// Precision switch: the FP64 state = the FP32 state (iterates, extrapolated point, averages,
// restart point; iteration counters and primal weight), so the FP64 PDLP continues the run.
void launch_continue(Ctl* c64, const Ctl* c32, const IterView<float>& it32,
                     const IterView<double>& it64, cudaStream_t s);
// The same from the FP64 point V[0], Y[0] of it64 with primal weight `omega`.
void launch_restart_at_point(Ctl* c64, double omega, const IterView<double>& it64,
                             long long max_iter, cudaStream_t s);

}  // namespace sg
