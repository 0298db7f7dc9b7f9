// Batched PDLP (see sg_batch.cu): device views and the host engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "sg_common.cuh"

namespace sg {

struct MatInfo {
  double eta;              // 0.99 / ||[A_eq -I]||
  double a_norm_max_col;   // relative-residual scales of the original matrix
  double at_norm_max_row;
  double pad;
};

struct InstResult {
  int status;
  int pad;
  long long iterations;
  double rel_primal, rel_dual, rel_gap, primal_obj, dual_obj;
  long long restarts;
};

struct BatchView {
  int nmat, count;
  const int* mat_m;
  const int* mat_n;
  const long long* mat_nnz_off;   // nmat + 1
  const long long* mat_kptr_off;  // start of each matrix's row starts (m + 1 entries each)
  const long long* mat_tptr_off;  // start of each matrix's column starts (n + 1 entries each)
  const long long* mat_col_off;   // start of each matrix's column scales (n each)
  const long long* mat_row_off;   // start of each matrix's row scales (m each)
  const int* k_ptr;
  const int* k_idx;
  double* k_val;
  const double* k_val0;
  float* k_val32;
  const int* t_ptr;
  const int* t_idx;
  double* t_val;
  const double* t_val0;
  float* t_val32;
  double* cs;
  double* rs;
  double* cn;
  double* rn;
  double* pu;
  double* pv;
  MatInfo* info;
  const double* power_start;
  // Instances.
  const int* inst_mat;
  const long long* vec_off;    // cost/lower/upper/x offsets (n + m each)
  const long long* row_off;    // y offsets (m each)
  const long long* state_off;  // iterate storage offsets (in elements of the storage type)
  const double* cost;
  const double* lower;
  const double* upper;
  void* state;
  double* x_out;
  double* y_out;
  InstResult* results;
  const int* order;
  unsigned* queue;
  long long total_nnz;
  long long max_iter;
  double tol;
  const unsigned long long* deadline;  // device word: %globaltimer deadline, 0 = none
  int algorithm;     // 0 reference, 1 enhanced, 2 Halpern (enhanced preconditioning)
  int fp32;
  double art_frac;   // forced restart once the iterations since the last reach this fraction
};

// Unrolled PDHG of every instance (the differentiable layer's forward and adjoint).
struct UnrollView {
  int iterations;            // K
  int every;                 // checkpoint interval
  int nck;                   // checkpoints per instance, ceil(K / every)
  const long long* ck_off;   // per instance: first double of its checkpoints
  const long long* mask_off; // per instance: first byte of its segment masks
  double* ck;                // checkpoints: nck x (v: n+m, v_bar: n+m, y: m)
  unsigned char* mask;       // every x (n+m): 0 inside, 1 at lower, 2 at upper
  double* v_out;             // v_K in the LpProblem's space (n+m per instance, vec_off)
  const double* grad_v;      // adjoint of v_K (n+m per instance, vec_off)
  double* grad_cost;         // outputs (n+m per instance, vec_off)
  double* grad_lower;
  double* grad_upper;
};

void launch_batch(const BatchView& b, int solve_grid, unsigned long long budget_ns,
                  cudaStream_t s);
void launch_batch_setup(const BatchView& b, cudaStream_t s);
void launch_unroll(const BatchView& b, const UnrollView& u, int adjoint, int grid,
                   cudaStream_t s);
int batch_threads();

class Batch {
 public:
  ~Batch();
  static int create(Batch** out, int nmat, const int* mat_m, const int* mat_n,
                    const int64_t* mat_colptr, const int32_t* mat_rowidx, const double* mat_val,
                    int count, const int* inst_mat, const double* cost, const double* lower,
                    const double* upper, double tol, long long max_iter, double time_limit,
                    int precision, int algorithm, std::string* err);
  int solve(InstResult* results, double* x, double* y, double* device_ms, std::string* err);
  // Differentiable layer: K fixed-step PDHG iterations of every instance (v_K out, n+m per
  // instance) and the adjoint of v_K with respect to cost, lower and upper.
  int unroll(int iterations, int every, double* v_out, std::string* err);
  int unroll_adjoint(const double* grad_v, double* grad_cost, double* grad_lower,
                     double* grad_upper, std::string* err);
  long long total_vec() const { return total_vec_; }
  long long total_rows() const { return total_rows_; }

 private:
  Batch() = default;
  BatchView v_{};
  std::vector<void*> allocs_;
  cudaStream_t stream_ = nullptr;
  int grid_ = 1;
  long long total_vec_ = 0, total_rows_ = 0;
  double time_limit_ = 0.0;
  // Unrolled PDHG: the host copies of the per-instance offsets and the device buffers.
  UnrollView u_{};
  std::vector<long long> vec_off_host_;
  std::vector<int> inst_nt_host_, inst_m_host_;
  bool unrolled_ = false;
  template <typename T>
  int alloc(T** p, size_t count);
};

}  // namespace sg
