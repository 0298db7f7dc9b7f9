// samaya's host setup of a model on the device: compute_scaling + make_problem (reference
// src/linalg/scaling.cpp:79-149, src/lp/lp_solver.cpp:28-51) and the CSC -> CSR transpose of
// the engine's row-major copy (src/linalg/sparse_matrix.cpp:48-78), giving the bits the host's
// sg_scale_model and sg_csc_to_csr give.
#pragma once

#include <stdint.h>

#include <string>

#include "sg_engine.cuh"

namespace sg {

// A model in the form of sg_scale_model's arguments (host arrays).
struct ModelView {
  int m = 0, n = 0;
  const int64_t* colptr = nullptr;
  const int32_t* rowidx = nullptr;
  const double* val = nullptr;
  const double* obj = nullptr;
  const double* col_lower = nullptr;
  const double* col_upper = nullptr;
  const double* row_lower = nullptr;
  const double* row_upper = nullptr;
  int maximize = 0;
};

// The LpProblem of the model built on the device, copied back to host arrays with
// sg_scale_model's layout (lp_rowidx / lp_val sized by the model's nonzeros).
int scale_model_device(const ModelView& mv, int64_t* lp_colptr, int32_t* lp_rowidx,
                       double* lp_val, double* cost, double* lower, double* upper,
                       double* col_scale, double* row_scale, int64_t* lp_nnz, std::string* err);

// An engine for an LpProblem on the host (the arguments of sg_pdlp_create), the row-major copy
// of A built on the device.
int create_engine_from_lp(Engine** out, int m, int n, const int64_t* colptr,
                          const int32_t* rowidx, const double* val, const double* cost,
                          const double* lower, const double* upper, const Options& opt,
                          std::string* err);

// An engine for the model's LpProblem, built on the device without a host round trip of the
// scaled matrix or a host transpose; the scale factors are copied out (either may be null).
int create_engine_from_model(Engine** out, const ModelView& mv, const Options& opt,
                             double* col_scale, double* row_scale, std::string* err);

}  // namespace sg
