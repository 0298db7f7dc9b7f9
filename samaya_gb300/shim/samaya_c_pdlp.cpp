// samaya_solve_params and samaya_solve_get_solution (samaya_c_pdlp.h): the additions a
// maintainer makes to samaya's src/core/c_api.cpp, beside samaya_solve (reference
// src/core/c_api.cpp:65-77), written against samaya's own headers.
#include "samaya_c_pdlp.h"

#include <cmath>
#include <limits>
#include <vector>

#include "samaya/solver.hpp"

// samaya's opaque model handle, as src/core/c_api.cpp:11-13 defines it.
struct samaya_model {
  samaya::Model model;
};

namespace {

struct LastSolution {
  bool present = false;
  bool verified = false;
  std::vector<double> col_value;
  std::vector<double> row_dual;
};

thread_local LastSolution g_last;

}  // namespace

extern "C" {

int samaya_solve_params(const samaya_model* model, int lp_method, int use_gpu, double time_limit,
                        double tol, double* objective) {
  if (objective != nullptr) *objective = std::numeric_limits<double>::quiet_NaN();
  g_last = LastSolution();
  if (model == nullptr) return SAMAYA_INVALID_MODEL;
  if (lp_method < SAMAYA_LP_AUTO || lp_method > SAMAYA_LP_CONCURRENT) return SAMAYA_INVALID_MODEL;
  try {
    samaya::Params params;
    params.log_level = 0;
    params.lp_method = static_cast<samaya::LpMethod>(lp_method);
    params.use_gpu = use_gpu != 0;
    if (time_limit > 0) params.time_limit = time_limit;
    if (tol > 0) {
      params.primal_feasibility_tol = tol;
      params.dual_feasibility_tol = tol;
    }
    samaya::Result result = samaya::Solver(params).solve(model->model);
    if (objective != nullptr) *objective = result.objective;
    if (!result.col_value.empty()) {
      g_last.present = true;
      g_last.verified = result.verified;
      g_last.col_value = std::move(result.col_value);
      g_last.row_dual = std::move(result.row_dual);
    }
    return static_cast<int>(result.status);
  } catch (...) {
    return SAMAYA_NUMERICAL_ERROR;
  }
}

int samaya_solve_get_solution(double* col_value, int ncols, double* row_dual, int nrows,
                              int* verified) {
  if (!g_last.present) return 1;
  if (col_value != nullptr) {
    if (static_cast<size_t>(ncols) != g_last.col_value.size()) return 1;
    for (int j = 0; j < ncols; ++j) col_value[j] = g_last.col_value[static_cast<size_t>(j)];
  }
  if (row_dual != nullptr) {
    if (static_cast<size_t>(nrows) != g_last.row_dual.size()) return 1;
    for (int i = 0; i < nrows; ++i) row_dual[i] = g_last.row_dual[static_cast<size_t>(i)];
  }
  if (verified != nullptr) *verified = g_last.verified ? 1 : 0;
  return 0;
}

}  // extern "C"
