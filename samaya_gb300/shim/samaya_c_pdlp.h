/* Additions to samaya's C API (reference include/samaya_c.h) that let a C caller choose the LP
 * method and the GPU, and read the solution back: the counterparts of the C++ Params fields
 * lp_method, use_gpu, time_limit and the tolerances (reference include/samaya/params.hpp:21-49),
 * which samaya_solve (samaya_c.h:39-41, src/core/c_api.cpp:65-77) leaves at their defaults
 * (lp_method kAuto, use_gpu false), so that a C caller could never reach the PDLP path or the
 * GPU.
 *
 * They belong beside samaya_solve in samaya's src/core/c_api.cpp (they use its samaya_model);
 * samaya_gb300/shim/samaya_c_pdlp.cpp is that code. Statuses are samaya_c.h's SAMAYA_* values.
 * Like the rest of samaya's C API they never throw. */
#ifndef SAMAYA_C_PDLP_H
#define SAMAYA_C_PDLP_H

#include "samaya_c.h"

#ifdef __cplusplus
extern "C" {
#endif

/* LP methods, identical in value to samaya::LpMethod (reference include/samaya/params.hpp:11-18). */
enum {
  SAMAYA_LP_AUTO = 0,
  SAMAYA_LP_DUAL_SIMPLEX = 1,
  SAMAYA_LP_PRIMAL_SIMPLEX = 2,
  SAMAYA_LP_BARRIER = 3,
  SAMAYA_LP_PDLP = 4,
  SAMAYA_LP_CONCURRENT = 5
};

/* Solves with the given LP method (SAMAYA_LP_*), GPU use (0 / 1: Params::use_gpu, which takes
 * PDLP to the GB300 engine when one is present and to the CPU PDLP otherwise), time limit in
 * seconds (<= 0: none) and tolerance (> 0: the primal and dual feasibility tolerances, which
 * also set PDLP's target, Params::dual_feasibility_tol; <= 0: the defaults). Every other
 * parameter keeps its default. Returns a status code; *objective receives the objective value
 * (NaN if no solution) when objective is non-NULL. The solution is kept for
 * samaya_solve_get_solution (per thread, until the next solve on that thread). */
int samaya_solve_params(const samaya_model* model, int lp_method, int use_gpu, double time_limit,
                        double tol, double* objective);

/* The last solution of this thread's samaya_solve_params: column values (ncols), row duals in
 * the convention d = c - A'y (nrows), and whether the verifier passed it (*verified, 0 / 1).
 * Any pointer may be NULL. Returns 0, or 1 when there is no solution or the sizes differ. */
int samaya_solve_get_solution(double* col_value, int ncols, double* row_dual, int nrows,
                              int* verified);

#ifdef __cplusplus
}
#endif

#endif /* SAMAYA_C_PDLP_H */
