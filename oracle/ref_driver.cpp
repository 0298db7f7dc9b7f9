// Test-infrastructure only: a C entry layer over the reference solver's own CPU code, compiled
// from the reference checkout by oracle/Makefile.ref into oracle/_ref/. It is used to pin the
// oracle restatement (oracle/pdlp_oracle.c) and to generate the golden fixtures under
// tests/golden/. Nothing on the product path links or loads it.
//
// Entry points mirror the reference's own call sites:
//   ref_pdlp_solve      -> samaya::solve_pdlp              (src/lp/pdlp.cpp:228)
//   ref_scale_model     -> compute_scaling + make_problem  (src/linalg/scaling.cpp:130,
//                                                           src/lp/lp_solver.cpp:28)
//   ref_dual_simplex    -> samaya::solve_lp                (src/lp/lp_solver.cpp:66)
//   ref_verify_optimal  -> samaya::verify_lp_optimality    (src/verify/verify.cpp:251)
//   ref_random_lp       -> samaya::test::random_lp         (tests/lp_generators.hpp:32)
//   ref_reference_lp    -> samaya::test::ReferenceLp       (tests/reference_lp.hpp:20)
//   ref_solver_pdlp     -> Solver::solve with LpMethod::kPdlp (src/core/solver.cpp:705)
//   ref_mps_read        -> samaya::read_mps_from_string     (src/io/mps_reader.cpp:517)
//   ref_mps_read_file   -> samaya::read_mps                 (src/io/mps_reader.cpp:530)

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <random>
#include <string>
#include <string_view>
#include <vector>

#include "core/log.hpp"
#include "linalg/scaling.hpp"
#include "lp/lp_solver.hpp"
#include "lp/pdlp.hpp"
#include "lp_generators.hpp"
#include "reference_lp.hpp"
#include "samaya/io.hpp"
#include "samaya/model.hpp"
#include "samaya/solver.hpp"
#include "samaya/verify.hpp"

namespace {

samaya::SparseMatrix csc_from_arrays(int rows, int cols, const int64_t* colptr,
                                     const int32_t* rowidx, const double* vals) {
  std::vector<samaya::Triplet> t;
  t.reserve(static_cast<std::size_t>(colptr[cols]));
  for (int j = 0; j < cols; ++j) {
    for (int64_t p = colptr[j]; p < colptr[j + 1]; ++p) t.push_back({rowidx[p], j, vals[p]});
  }
  return samaya::SparseMatrix::from_triplets(rows, cols, std::move(t));
}

samaya::Model model_from_arrays(int m, int n, const int64_t* colptr, const int32_t* rowidx,
                                const double* vals, const double* obj, const double* col_lower,
                                const double* col_upper, const double* row_lower,
                                const double* row_upper, int maximize, double obj_offset) {
  samaya::Model model;
  model.sense = maximize ? samaya::ObjSense::kMaximize : samaya::ObjSense::kMinimize;
  model.obj_offset = obj_offset;
  model.obj.assign(obj, obj + n);
  model.col_lower.assign(col_lower, col_lower + n);
  model.col_upper.assign(col_upper, col_upper + n);
  model.col_type.assign(static_cast<std::size_t>(n), samaya::VarType::kContinuous);
  model.row_lower.assign(row_lower, row_lower + m);
  model.row_upper.assign(row_upper, row_upper + m);
  model.A = csc_from_arrays(m, n, colptr, rowidx, vals);
  return model;
}

void copy_csc(const samaya::SparseMatrix& a, int64_t* colptr, int32_t* rowidx, double* vals) {
  const auto s = a.col_start();
  const auto i = a.row_index();
  const auto v = a.values();
  for (std::size_t k = 0; k < s.size(); ++k) colptr[k] = s[k];
  for (std::size_t k = 0; k < i.size(); ++k) rowidx[k] = i[k];
  for (std::size_t k = 0; k < v.size(); ++k) vals[k] = v[k];
}

}  // namespace

extern "C" {

// Solves an LpProblem (computational form, A as CSC m x n) with the reference's solve_pdlp on
// the CPU. x has n+m entries, y m. Rays are written when the status carries one (flags set).
int ref_pdlp_solve(int m, int n, const int64_t* colptr, const int32_t* rowidx, const double* vals,
                   const double* cost, const double* lower, const double* upper, double tol,
                   long long max_iter, double time_limit, long long* iterations, double* res3,
                   double* x, double* y, double* dual_ray, double* primal_ray, int* ray_flags) {
  samaya::LpProblem lp;
  lp.m = m;
  lp.n = n;
  lp.A = csc_from_arrays(m, n, colptr, rowidx, vals);
  lp.At = lp.A.transpose();
  lp.cost.assign(cost, cost + n + m);
  lp.lower.assign(lower, lower + n + m);
  lp.upper.assign(upper, upper + n + m);
  samaya::PdlpOptions opts;
  opts.tol = tol;
  opts.max_iterations = max_iter;
  opts.time_limit = time_limit > 0 ? time_limit : samaya::kInf;
  opts.use_gpu = false;
  const samaya::PdlpResult r = samaya::solve_pdlp(lp, opts, samaya::Logger(0));
  *iterations = r.iterations;
  res3[0] = r.primal_residual;
  res3[1] = r.dual_residual;
  res3[2] = r.gap;
  for (std::size_t k = 0; k < r.x.size(); ++k) x[k] = r.x[k];
  for (std::size_t k = 0; k < r.y.size(); ++k) y[k] = r.y[k];
  ray_flags[0] = r.dual_ray.empty() ? 0 : 1;
  ray_flags[1] = r.primal_ray.empty() ? 0 : 1;
  for (std::size_t k = 0; k < r.dual_ray.size(); ++k) dual_ray[k] = r.dual_ray[k];
  for (std::size_t k = 0; k < r.primal_ray.size(); ++k) primal_ray[k] = r.primal_ray[k];
  return static_cast<int>(r.status);
}

// compute_scaling + make_problem on a model: writes the scaled computational-form problem (A as
// CSC, nnz_out entries; the caller sizes the arrays by the model's nnz) and the scale factors.
int ref_scale_model(int m, int n, const int64_t* colptr, const int32_t* rowidx, const double* vals,
                    const double* obj, const double* col_lower, const double* col_upper,
                    const double* row_lower, const double* row_upper, int maximize,
                    int64_t* out_colptr, int32_t* out_rowidx, double* out_vals, double* out_cost,
                    double* out_lower, double* out_upper, double* col_scale, double* row_scale,
                    int64_t* nnz_out) {
  const samaya::Model model = model_from_arrays(m, n, colptr, rowidx, vals, obj, col_lower,
                                                col_upper, row_lower, row_upper, maximize, 0.0);
  const samaya::Scaling s = samaya::compute_scaling(model.A);
  const samaya::LpProblem lp = samaya::make_problem(model, s);
  copy_csc(lp.A, out_colptr, out_rowidx, out_vals);
  *nnz_out = lp.A.nnz();
  for (int k = 0; k < n + m; ++k) {
    out_cost[k] = lp.cost[k];
    out_lower[k] = lp.lower[k];
    out_upper[k] = lp.upper[k];
  }
  for (int j = 0; j < n; ++j) col_scale[j] = s.col[j];
  for (int i = 0; i < m; ++i) row_scale[i] = s.row[i];
  return 0;
}

// The reference dual simplex on a model (x: n, y: m row duals with d = c - A'y).
int ref_dual_simplex(int m, int n, const int64_t* colptr, const int32_t* rowidx,
                     const double* vals, const double* obj, const double* col_lower,
                     const double* col_upper, const double* row_lower, const double* row_upper,
                     int maximize, double time_limit, double* objective, double* x, double* y,
                     long long* iterations) {
  const samaya::Model model = model_from_arrays(m, n, colptr, rowidx, vals, obj, col_lower,
                                                col_upper, row_lower, row_upper, maximize, 0.0);
  samaya::LpSolveOptions opts;
  if (time_limit > 0) opts.simplex.time_limit = time_limit;
  const samaya::LpResult r = samaya::solve_lp(model, opts, samaya::Logger(0));
  *objective = r.objective;
  *iterations = r.iterations;
  for (std::size_t k = 0; k < r.col_value.size(); ++k) x[k] = r.col_value[k];
  for (std::size_t k = 0; k < r.row_dual.size(); ++k) y[k] = r.row_dual[k];
  return static_cast<int>(r.status);
}

// verify_lp_optimality at the given relative tolerances; returns 1 when the point verifies.
int ref_verify_optimal(int m, int n, const int64_t* colptr, const int32_t* rowidx,
                       const double* vals, const double* obj, const double* col_lower,
                       const double* col_upper, const double* row_lower, const double* row_upper,
                       int maximize, const double* x, const double* y, double tol,
                       double* objective) {
  const samaya::Model model = model_from_arrays(m, n, colptr, rowidx, vals, obj, col_lower,
                                                col_upper, row_lower, row_upper, maximize, 0.0);
  samaya::VerifyTolerances t;
  t.primal = tol;
  t.dual = tol;
  const samaya::VerifyReport r = samaya::verify_lp_optimality(
      model, std::span<const double>(x, n), std::span<const double>(y, m), t);
  *objective = r.objective;
  return r.ok ? 1 : 0;
}

// The reference test generator: draws `prefix_count` models of `prefix_family`, then `index + 1`
// models of `family` from a fresh std::mt19937(seed), and returns the last one. First call with nnz_cap = 0 to get sizes (dims[0..2] = m, n, nnz).
int ref_random_lp(int family, int max_rows, int max_cols, unsigned seed, int index,
                  int prefix_family, int prefix_count, int* dims,
                  int64_t* colptr, int32_t* rowidx, double* vals, double* obj, double* col_lower,
                  double* col_upper, double* row_lower, double* row_upper, int* maximize,
                  double* obj_offset) {
  std::mt19937 rng(seed);
  samaya::Model model;
  for (int k = 0; k < prefix_count; ++k) {
    model = samaya::test::random_lp(static_cast<samaya::test::LpFamily>(prefix_family), max_rows,
                                    max_cols, rng);
  }
  for (int k = 0; k <= index; ++k) {
    model = samaya::test::random_lp(static_cast<samaya::test::LpFamily>(family), max_rows,
                                    max_cols, rng);
  }
  const int m = model.num_rows();
  const int n = model.num_cols();
  dims[0] = m;
  dims[1] = n;
  dims[2] = static_cast<int>(model.A.nnz());
  if (colptr == nullptr) return 0;
  copy_csc(model.A, colptr, rowidx, vals);
  for (int j = 0; j < n; ++j) {
    obj[j] = model.obj[j];
    col_lower[j] = model.col_lower[j];
    col_upper[j] = model.col_upper[j];
  }
  for (int i = 0; i < m; ++i) {
    row_lower[i] = model.row_lower[i];
    row_upper[i] = model.row_upper[i];
  }
  *maximize = model.sense == samaya::ObjSense::kMaximize ? 1 : 0;
  *obj_offset = model.obj_offset;
  return 0;
}

// The reference's dense long-double tableau simplex: 0 optimal, 1 infeasible, 2 unbounded.
int ref_reference_lp(int m, int n, const int64_t* colptr, const int32_t* rowidx,
                     const double* vals, const double* obj, const double* col_lower,
                     const double* col_upper, const double* row_lower, const double* row_upper,
                     int maximize, double obj_offset, double* objective) {
  const samaya::Model model = model_from_arrays(m, n, colptr, rowidx, vals, obj, col_lower,
                                                col_upper, row_lower, row_upper, maximize,
                                                obj_offset);
  const samaya::test::ReferenceResult r = samaya::test::ReferenceLp(model).solve();
  *objective = r.objective;
  return static_cast<int>(r.status);
}

// Solver::solve with --lp-method pdlp (no presolve), as tests/test_pdlp.cpp:497-540 calls it.
int ref_solver_pdlp(int m, int n, const int64_t* colptr, const int32_t* rowidx,
                    const double* vals, const double* obj, const double* col_lower,
                    const double* col_upper, const double* row_lower, const double* row_upper,
                    int maximize, double obj_offset, double* objective, int* verified,
                    long long* simplex_iterations, long long* pdlp_iterations) {
  const samaya::Model model = model_from_arrays(m, n, colptr, rowidx, vals, obj, col_lower,
                                                col_upper, row_lower, row_upper, maximize,
                                                obj_offset);
  samaya::Params params;
  params.log_level = 0;
  params.presolve = false;
  params.lp_method = samaya::LpMethod::kPdlp;
  const samaya::Result r = samaya::Solver(params).solve(model);
  *objective = r.objective;
  *verified = r.verified ? 1 : 0;
  *simplex_iterations = r.simplex_iterations;
  *pdlp_iterations = r.barrier_iterations;
  return static_cast<int>(r.status);
}

// ---- MPS: a model read by samaya's own reader, held until ref_mps_free ----

struct RefMps {
  samaya::Model model;
  double seconds = 0.0;
};

static int ref_mps_finish(RefMps* r, void** out, char* err, size_t errlen, int code,
                          const char* what) {
  if (code == 0) {
    *out = r;
    return 0;
  }
  delete r;
  if (err != nullptr && errlen > 0) {
    std::strncpy(err, what, errlen - 1);
    err[errlen - 1] = '\0';
  }
  return code;
}

// 0: read; 1: samaya::ParseError (message in err); 2: another exception.
int ref_mps_read(const char* text, size_t len, void** out, char* err, size_t errlen) {
  RefMps* r = new RefMps;
  try {
    const auto t0 = std::chrono::steady_clock::now();
    r->model = samaya::read_mps_from_string(std::string_view(text, len));
    r->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return ref_mps_finish(r, out, err, errlen, 0, "");
  } catch (const samaya::ParseError& e) {
    return ref_mps_finish(r, out, err, errlen, 1, e.what());
  } catch (const std::exception& e) {
    return ref_mps_finish(r, out, err, errlen, 2, e.what());
  }
}

int ref_mps_read_file(const char* path, void** out, char* err, size_t errlen) {
  RefMps* r = new RefMps;
  try {
    const auto t0 = std::chrono::steady_clock::now();
    r->model = samaya::read_mps(path);
    r->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return ref_mps_finish(r, out, err, errlen, 0, "");
  } catch (const samaya::ParseError& e) {
    return ref_mps_finish(r, out, err, errlen, 1, e.what());
  } catch (const std::exception& e) {
    return ref_mps_finish(r, out, err, errlen, 2, e.what());
  }
}

// info: m, n, nnz, maximize, integers, name bytes, row name bytes, column name bytes, Q entries,
// quadratic row terms; *obj_offset; *seconds (the read's wall time).
void ref_mps_info(void* h, int64_t* info, double* obj_offset, double* seconds) {
  const RefMps& r = *static_cast<RefMps*>(h);
  const samaya::Model& md = r.model;
  int64_t rn = 0, cn = 0;
  for (const auto& s : md.row_names) rn += static_cast<int64_t>(s.size());
  for (const auto& s : md.col_names) cn += static_cast<int64_t>(s.size());
  info[0] = md.num_rows();
  info[1] = md.num_cols();
  info[2] = md.A.nnz();
  info[3] = md.sense == samaya::ObjSense::kMaximize ? 1 : 0;
  info[4] = md.num_integers();
  info[5] = static_cast<int64_t>(md.name.size());
  info[6] = rn;
  info[7] = cn;
  info[8] = md.Q.nnz();
  info[9] = static_cast<int64_t>(md.row_quadratic.size());
  *obj_offset = md.obj_offset;
  *seconds = r.seconds;
}

void ref_mps_get(void* h, int64_t* colptr, int32_t* rowidx, double* vals, double* obj,
                 double* col_lower, double* col_upper, uint8_t* col_integer, double* row_lower,
                 double* row_upper) {
  const samaya::Model& md = static_cast<RefMps*>(h)->model;
  copy_csc(md.A, colptr, rowidx, vals);
  const std::size_t n = md.obj.size(), m = md.row_lower.size();
  for (std::size_t j = 0; j < n; ++j) {
    obj[j] = md.obj[j];
    col_lower[j] = md.col_lower[j];
    col_upper[j] = md.col_upper[j];
    col_integer[j] = md.col_type[j] == samaya::VarType::kInteger ? 1 : 0;
  }
  for (std::size_t i = 0; i < m; ++i) {
    row_lower[i] = md.row_lower[i];
    row_upper[i] = md.row_upper[i];
  }
}

void ref_mps_names(void* h, char* name, char* row_names, int64_t* row_starts, char* col_names,
                   int64_t* col_starts) {
  const samaya::Model& md = static_cast<RefMps*>(h)->model;
  std::memcpy(name, md.name.data(), md.name.size());
  int64_t p = 0;
  row_starts[0] = 0;
  for (std::size_t i = 0; i < md.row_names.size(); ++i) {
    std::memcpy(row_names + p, md.row_names[i].data(), md.row_names[i].size());
    p += static_cast<int64_t>(md.row_names[i].size());
    row_starts[i + 1] = p;
  }
  p = 0;
  col_starts[0] = 0;
  for (std::size_t j = 0; j < md.col_names.size(); ++j) {
    std::memcpy(col_names + p, md.col_names[j].data(), md.col_names[j].size());
    p += static_cast<int64_t>(md.col_names[j].size());
    col_starts[j + 1] = p;
  }
}

void ref_mps_free(void* h) { delete static_cast<RefMps*>(h); }

}  // extern "C"
