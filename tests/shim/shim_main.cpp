// Test driver of the samaya integration (CPU test, built only where the samaya checkout and
// its compiled library exist): samaya's own Solver and C API, with solve_pdlp routed through the
// GB300 binding (samaya_gb300/shim/solve_pdlp_gpu.cpp).
//
// The maintainer's change to samaya is one line in src/lp/pdlp.cpp: solve_pdlp's body becomes a
// call of samaya_gb300::solve_pdlp with samaya's own CPU routine as the fallback. Here samaya is
// a prebuilt library, so the same routing is made by defining samaya::solve_pdlp in this
// executable (its definition takes precedence over the library's for the library's own calls)
// and reaching the library's CPU routine with dlsym(RTLD_NEXT).
//
//   shim_main <model.mps> <lp_method> <use_gpu> <tol> [<solution.bin>]
// prints one line: status objective verified engine_solves cpu_solves; with a path, writes the
// column values then the row duals (float64) there.
//
//   shim_main --crossover <model.mps> [dual]
// runs samaya's Solver with lp_method PDLP, use_gpu, crossover and no presolve (the PDLP point
// seeds the crossover basis and the simplex finishes from it, src/core/solver.cpp:451-461,
// 541-571) and prints: status objective simplex_iterations crossover verified engine_solves
// cpu_solves replayed_solves. With SG_SHIM_REPLAY=<file>, solve_pdlp returns the PDLP answer
// stored in that file (int64 n, int64 m, int32 status, int64 iterations, float64 x[n + m],
// float64 y[m]: an answer the GB300 engine computed for the same LpProblem on a GPU machine) in
// place of a solve, so that samaya's crossover can be measured from the engine's point on a
// machine without a GPU. With `dual`: the dual simplex from its own start instead (no PDLP, no
// crossover), the work the crossover saves.
//
//   shim_main --read <model.mps>
// reads the file with the fast reader's binding (samaya_gb300/shim/read_mps_fast.cpp) and with
// samaya::read_mps, compares every field of the two Models bit for bit and prints: same
// fast_reads samaya_reads binding_seconds samaya_seconds.
//
//   shim_main --cli <model.mps> <tol>
// the CLI's `--lp-method pdlp --gpu` chain with the fast reader: the model read by the binding,
// then samaya's Solver with lp_method PDLP and use_gpu (solve_pdlp routed through the engine's
// binding, as above); and the same with samaya::read_mps. Prints: same_bits status objective
// verified fast_reads engine_solves cpu_solves.
#include <dlfcn.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <vector>

#include "samaya/io.hpp"
#include "samaya/solver.hpp"
#include "read_mps_fast.hpp"
#include "samaya_c_pdlp.h"
#include "solve_pdlp_gpu.hpp"

namespace {

samaya_gb300::CpuPdlp library_solve_pdlp() {
  static samaya_gb300::CpuPdlp f = reinterpret_cast<samaya_gb300::CpuPdlp>(dlsym(
      RTLD_NEXT, "_ZN6samaya10solve_pdlpERKNS_9LpProblemERKNS_11PdlpOptionsERKNS_6LoggerE"));
  return f;
}

long long g_replayed = 0;

// The stored answer for an LpProblem of these sizes, if SG_SHIM_REPLAY names one.
bool replay(const samaya::LpProblem& lp, samaya::PdlpResult* out) {
  const char* path = std::getenv("SG_SHIM_REPLAY");
  if (path == nullptr || *path == '\0') return false;
  FILE* f = std::fopen(path, "rb");
  if (f == nullptr) return false;
  int64_t n = 0, m = 0, iterations = 0;
  int32_t status = 0;
  bool ok = std::fread(&n, sizeof(n), 1, f) == 1 && std::fread(&m, sizeof(m), 1, f) == 1 &&
            std::fread(&status, sizeof(status), 1, f) == 1 &&
            std::fread(&iterations, sizeof(iterations), 1, f) == 1 && n == lp.n && m == lp.m;
  if (ok) {
    out->x.resize(static_cast<size_t>(n + m));
    out->y.resize(static_cast<size_t>(m));
    ok = std::fread(out->x.data(), sizeof(double), out->x.size(), f) == out->x.size() &&
         std::fread(out->y.data(), sizeof(double), out->y.size(), f) == out->y.size();
    out->status = static_cast<samaya::SimplexStatus>(status);
    out->iterations = iterations;
  }
  std::fclose(f);
  return ok;
}

int crossover_mode(const char* mps, bool dual_simplex) {
  samaya::Params params;
  params.log_level = 0;
  params.lp_method = dual_simplex ? samaya::LpMethod::kDualSimplex : samaya::LpMethod::kPdlp;
  params.use_gpu = true;
  params.crossover = !dual_simplex;
  params.presolve = false;
  const samaya::Model model = samaya::read_mps(mps);
  const samaya::Result r = samaya::Solver(params).solve(model);
  const samaya_gb300::ShimCounts c = samaya_gb300::shim_counts();
  std::printf("%d %.17g %lld %d %d %lld %lld %lld\n", static_cast<int>(r.status), r.objective,
              r.simplex_iterations, r.crossover ? 1 : 0, r.verified ? 1 : 0, c.engine, c.cpu,
              g_replayed);
  return 0;
}

template <class T>
bool same_bits(const std::vector<T>& a, const std::vector<T>& b) {
  return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}

template <class S>
bool same_span(S a, S b) {
  return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size_bytes()) == 0);
}

bool same_matrix(const samaya::SparseMatrix& a, const samaya::SparseMatrix& b) {
  return a.rows() == b.rows() && a.cols() == b.cols() && same_span(a.col_start(), b.col_start()) &&
         same_span(a.row_index(), b.row_index()) && same_span(a.values(), b.values());
}

bool same_model(const samaya::Model& a, const samaya::Model& b) {
  bool q = a.row_quadratic.size() == b.row_quadratic.size();
  for (size_t k = 0; q && k < a.row_quadratic.size(); ++k) {
    const auto &x = a.row_quadratic[k], &y = b.row_quadratic[k];
    q = x.row == y.row && x.col1 == y.col1 && x.col2 == y.col2 &&
        std::memcmp(&x.value, &y.value, sizeof(double)) == 0;
  }
  return q && a.name == b.name && a.sense == b.sense &&
         std::memcmp(&a.obj_offset, &b.obj_offset, sizeof(double)) == 0 && same_bits(a.obj, b.obj) &&
         same_bits(a.col_lower, b.col_lower) && same_bits(a.col_upper, b.col_upper) &&
         a.col_type == b.col_type && a.col_names == b.col_names &&
         same_bits(a.row_lower, b.row_lower) && same_bits(a.row_upper, b.row_upper) &&
         a.row_names == b.row_names && same_matrix(a.A, b.A) && same_matrix(a.Q, b.Q);
}

int read_mode(const char* path) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  const samaya::Model fast = samaya_gb300::read_mps(path);
  const auto t1 = clock::now();
  const samaya::Model own = samaya::read_mps(path);
  const auto t2 = clock::now();
  const samaya_gb300::ReadCounts c = samaya_gb300::read_counts();
  std::printf("%d %lld %lld %.6f %.6f\n", same_model(fast, own) ? 1 : 0, c.fast, c.samaya,
              std::chrono::duration<double>(t1 - t0).count(),
              std::chrono::duration<double>(t2 - t1).count());
  return 0;
}

int cli_mode(const char* path, double tol) {
  samaya::Params params;
  params.log_level = 0;
  params.lp_method = samaya::LpMethod::kPdlp;
  params.use_gpu = true;
  params.primal_feasibility_tol = tol;
  params.dual_feasibility_tol = tol;
  const samaya::Result a = samaya::Solver(params).solve(samaya_gb300::read_mps(path));
  const samaya::Result b = samaya::Solver(params).solve(samaya::read_mps(path));
  const bool same = a.status == b.status && same_bits(a.col_value, b.col_value) &&
                    same_bits(a.row_dual, b.row_dual) &&
                    std::memcmp(&a.objective, &b.objective, sizeof(double)) == 0;
  const samaya_gb300::ShimCounts c = samaya_gb300::shim_counts();
  std::printf("%d %d %.17g %d %lld %lld %lld\n", same ? 1 : 0, static_cast<int>(a.status),
              a.objective, a.verified ? 1 : 0, samaya_gb300::read_counts().fast, c.engine,
              c.cpu);
  return 0;
}

}  // namespace

namespace samaya {

PdlpResult solve_pdlp(const LpProblem& lp, const PdlpOptions& options, const Logger& log) {
  PdlpResult stored;
  if (replay(lp, &stored)) {
    ++g_replayed;
    return stored;
  }
  return samaya_gb300::solve_pdlp(lp, options, log, library_solve_pdlp());
}

}  // namespace samaya

int main(int argc, char** argv) {
  if (argc == 4 && std::strcmp(argv[1], "--cli") == 0) {
    if (library_solve_pdlp() == nullptr) return 2;
    try {
      return cli_mode(argv[2], std::atof(argv[3]));
    } catch (const std::exception& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return 3;
    }
  }
  if (argc == 3 && std::strcmp(argv[1], "--read") == 0) {
    try {
      return read_mode(argv[2]);
    } catch (const std::exception& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return 3;
    }
  }
  if ((argc == 3 || argc == 4) && std::strcmp(argv[1], "--crossover") == 0) {
    if (library_solve_pdlp() == nullptr) return 2;
    try {
      return crossover_mode(argv[2], argc == 4 && std::strcmp(argv[3], "dual") == 0);
    } catch (const std::exception& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return 2;
    }
  }
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s model.mps lp_method use_gpu tol [solution.bin]\n", argv[0]);
    return 2;
  }
  if (library_solve_pdlp() == nullptr) {
    std::fprintf(stderr, "samaya's solve_pdlp not found\n");
    return 2;
  }
  samaya_model* model = nullptr;
  char err[256];
  if (samaya_read_mps(argv[1], &model, err, sizeof(err)) != 0) {
    std::fprintf(stderr, "read: %s\n", err);
    return 2;
  }
  double objective = 0.0;
  const int status = samaya_solve_params(model, std::atoi(argv[2]), std::atoi(argv[3]), 0.0,
                                         std::atof(argv[4]), &objective);
  const int n = samaya_model_num_cols(model);
  const int m = samaya_model_num_rows(model);
  std::vector<double> x(static_cast<size_t>(n)), y(static_cast<size_t>(m));
  int verified = 0;
  const int got = samaya_solve_get_solution(x.data(), n, y.data(), m, &verified);
  const samaya_gb300::ShimCounts c = samaya_gb300::shim_counts();
  std::printf("%d %.17g %d %lld %lld\n", status, objective, got == 0 ? verified : -1, c.engine,
              c.cpu);
  if (argc > 5 && got == 0) {
    FILE* f = std::fopen(argv[5], "wb");
    if (f == nullptr) return 2;
    std::fwrite(x.data(), sizeof(double), x.size(), f);
    std::fwrite(y.data(), sizeof(double), y.size(), f);
    std::fclose(f);
  }
  samaya_model_free(model);
  return 0;
}
