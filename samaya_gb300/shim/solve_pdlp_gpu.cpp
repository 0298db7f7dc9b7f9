// The use_gpu branch of samaya::solve_pdlp on the GB300 engine (see solve_pdlp_gpu.hpp).
#include "solve_pdlp_gpu.hpp"

#include <atomic>
#include <utility>
#include <vector>

namespace samaya_gb300 {

namespace {

std::atomic<long long> g_engine{0};
std::atomic<long long> g_cpu{0};

samaya::PdlpResult on_cpu(const samaya::LpProblem& lp, const samaya::PdlpOptions& options,
                          const samaya::Logger& log, CpuPdlp cpu) {
  ++g_cpu;
  samaya::PdlpOptions o = options;
  o.use_gpu = false;
  return cpu(lp, o, log);
}

}  // namespace

ShimCounts shim_counts() { return ShimCounts{g_engine.load(), g_cpu.load()}; }

samaya::PdlpResult solve_pdlp(const samaya::LpProblem& lp, const samaya::PdlpOptions& options,
                              const samaya::Logger& log, CpuPdlp cpu,
                              const sg_pdlp_opts* engine_opts) {
  if (!options.use_gpu || sg_pdlp_available(nullptr, nullptr, nullptr, 0) != SG_OK) {
    return on_cpu(lp, options, log, cpu);
  }
  sg_pdlp_opts o;
  if (engine_opts != nullptr) {
    o = *engine_opts;
  } else {
    sg_pdlp_default_opts(&o);
  }
  o.tol = options.tol;
  o.max_iterations = options.max_iterations;
  o.time_limit = options.time_limit < samaya::kInf ? options.time_limit : 0.0;
  const auto start = lp.A.col_start();  // int64 column starts, int32 rows, float64 values
  sg_pdlp* h = nullptr;
  int rc = sg_pdlp_create(&h, lp.m, lp.n, start.data(), lp.A.row_index().data(),
                          lp.A.values().data(), lp.cost.data(), lp.lower.data(), lp.upper.data(),
                          &o);
  if (rc == SG_OK) {
    samaya::PdlpResult r;
    r.x.resize(static_cast<size_t>(lp.n) + lp.m);
    r.y.resize(static_cast<size_t>(lp.m));
    std::vector<double> dual_ray(static_cast<size_t>(lp.m)), primal_ray(static_cast<size_t>(lp.n));
    sg_pdlp_result res;
    rc = sg_pdlp_solve(h, &res, r.x.data(), r.y.data(), dual_ray.data(), primal_ray.data());
    sg_pdlp_destroy(h);
    if (rc == SG_OK) {
      ++g_engine;
      r.status = static_cast<samaya::SimplexStatus>(res.status);
      r.iterations = res.iterations;
      r.primal_residual = res.primal_residual;
      r.dual_residual = res.dual_residual;
      r.gap = res.gap;
      if (res.has_dual_ray) r.dual_ray = std::move(dual_ray);
      if (res.has_primal_ray) r.primal_ray = std::move(primal_ray);
      r.stats.dual_iterations = r.iterations;
      return r;
    }
  }
  log.log(1, "pdlp: GPU engine unavailable (%s); solving on the CPU", sg_pdlp_last_error());
  return on_cpu(lp, options, log, cpu);
}

}  // namespace samaya_gb300
