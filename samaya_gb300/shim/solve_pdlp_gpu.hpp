// The binding a samaya maintainer adds to src/lp/pdlp.cpp: the use_gpu branch of
// samaya::solve_pdlp (reference src/lp/pdlp.hpp:35, src/lp/pdlp.cpp:228-246) on the GB300
// engine's C ABI (include/sg_pdlp.h). It compiles against samaya's own headers (include/ and
// src/ of the samaya tree) and is not part of libsamaya_gb300.so.
#pragma once

#include "lp/pdlp.hpp"
#include "sg_pdlp.h"

namespace samaya_gb300 {

// samaya's own PDLP (its CPU path), called when the engine is absent or fails: the engine has
// no CPU fallback inside; the fallback lives here, in the caller, as the reference keeps its
// own (pdlp.cpp:228-246).
using CpuPdlp = samaya::PdlpResult (*)(const samaya::LpProblem&, const samaya::PdlpOptions&,
                                       const samaya::Logger&);

// Solves an LpProblem as samaya::solve_pdlp does. With options.use_gpu and a usable GB300 the
// engine answers (engine_opts, when non-null, carries the engine's own knobs: precision,
// algorithm); otherwise, or when the engine reports an error, `cpu` does.
samaya::PdlpResult solve_pdlp(const samaya::LpProblem& lp, const samaya::PdlpOptions& options,
                              const samaya::Logger& log, CpuPdlp cpu,
                              const sg_pdlp_opts* engine_opts = nullptr);

// How many solves of this process the engine answered and how many went to `cpu`.
struct ShimCounts {
  long long engine = 0;
  long long cpu = 0;
};
ShimCounts shim_counts();

}  // namespace samaya_gb300
