"""samaya_gb300 — a GB300-native PDLP engine for samaya's LP solver.

The engine (CUDA for sm_103a behind the C ABI in include/sg_pdlp.h) replaces the reference's
PDLP path: ``samaya::solve_pdlp`` (src/lp/pdlp.cpp) and its GPU back end (src/gpu/); the fast
MPS reader (include/sg_mps.h) replaces ``samaya::read_mps`` (src/io/mps_reader.cpp) for the free
MPS files of linear models that the path starts from.
"""
from .model import LpProblem, Model  # noqa: F401
from .mps import MpsFile, MpsReadError, read_mps, read_mps_text, write_mps  # noqa: F401
from .pdlp import (ENHANCED, FP32_REFINED, FP32_THEN_FP64, FP64, HALPERN, REFERENCE,  # noqa: F401
                   INFEASIBLE,
                   ITERATION_LIMIT, NUMERICAL_ERROR,
                   OPTIMAL, STATUS_NAMES, TIME_LIMIT, UNBOUNDED, PdhgDevice, PdlpOptions,
                   PdlpResult, PdlpSolver, gpu_info, solve_pdlp)

__version__ = "0.1.0"
