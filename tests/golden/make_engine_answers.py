"""Answers of the GB300 engine for the crossover-seeding measurement (needs a GB300).

For each LP below, solves its LpProblem (compute_scaling + make_problem, the same problem
samaya's solve_pdlp_lp builds without presolve) with the engine to 1e-8 — in the bench's mode
(FP32 then FP64, Halpern), or where that stops at its iteration limit, FP64 Halpern, then FP64
with the reference algorithm — and stores the answer in the LpProblem's space:
tests/golden/engine_answers.npz: <name>_x (n + m), <name>_y (m), <name>_meta (status,
iterations, mode: 0 FP32 then FP64 Halpern, 1 FP64 Halpern, 2 FP64 reference). tests/test_shim.py replays these answers into samaya's own Solver (crossover on) on
a machine with the samaya checkout and measures the simplex work left after the crossover.
Run from the repository root on a GPU machine:

    python tests/golden/make_engine_answers.py [output.npz]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.join(ROOT, "tests", "golden", "engine_answers.npz")


def crossover_lps():
    """(name, Model) of the crossover-seeding measurement: degenerate LPs where a vertex is
    far from a first-order method's point (transportation, facility location), a power-law LP
    and a random sparse LP."""
    from samaya_gb300 import generators as g
    return [("transport100x200", g.transportation_lp(100, 200, seed=1)),
            ("facility50x200", g.facility_location_lp(50, 200, seed=1)),
            ("powerlaw5k", g.power_law_lp(m=5000, n=10000, seed=1)),
            ("random500", g.random_sparse_lp(500, 1200, seed=0))]


def main(out_path=OUT):
    import samaya_gb300 as sg
    from samaya_gb300.problem import make_problem
    out = {}
    modes = [dict(precision=sg.FP32_THEN_FP64, algorithm=sg.HALPERN, inner_tol=1e-6),
             dict(precision=sg.FP64, algorithm=sg.HALPERN),
             dict(precision=sg.FP64, algorithm=sg.REFERENCE)]
    for name, model in crossover_lps():
        lp, _ = make_problem(model)
        for mode, kw in enumerate(modes):
            r = sg.solve_pdlp(lp, sg.PdlpOptions(tol=1e-8, **kw))
            print(name, mode, r.status_name, r.iterations, flush=True)
            if r.status == sg.OPTIMAL:
                break
        out[f"{name}_x"] = r.x
        out[f"{name}_y"] = r.y
        out[f"{name}_meta"] = np.array([r.status, r.iterations, mode], dtype=np.int64)
    np.savez_compressed(out_path, **out)


if __name__ == "__main__":
    main(*sys.argv[1:2])
