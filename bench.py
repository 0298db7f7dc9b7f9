#!/usr/bin/env python3
"""Benchmark of the GB300 PDLP engine: time to 1e-8 relative KKT on the transportation LP
(1000 supplies x 2000 demands: 3000 equality rows, 2,000,000 columns, 4,000,000 nonzeros) with
mixed precision (FP32 PDLP to a switch tolerance, then FP64 PDLP from its answer: the headline),
next to FP32 + FP64 iterative refinement and plain FP64 on the same GPU.

One step = one full PDLP solve of the LP, inputs resident in HBM (the problem uploaded once);
``e2e`` = the same solve through the public C ABI from pinned host buffers (upload, solve,
download of x and y). ``roofline`` reports the dominant step kernel (both launch once per
iteration; the slower one) against the measured HBM copy bandwidth; ``cpu_baseline`` times the
reference's CPU PDLP (the oracle port, 1 core) on a bounded run of the same LP.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --workload powerlaw|random|batchA|batchB|diff   (the other configurations)
    python bench.py --workload mps      (the MPS reader on the transportation LP's 93 MB file)

With N > 1 (torchrun) every rank solves its own replica (replicas only; no collective on the
data path); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PDLP time-to-1e-8 KKT (mixed vs FP64 GPU)"
TOL = 1e-8
CPU_CAP_S = 20.0
# The FP32 phase's tolerance: the latest switch that still leaves FP32 progressing on the
# transportation LP (seeds 0-3: 97-110 ms at 3e-7 against 116-128 ms at 1e-6; at 1e-7 the FP32
# phase reaches its precision floor and the stall test ends it late, 286 ms).
SWITCH_TOL = 3e-7
ALGORITHM_NAMES = {
    "enhanced": "enhanced (inf-norm Ruiz + Pock-Chambolle, primal weight |c|/|b|)",
    "halpern": "halpern (enhanced scaling, reflected Halpern PDHG)",
    "reference": "reference (samaya's L2 Ruiz, primal weight 1)",
}
ALGORITHM_IDS = {"reference": 0, "enhanced": 1, "halpern": 2}
PRECISION_NAMES = {
    "mixed": "fp32 PDLP to the switch tolerance, then fp64 PDLP from its answer",
    "refined": "fp32 storage + fp64 iterative refinement",
    "fp64": "fp64",
}


def solver_options(args, precision, time_limit=None):
    """PdlpOptions of a precision mode with the chosen algorithm (time_limit: seconds, None for
    none)."""
    import samaya_gb300 as sg
    prec = {"mixed": sg.FP32_THEN_FP64, "refined": sg.FP32_REFINED, "fp64": sg.FP64}[precision]
    kw = {"inner_tol": args.switch_tol} if precision == "mixed" else {}
    if time_limit is not None:
        kw["time_limit"] = time_limit
    alg = ALGORITHM_IDS[getattr(args, "algorithm", "enhanced")]
    return sg.PdlpOptions(tol=TOL, algorithm=alg, precision=prec,
                          max_iterations=getattr(args, "max_iterations", -1) if args.profile
                          else -1, **kw)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="transport",
                    choices=["transport", "powerlaw", "random", "batchA", "batchB", "diff", "mps"],
                    help="transport (the headline), powerlaw, random (2000 x 5000): one LP to "
                         "1e-8; batchA / batchB: LPs/s of the batched engine against sequential "
                         "solves; diff: the differentiable layer's forward and backward; mps: "
                         "the fast MPS reader on the transportation LP's file")
    ap.add_argument("--mps-lp", default="transport", choices=["transport", "powerlaw"],
                    help="--workload mps: the LP written to the file (transport: 93 MB; "
                         "powerlaw: the 1M x 2M power-law LP, 515 MB)")
    ap.add_argument("--precision", default="auto",
                    choices=["auto", "mixed", "refined", "fp64"],
                    help="mixed: FP32 PDLP then FP64 PDLP from its answer; refined: FP32 "
                         "iterations with FP64 iterative refinement; fp64: FP64 throughout; "
                         "auto: fp64 on the power-law LP (FP32 storage of its iterate leaves a "
                         "1e-5 relative residual floor there), mixed otherwise")
    ap.add_argument("--other-time-limit", type=float, default=150.0,
                    help="seconds each comparison solve (the other precisions, the largest "
                         "configuration's modes) may take before it stops with status "
                         "time_limit")
    ap.add_argument("--no-largest", action="store_true",
                    help="skip the power-law LP (the largest configuration) measurement that "
                         "the transportation line carries")
    ap.add_argument("--switch-tol", type=float, default=SWITCH_TOL,
                    help="relative KKT at which the mixed path leaves FP32")
    ap.add_argument("--profile", action="store_true",
                    help="one solve of the workload and nothing else (for profilers)")
    ap.add_argument("--max-iterations", type=int, default=-1,
                    help="iteration cap of the --profile solve (-1: none)")
    ap.add_argument("--tol", type=float, default=1e-8,
                    help="relative KKT tolerance of the single-LP workloads")
    ap.add_argument("--algorithm", default="auto",
                    choices=["auto", "enhanced", "halpern", "reference"],
                    help="enhanced: inf-norm Ruiz + Pock-Chambolle, primal weight |c|/|b|; "
                         "halpern: enhanced with the reflected Halpern iteration; "
                         "reference: samaya's PDLP step for step; auto: the faster one for "
                         "the workload (halpern on the transportation LP, reference on the "
                         "random sparse LPs, enhanced otherwise)")
    args = ap.parse_args()
    if args.algorithm == "auto":
        args.algorithm = {"transport": "halpern", "random": "reference", "powerlaw": "halpern",
                          "batchA": "reference", "mps": "halpern"}.get(args.workload,
                                                                     "enhanced")
    if args.precision == "auto":
        args.precision = "fp64" if args.workload == "powerlaw" else "mixed"
    global TOL
    TOL = args.tol
    return args


def run_profile(args):
    """One solve of the workload (no baselines, no JSON): the command profilers wrap."""
    import samaya_gb300 as sg
    from samaya_gb300.problem import make_problem
    model, cfg = workload(args.workload)
    lp, _ = make_problem(model)
    r = sg.solve_pdlp(lp, solver_options(args, args.precision))
    print(f"{cfg['workload']}: {r.status_name} {r.iterations} iterations "
          f"{r.device_ms:.1f} ms", flush=True)
    return 0


def workload(name, seed=0):
    from samaya_gb300 import generators as g
    if name == "transport":
        return g.transportation_lp(1000, 2000, seed=seed), {
            "workload": "transportation LP 1000 supplies x 2000 demands", "rows": 3000,
            "columns": 2_000_000, "nnz": 4_000_000, "seed": seed}
    if name == "powerlaw":
        return g.power_law_lp(seed=seed), {
            "workload": "power-law LP 1e6 x 2e6, Zipf(1.5) rows", "rows": 1_000_000,
            "columns": 2_000_000, "nnz": 12_000_000, "seed": seed}
    return g.random_sparse_lp(2000, 5000, seed=seed), {
        "workload": "random sparse LP 2000 x 5000", "rows": 2000, "columns": 5000,
        "nnz": 30000, "seed": seed}


def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """nvidia-smi samples of the SM clock and throttle reasons during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([s.strip() for s in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.thread is not None:
                self.thread.join(timeout=2)

    def summary(self):
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                mhz.append(float(s[0]))
                mx = float(s[1])
                for k, name in enumerate(names):
                    if s[3 + k].lower().startswith("active"):
                        reasons.add(name)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(mhz)}


def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_summary():
    path = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def primal_step_bytes(lp, value_bytes, halpern=False):
    """Compulsory bytes of one primal-step launch (rows of A' = the n columns): the nonzeros
    (value + int32 index), the n + 1 row starts, the duals of the rows with nonzeros gathered
    once, and the column epilogue: classic, 8 n-vectors (c, l, u, x, x_avg read; x_new, x_bar,
    x_avg written); Halpern, 7 (c, l, u, x, x0 read; x_new, x_bar written; x^ is written only by
    a chunk's last step, before an evaluation). When every column has the same bounds, each 0
    or infinite (the transportation LP: x >= 0), the engine reads no bound vectors: 2 fewer;
    when every column has the same number of nonzeros (two in the transportation LP), no row
    starts."""
    import numpy as np
    n, nnz = lp.n, lp.nnz
    m = int(np.count_nonzero(np.bincount(lp.rowidx[:nnz], minlength=lp.m)))
    lens = np.diff(lp.colptr)
    starts = 0 if n > 0 and np.all(lens == lens[0]) and lens[0] > 0 else (n + 1) * 4
    vecs = 7 if halpern else 8
    lo, up = lp.lower[:n], lp.upper[:n]
    if n > 0 and lo[0] in (0.0, -np.inf) and up[0] in (0.0, np.inf) and np.all(lo == lo[0]) \
            and np.all(up == up[0]):
        vecs -= 2
    return nnz * (value_bytes + 4) + starts + m * value_bytes + vecs * n * value_bytes


def dual_step_bytes(lp, value_bytes, halpern=False, step_rows=None):
    """Rows of A: nonzeros, m + 1 starts, x_bar gathered once (n), and the row epilogue:
    classic, 13 m-vectors (y, r, r_bar, c_r, l_r, u_r, y_avg, r_avg read; y_new, r_new, r_bar,
    y_avg, r_avg written); Halpern, 9 (y, r, c_r, l_r, u_r, y0, r0 read; y_new, r_new written;
    y^, r^ only by a chunk's last step). (The solves here have no right-hand side vector, which
    adds one.) With step_rows < m (inert rows left out: no nonzeros, a logical that stays 0),
    the epilogue covers the stepped rows only, which the launch reads from a row list (4 bytes
    each) beside their starts."""
    n, m, nnz = lp.n, lp.m, lp.nnz
    vecs = 9 if halpern else 13
    if step_rows is not None and step_rows < m:
        return (nnz * (value_bytes + 4) + step_rows * 8 + n * value_bytes
                + vecs * step_rows * value_bytes)
    return nnz * (value_bytes + 4) + (m + 1) * 4 + n * value_bytes + vecs * m * value_bytes


def oracle_problem(model):
    """The LpProblem of a model built by the oracle's restatement of the reference's
    compute_scaling + make_problem (bit-identical to the reference's): the reference arm loads no
    library of the engine."""
    from oracle import oracle as o
    from samaya_gb300.model import LpProblem
    col, row = o.compute_scaling(model.m, model.n, model.colptr, model.rowidx, model.vals)
    colptr, rowidx, vals, cost, lower, upper = o.make_problem(model, col, row)
    return LpProblem(m=model.m, n=model.n, colptr=colptr, rowidx=rowidx, vals=vals, cost=cost,
                     lower=lower, upper=upper)


def cpu_reference_run(lp, cap_s=CPU_CAP_S):
    """The reference's CPU PDLP (oracle port of src/lp/pdlp.cpp, one core) on the LP to the
    tolerance with a time cap: (seconds, converged, iterations, relative [primal, dual, gap] at
    the end)."""
    from oracle import oracle as o
    t0 = time.perf_counter()
    r = o.pdlp_solve(*lp.arrays(), tol=TOL, max_iter=-1, time_limit=cap_s)
    dt = time.perf_counter() - t0
    if r.status == o.OPTIMAL:
        last = (r.primal_residual, r.dual_residual, r.gap)
    else:
        last = r.stats.get("last", (r.primal_residual, r.dual_residual, r.gap))
    return dt, r.status == o.OPTIMAL, r.iterations, [float(q) for q in last]


def _device_clock_line(line, clk):
    line["clocks"] = clk.summary()
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args):
    """LPs/s of one persistent batched launch against sequential single-LP GPU solves (1e-4, the
    batch's tolerance for node relaxations and screening), FP64 and FP32 storage.
    batchA: 512 random sparse LPs, m ~ U[100, 5000], n = ceil(m U[2, 3]);
    batchB: 256 node relaxations of one facility-location LP (100 x 400), 5% of the facility
    variables fixed to 0 or 1 per node."""
    import numpy as np
    import samaya_gb300 as sg
    from samaya_gb300 import generators as g
    from samaya_gb300.batch import BatchSolver
    from samaya_gb300.problem import make_problem
    tol = 1e-4
    if args.workload == "batchA":
        sizes = g.batch_a_sizes(512, seed=0)
        probs = [make_problem(g.random_sparse_lp(mm, nn, seed=1000 + k))[0]
                 for k, (mm, nn) in enumerate(sizes)]
        make = lambda opts: BatchSolver.from_problems(probs, opts)  # noqa: E731
        singles = probs
        cfg = {"workload": "512 random sparse LPs, m ~ U[100,5000], n = ceil(m U[2,3])",
               "instances": 512, "nnz": int(sum(p.nnz for p in probs))}
    else:
        model = g.facility_location_lp(100, 400, seed=0)
        lp, sc = make_problem(model)
        bounds = []
        for lo, up in g.facility_node_bounds(model, 100, 256, seed=1):
            l2 = lp.lower.copy()
            u2 = lp.upper.copy()
            l2[:lp.n] = lo / sc.col
            u2[:lp.n] = up / sc.col
            bounds.append((l2, u2))
        make = lambda opts: BatchSolver.shared(lp, bounds, opts)  # noqa: E731
        singles = [sg.LpProblem(m=lp.m, n=lp.n, colptr=lp.colptr, rowidx=lp.rowidx,
                                vals=lp.vals, cost=lp.cost, lower=lo, upper=up)
                   for lo, up in bounds]
        cfg = {"workload": "256 facility-location node relaxations (100 x 400) sharing A",
               "instances": 256, "nnz": int(lp.nnz)}
    out = {}
    # The workload's algorithm and the Halpern iteration beside it.
    names = {"reference": sg.REFERENCE, "enhanced": sg.ENHANCED, "halpern": sg.HALPERN}
    algs = tuple((a, names[a]) for a in dict.fromkeys((args.algorithm, "halpern")))
    with Clocks(0) as clk:
        for name, prec in (("fp64", sg.FP64), ("fp32", sg.FP32_REFINED)):
            for alg_name, alg in algs:
                s = make(sg.PdlpOptions(tol=tol, precision=prec, algorithm=alg))
                for _ in range(args.warmup):
                    s.solve(download=False)
                times = []
                for _ in range(args.steps):
                    r = s.solve(download=False)
                    times.append(s.device_ms / 1e3)
                s.close()
                t = sum(times) / len(times)
                out[f"{name}_{alg_name}"] = {
                    "seconds": t, "lps_per_s": len(r) / t,
                    "optimal": int(sum(x.status == sg.OPTIMAL for x in r)),
                    "mean_iterations": float(np.mean([x.iterations for x in r])),
                    "max_iterations": int(max(x.iterations for x in r))}
        # Sequential single-LP GPU solves (each precision and algorithm) on a sample of the
        # instances.
        seq = {}
        k = 16
        for name, prec in (("fp64", sg.FP64), ("fp32", sg.FP32_REFINED)):
            for alg_name, alg in algs:
                ms = 0.0
                for p in singles[:k]:
                    ms += sg.solve_pdlp(p, sg.PdlpOptions(tol=tol, precision=prec,
                                                          algorithm=alg)).device_ms
                seq[f"{name}_{alg_name}"] = {"lps_per_s": k / (ms / 1e3), "sample": k}
    best = max(out.values(), key=lambda v: v["lps_per_s"])
    line = {"metric": "batched PDLP LPs/s at 1e-4 (one persistent launch)",
            "value": best["lps_per_s"], "unit": "LPs/s", "higher_is_better": True,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
            "config": dict(cfg, tol=tol), "batch": out, "sequential": seq,
            "speedup_vs_sequential": {key: out[key]["lps_per_s"] / seq[key]["lps_per_s"]
                                      for key in seq}}
    return _device_clock_line(line, clk)


def run_diff(args):
    """The differentiable layer on 64 random sparse LPs (m = 500, n = 1200, FP64): forward
    (batched PDLP to 1e-8 + 2000 unrolled PDHG iterations) and backward (envelope gradients +
    the checkpointed adjoint), seconds per step."""
    import numpy as np
    import samaya_gb300 as sg
    from samaya_gb300 import generators as g
    from samaya_gb300.diff import LpLayer, UnrolledPdhg
    from samaya_gb300.problem import make_problem
    B, m, n = 64, 500, 1200
    probs = [make_problem(g.random_sparse_lp(m, n, seed=k))[0] for k in range(B)]
    cost = np.stack([p.cost for p in probs])
    lower = np.stack([p.lower for p in probs])
    upper = np.stack([p.upper for p in probs])
    layer = LpLayer(probs, tol=1e-8, iterations=2000, checkpoint_every=64)
    fw, bw, un_f, un_b = [], [], [], []
    with Clocks(0) as clk:
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            obj, vstar, ystar, vk, status = layer.evaluate(cost, lower, upper)
            t1 = time.perf_counter()
            layer.vjp(np.ones(B), np.concatenate([vk[:, :n], np.zeros((B, m))], axis=1))
            t2 = time.perf_counter()
            batch, unroll = layer._state[0], layer._state[1]
            t3 = time.perf_counter()
            unroll.forward()
            t4 = time.perf_counter()
            unroll.adjoint(np.ones(unroll.total))
            t5 = time.perf_counter()
            if i >= args.warmup:
                fw.append(t1 - t0)
                bw.append(t2 - t1)
                un_f.append(t4 - t3)
                un_b.append(t5 - t4)
    layer.close()
    mean = lambda a: sum(a) / len(a)  # noqa: E731
    line = {"metric": "differentiable LP layer, seconds per forward + backward",
            "value": mean(fw) + mean(bw), "unit": "s", "higher_is_better": False,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
            "config": {"workload": "64 random sparse LPs m=500 n=1200 (nnz 7200 each), FP64",
                       "unrolled_iterations": 2000, "checkpoint_every": 64, "tol": 1e-8},
            "forward_s": mean(fw), "backward_s": mean(bw),
            "unroll_forward_s": mean(un_f), "unroll_adjoint_s": mean(un_b),
            "all_optimal": bool(np.all(status == sg.OPTIMAL))}
    return _device_clock_line(line, clk)


MPS_WORKLOADS = {
    "transport": "transportation LP 1000 supplies x 2000 demands as a free-MPS file (3,000 rows, "
                 "2,000,000 columns, 4,000,000 entries, two entries to a line)",
    "powerlaw": "power-law LP 1,000,000 x 2,000,000 as a free-MPS file (12,000,000 entries, "
                "two to a line; 1,000,000 RHS and 2,000,000 bound lines)"}


def mps_file(which="transport"):
    """An LP written as free MPS into a temporary directory (and read once, so that the timed
    reads come from the page cache). Returns (path, bytes, directory)."""
    import tempfile
    from samaya_gb300 import generators as g
    from samaya_gb300.mps import write_mps
    tmp = tempfile.mkdtemp(prefix="sg_mps_")
    path = os.path.join(tmp, f"{which}.mps")
    model = g.transportation_lp(1000, 2000, seed=0) if which == "transport" else \
        g.power_law_lp(seed=0)
    write_mps(model, path)
    with open(path, "rb") as f:
        while f.read(1 << 24):
            pass
    return path, os.path.getsize(path), tmp


def run_mps(args):
    """The fast MPS reader (include/sg_mps.h): seconds per read of the transportation LP's file
    through the C ABI (value; the model stays in the engine library's handle) and through the
    Python API (e2e: the arrays copied out into numpy); where a GPU is present also file to
    answer (read, create on the device, solve to 1e-8) against the same solve from the model in
    memory; samaya's own reader (oracle/_ref) beside it where it was built."""
    import ctypes
    import shutil
    from samaya_gb300 import _native
    from samaya_gb300 import mps
    path, size, tmp = mps_file(args.mps_lp)
    lib = _native.load()
    mps._declare(lib)
    try:
        def c_read():
            h = ctypes.c_void_p()
            t0 = time.perf_counter()
            rc = lib.sg_mps_read(os.fsencode(path), 0, ctypes.byref(h))
            dt = time.perf_counter() - t0
            if rc != 0:
                raise RuntimeError(lib.sg_pdlp_last_error().decode())
            lib.sg_mps_free(h)
            return dt
        c_times, py_times = [], []
        for i in range(args.warmup + args.steps):
            dt = c_read()
            t0 = time.perf_counter()
            f = mps.read_mps(path)
            dp = time.perf_counter() - t0
            if i >= args.warmup:
                c_times.append(dt)
                py_times.append(dp)
        value = sum(c_times) / len(c_times)
        e2e = sum(py_times) / len(py_times)
        line = {"metric": "MPS read time (fast reader)", "value": value, "unit": "s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": MPS_WORKLOADS[args.mps_lp], "file_bytes": size,
                           "threads": "automatic (one per MiB of a section, at most "
                                      "the hardware's)"},
                "mb_per_s": size / value / 1e6, "host_cores": os.cpu_count(),
                "gpu_launches": 0,
                "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0,
                        "what": "samaya_gb300.mps.read_mps: the C read plus the copy of the "
                                "model's arrays and names into numpy"},
                "nnz": f.model.nnz}
        try:
            from oracle import ref
            if ref.available() and ref.build():
                t = [ref.mps_read_file(path)["seconds"] for _ in range(2)]
                line["cpu_baseline"] = {"value": min(t), "unit": "s", "cores": 1,
                                        "kind": "reference",
                                        "sample": "samaya::read_mps on the same file (the "
                                                  "reference's reader, compiled by "
                                                  "oracle/Makefile.ref)"}
        except Exception as e:  # the reference build is optional test infrastructure
            line["cpu_baseline"] = {"unavailable": str(e)}
        if _native_gpu() and args.mps_lp == "transport":
            line["from_file"] = mps_to_answer(path, args)
        print(json.dumps(line), flush=True)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return 0


def mps_reader_summary(reads=3):
    """The fast MPS reader on this LP's 93.5 MB file, beside the solve: the fastest of a few
    reads through the C ABI (host threads; no GPU). A failure is reported in the field, not in
    the line."""
    import ctypes
    import shutil
    from samaya_gb300 import _native
    from samaya_gb300 import mps
    tmp = None
    try:
        path, size, tmp = mps_file("transport")
        lib = _native.load()
        mps._declare(lib)
        best = None
        for _ in range(reads):
            h = ctypes.c_void_p()
            t0 = time.perf_counter()
            rc = lib.sg_mps_read(os.fsencode(path), 0, ctypes.byref(h))
            dt = time.perf_counter() - t0
            if rc != 0:
                return {"error": lib.sg_pdlp_last_error().decode(errors="replace")}
            lib.sg_mps_free(h)
            best = dt if best is None else min(best, dt)
        return {"seconds": best, "file_bytes": size, "mb_per_s": size / best / 1e6,
                "host_cores": os.cpu_count(), "workload": MPS_WORKLOADS["transport"],
                "what": "sg_mps_read of the file (page cache), fastest of "
                        f"{reads}; samaya's read_mps takes 2.3-2.7 s on 8 Xeon cores"}
    except Exception as e:  # the headline line stands without this extra figure
        return {"error": f"{type(e).__name__}: {e}"}
    finally:
        if tmp is not None:
            shutil.rmtree(tmp, ignore_errors=True)


def _native_gpu():
    import samaya_gb300 as sg
    return sg.gpu_info()["gpu"] is not None


def mps_to_answer(path, args):
    """Seconds from the MPS file to the answer (fast read, device setup from the model, mixed
    precision solve to 1e-8), and the same solve from the model already in memory."""
    import samaya_gb300 as sg
    from samaya_gb300 import mps
    opts = solver_options(args, "mixed")
    model = mps.read_mps(path).model

    def solve(md):
        with sg.PdlpSolver.from_model(md, opts) as s:
            return s.solve()
    file_s, mem_s = [], []
    for _ in range(2):
        t0 = time.perf_counter()
        r = solve(mps.read_mps(path).model)
        file_s.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        solve(model)
        mem_s.append(time.perf_counter() - t0)
    return {"file_s": min(file_s), "memory_s": min(mem_s), "status": r.status_name}


def run_reference(args):
    world, rank, _ = dist()
    if rank != 0:
        return 0
    if args.workload == "mps":
        return run_reference_mps(args)
    if args.workload not in ("transport", "powerlaw", "random"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference solves one LP at "
                          "a time and has no adjoint: no counterpart of this workload"}))
        return 0
    model, cfg = workload(args.workload)
    lp = oracle_problem(model)
    times, info = [], None
    for i in range(args.warmup + args.steps):
        dt, conv, iters, last = cpu_reference_run(lp)
        if i >= args.warmup:
            times.append(dt)
            info = (conv, iters, last)
    value = sum(times) / len(times)
    sample = (f"reference CPU PDLP (oracle port of samaya src/lp/pdlp.cpp, bit-identical to it) "
              f"to {TOL:g} capped at {CPU_CAP_S:.0f} s per step on the same LP; converged="
              f"{info[0]}, {info[1]} iterations, relative primal / dual / gap at the end "
              f"{info[2][0]:.2e} / {info[2][1]:.2e} / {info[2][2]:.2e}")
    line = {"metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": dict(cfg, tol=TOL), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "s", "cores": 1, "kind": "port",
                             "sample": sample, "converged": info[0], "iterations": info[1],
                             "relative_kkt": info[2]},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_reference_mps(args):
    """samaya::read_mps on the same file, where the reference's reader was compiled
    (oracle/_ref: built from the reference checkout, which only the build machine has)."""
    import shutil
    try:
        from oracle import ref
        if not (ref.available() and ref.build()):
            raise RuntimeError("samaya's compiled reader (oracle/_ref) is not on this machine")
    except Exception as e:
        print(json.dumps({"impl": "reference", "unavailable": str(e)}))
        return 0
    path, size, tmp = mps_file(args.mps_lp)
    try:
        times = []
        for i in range(args.warmup + args.steps):
            dt = ref.mps_read_file(path)["seconds"]
            if i >= args.warmup:
                times.append(dt)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    value = sum(times) / len(times)
    sample = "samaya::read_mps (src/io/mps_reader.cpp:530) on the same file, 1 thread"
    print(json.dumps({"metric": "MPS read time (fast reader)", "value": value, "unit": "s",
                      "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                      "config": {"workload": MPS_WORKLOADS[args.mps_lp], "file_bytes": size},
                      "impl": "reference",
                      "cpu_baseline": {"value": value, "unit": "s", "cores": 1,
                                       "kind": "reference", "sample": sample},
                      "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args)
    if args.workload in ("batchA", "batchB"):
        return run_batch(args)
    if args.workload == "diff":
        return run_diff(args)
    if args.workload == "mps":
        return run_mps(args)
    world, rank, local = dist()
    import numpy as np
    import samaya_gb300 as sg
    from samaya_gb300.problem import make_problem
    from samaya_gb300 import _native
    _native.load()
    torch = None
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", "0"))

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    model, cfg = workload(args.workload, seed=rank)
    lp, scaling = make_problem(model)
    mixed = args.precision != "fp64"
    opts = solver_options(args, args.precision)
    solver = sg.PdlpSolver(lp, opts)
    cfg["tiles"] = {k: {"nnz_per_tile": v[0], "rows_per_tile": v[1], "tiles": v[2],
                        "kernel_variant": v[3], "team_split": v[4]}
                    for k, v in solver.tile_shapes().items()}
    for _ in range(args.warmup):
        warm = solver.solve(download=False)
    barrier()
    results = []
    with Clocks(local) as clk:
        barrier()
        for _ in range(args.steps):
            results.append(solver.solve(download=False))
        barrier()
    dev_s = [r.device_ms / 1e3 for r in results]
    t_step = sum(dev_s) / len(dev_s)
    if world > 1:
        t = torch.tensor([t_step], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item())
    last = results[-1]
    # The other precision modes (same algorithm, same LP), FP64 above all: the mixed-vs-FP64
    # comparison of the metric.
    others = {}
    for name in PRECISION_NAMES:
        if name == args.precision:
            continue
        with sg.PdlpSolver(lp, solver_options(args, name, args.other_time_limit)) as so:
            first = so.solve(download=False)
            reps = max(1, min(args.steps, 3)) if first.device_ms < 10e3 else 1
            ro = [first] if reps == 1 and first.device_ms >= 10e3 else [
                so.solve(download=False) for _ in range(reps)]
        others[name] = {"seconds": sum(r.device_ms for r in ro) / len(ro) / 1e3,
                        "iterations": ro[-1].iterations, "status": ro[-1].status_name,
                        "relative_kkt": [ro[-1].primal_residual, ro[-1].dual_residual,
                                         ro[-1].gap]}
    # End to end through the C ABI from pinned host buffers.
    e2e_times = []
    h2d = (lp.colptr.nbytes + lp.rowidx.nbytes + lp.vals.nbytes + lp.cost.nbytes +
           lp.lower.nbytes + lp.upper.nbytes)
    d2h = 8 * (lp.n + lp.m) + 8 * lp.m
    pinned = _pinned_problem(lp)
    x_pin, y_pin = _pinned_outputs(lp)
    for _ in range(max(1, min(args.steps, 3)) if t_step < 10.0 else 1):
        t0 = time.perf_counter()
        # solve_pdlp's create + solve + destroy, the answer read into page-locked buffers.
        with sg.PdlpSolver(pinned, opts) as s:
            r = s.solve(x_out=x_pin, y_out=y_pin)
        e2e_times.append(time.perf_counter() - t0)
        assert r.status == sg.OPTIMAL
    # Roofline of the dominant kernel: event-timed launches on the engine's stream.
    ms_dual, ms_primal, ms_eval = solver.time_kernels(20)
    vb = 4 if mixed else 8
    halpern = args.algorithm == "halpern"
    pbytes = primal_step_bytes(lp, vb, halpern)
    dbytes = dual_step_bytes(lp, vb, halpern, solver.step_rows()[0])
    peak, peak_kind = peak_hbm()
    # Both step kernels launch once per iteration: the dominant one is the slower.
    prec_key = "fp32" if mixed else "fp64"
    traffic = traffic_summary()
    tkey = f"{args.workload}_{prec_key}" + ("_halpern" if halpern else "")
    steps = {
        "primal_step": {"kernel": "primal_step (A'y + projected x update + averages)",
                        "bytes_per_launch": pbytes, "ms_per_launch": ms_primal,
                        "achieved": pbytes / (ms_primal * 1e-3) / 1e9,
                        "traffic": traffic.get(f"{tkey}_primal_step")},
        "dual_step": {"kernel": "dual_step (A xbar + y update + logicals + averages)",
                      "bytes_per_launch": dbytes, "ms_per_launch": ms_dual,
                      "achieved": dbytes / (ms_dual * 1e-3) / 1e9,
                      "traffic": traffic.get(f"{tkey}_dual_step")},
    }
    top = max(steps, key=lambda k: steps[k]["ms_per_launch"])
    other = "dual_step" if top == "primal_step" else "primal_step"
    ach = steps[top]["achieved"]
    line = {
        "metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64",
        "data": "synthetic",
        "config": dict(cfg, tol=TOL, precision=PRECISION_NAMES[args.precision],
                       switch_tol=args.switch_tol if args.precision == "mixed" else None,
                       algorithm=ALGORITHM_NAMES[args.algorithm],
                       l2="inputs larger than L2" if lp.nnz >= 4_000_000 else
                       "inputs smaller than L2"),
        "status": last.status_name, "iterations": last.iterations,
        "refinement_rounds": last.refinement_rounds,
        "relative_kkt": [last.primal_residual, last.dual_residual, last.gap],
        "other_precisions": others,
        "e2e": {"value": min(e2e_times), "unit": "s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(sum(r.kernel_launches for r in results)),
        "roofline": {"bound": "hbm", "kernel": steps[top]["kernel"], "achieved": ach,
                     "peak": peak, "unit": "GB/s", "frac": ach / peak,
                     "peak_kind": peak_kind, "traffic": steps[top]["traffic"],
                     "bytes_per_launch": steps[top]["bytes_per_launch"],
                     "ms_per_launch": steps[top]["ms_per_launch"],
                     "precision_timed": prec_key, other: steps[other],
                     "evaluation_ms": ms_eval,
                     # One whole iteration (both fused steps): bytes over the sum of their
                     # event-timed launches.
                     "iteration": {
                         "bytes": pbytes + dbytes, "ms": ms_primal + ms_dual,
                         "achieved": (pbytes + dbytes) / ((ms_primal + ms_dual) * 1e-3) / 1e9,
                         "frac": (pbytes + dbytes) / ((ms_primal + ms_dual) * 1e-3) / 1e9
                         / peak}},
        "iterations_per_s": last.iterations / t_step,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1:
        line["e2e"]["from_model"] = setup_paths(model, opts)
        line["e2e"]["cold_process_s"] = cold_e2e(lp, args, args.precision)
        line["e2e"]["cold_process"] = (
            "the same call in a fresh process: library load, CUDA context, checks, transpose, "
            "upload, the tile tuner's first timing of both operators (cached afterwards), "
            "solve, download")
        if args.workload == "transport" and not args.no_largest:
            line["largest_config"] = largest_config(args)
        if args.workload == "transport":
            line["mps_reader"] = mps_reader_summary()
        dt, conv, iters, last_res = cpu_reference_run(lp)
        line["cpu_baseline"] = {
            "value": dt, "unit": "s", "cores": 1, "kind": "port",
            "sample": f"reference CPU PDLP (oracle port of samaya src/lp/pdlp.cpp) to {TOL:g} "
                      f"capped at {CPU_CAP_S:.0f} s on the same LP: converged={conv}, "
                      f"{iters} iterations, relative primal / dual / gap at the end "
                      f"{last_res[0]:.2e} / {last_res[1]:.2e} / {last_res[2]:.2e} (value is a "
                      f"lower bound of its time to the tolerance when not converged)",
            "converged": conv, "iterations": iters, "relative_kkt": last_res}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


_COLD_SCRIPT = """
import json, sys, time
sys.path.insert(0, {root!r})
import numpy as np
import samaya_gb300 as sg
from samaya_gb300.model import LpProblem
import torch
z = np.load({path!r})
def pin(a):
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
lp = LpProblem(m=int(z["m"]), n=int(z["n"]), **{{k: pin(z[k]) for k in
               ("colptr", "rowidx", "vals", "cost", "lower", "upper")}})
opts = sg.PdlpOptions(**json.loads({opts!r}))
t0 = time.perf_counter()
r = sg.solve_pdlp(lp, opts)
dt = time.perf_counter() - t0
print(json.dumps({{"seconds": dt, "status": r.status_name}}))
"""


def setup_paths(model, opts, reps=2):
    """The model's setup to a solved answer in the model's space, two ways (best of reps):
    host scaling + computational form (sg_scale_model) + sg_pdlp_create (host transpose,
    upload), against sg_pdlp_create_model (one upload, the same steps on the device); each then
    solves, downloads and maps the answer back. Seconds of each and of its setup part."""
    import samaya_gb300 as sg
    from samaya_gb300.problem import make_problem, model_solution
    out = {}
    for name in ("host_setup", "device_setup"):
        best = None
        for _ in range(reps):
            t0 = time.perf_counter()
            if name == "host_setup":
                lp, sc = make_problem(model)
                s = sg.PdlpSolver(lp, opts)
            else:
                s = sg.PdlpSolver.from_model(model, opts)
                sc = s.scaling
            t1 = time.perf_counter()
            r = s.solve()
            model_solution(model, sc, r.x, r.y)
            t2 = time.perf_counter()
            s.close()
            if best is None or t2 - t0 < best[0]:
                best = (t2 - t0, t1 - t0, r.status_name)
        out[name] = {"seconds": best[0], "setup_seconds": best[1], "status": best[2]}
    return out


def cold_e2e(lp, args, precision):
    """Seconds of one solve_pdlp through the C ABI from pinned host buffers in a fresh process
    (None if it fails): what a caller pays the first time, the tile tuner included."""
    import tempfile
    o = solver_options(args, precision)
    kw = {k: getattr(o, k) for k in ("tol", "precision", "algorithm", "inner_tol")}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "lp.npz")
        import numpy as np
        np.savez(path, m=lp.m, n=lp.n, colptr=lp.colptr, rowidx=lp.rowidx, vals=lp.vals,
                 cost=lp.cost, lower=lp.lower, upper=lp.upper)
        script = _COLD_SCRIPT.format(root=ROOT, path=path, opts=json.dumps(kw))
        env = dict(os.environ)
        env.pop("SG_TILE_CACHE", None)
        p = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True,
                           env=env, timeout=1200)
    try:
        out = json.loads(p.stdout.strip().splitlines()[-1])
        return out["seconds"] if out["status"] == "optimal" else None
    except Exception:
        return None


def largest_config(args):
    """The power-law LP (the largest configuration: 1e6 x 2e6, 12M nonzeros, Zipf(1.5) rows)
    to the tolerance in each precision mode with the Halpern iteration: one timed solve each
    (device time; a solve takes tens of seconds, so it is not repeated; each stops at
    --other-time-limit), the step kernels' roofline in FP64 and FP32 storage, and the
    reference's CPU PDLP (the oracle port, one core) on a capped run of the same LP."""
    import samaya_gb300 as sg
    from samaya_gb300.problem import make_problem
    model, cfg = workload("powerlaw")
    lp, _ = make_problem(model)
    a2 = argparse.Namespace(**vars(args))
    a2.algorithm = "halpern"
    peak, peak_kind = peak_hbm()
    traffic = traffic_summary()
    modes = {}
    for name in ("fp64", "refined", "mixed"):
        with sg.PdlpSolver(lp, solver_options(a2, name, args.other_time_limit)) as s:
            r = s.solve(download=False)
            entry = {"seconds": r.device_ms / 1e3, "iterations": r.iterations,
                     "status": r.status_name,
                     "relative_kkt": [r.primal_residual, r.dual_residual, r.gap],
                     "refinement_rounds": r.refinement_rounds}
            if name in ("fp64", "refined"):
                md, mp, _ = s.time_kernels(20)
                vb = 8 if name == "fp64" else 4
                db = dual_step_bytes(lp, vb, True, s.step_rows()[0])
                pb = primal_step_bytes(lp, vb, True)
                key = "powerlaw_fp64_halpern" if vb == 8 else "powerlaw_fp32_halpern"
                entry["step_kernels"] = {
                    "storage": "fp64" if vb == 8 else "fp32",
                    "dual_step": {"ms": md, "bytes": db, "achieved_gbs": db / (md * 1e-3) / 1e9,
                                  "frac": db / (md * 1e-3) / 1e9 / peak,
                                  "traffic": traffic.get(f"{key}_dual_step")},
                    "primal_step": {"ms": mp, "bytes": pb,
                                    "achieved_gbs": pb / (mp * 1e-3) / 1e9,
                                    "frac": pb / (mp * 1e-3) / 1e9 / peak,
                                    "traffic": traffic.get(f"{key}_primal_step")},
                    "peak_gbs": peak, "peak_kind": peak_kind}
        modes[name] = entry
    optimal = {k: v for k, v in modes.items() if v["status"] == "optimal"}
    dt, conv, iters, last_res = cpu_reference_run(oracle_problem(model))
    return {"config": dict(cfg, tol=TOL, algorithm=ALGORITHM_NAMES["halpern"]),
            "modes": modes,
            "fastest_optimal": min(optimal, key=lambda k: optimal[k]["seconds"]) if optimal
            else None,
            "cpu_baseline": {"value": dt, "unit": "s", "cores": 1, "kind": "port",
                             "converged": conv, "iterations": iters, "relative_kkt": last_res,
                             "sample": f"reference CPU PDLP (oracle port) capped at "
                                       f"{CPU_CAP_S:.0f} s on the same LP"}}


def _pinned_problem(lp):
    """The LpProblem's arrays copied into page-locked host memory (torch), if available."""
    try:
        import torch
        from samaya_gb300.model import LpProblem

        def pin(a):
            t = torch.from_numpy(a.copy()).pin_memory()
            return t.numpy()
        return LpProblem(m=lp.m, n=lp.n, colptr=pin(lp.colptr), rowidx=pin(lp.rowidx),
                         vals=pin(lp.vals), cost=pin(lp.cost), lower=pin(lp.lower),
                         upper=pin(lp.upper))
    except Exception:
        return lp


def _pinned_outputs(lp):
    """Page-locked host buffers for the answer (x: n + m, y: m), if torch can pin memory."""
    import numpy as np
    try:
        import torch
        x = torch.empty(lp.n + lp.m, dtype=torch.float64).pin_memory().numpy()
        y = torch.empty(max(lp.m, 1), dtype=torch.float64).pin_memory().numpy()
        return x, y
    except Exception:
        return np.empty(lp.n + lp.m), np.empty(max(lp.m, 1))


if __name__ == "__main__":
    sys.exit(main())
