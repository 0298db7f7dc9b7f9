"""Host-side mirror of samaya's PDLP interface, over the engine's C ABI.

``solve_pdlp(lp, options)`` follows ``samaya::solve_pdlp(const LpProblem&, const PdlpOptions&,
const Logger&) -> PdlpResult`` (reference src/lp/pdlp.hpp:35): same problem form, option
meanings, status values and result fields, results in the LpProblem's space.  Unlike the
reference's GPU path there is no CPU fallback inside: without the CUDA library or a GB300 the
call raises.  ``PdhgDevice`` mirrors the reference's inner seam ``gpu::PdhgDevice``
(src/gpu/pdhg_core.hpp:24-79).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _native
from .model import LpProblem

# SimplexStatus (reference src/lp/simplex.hpp:28-35).
OPTIMAL, INFEASIBLE, UNBOUNDED, ITERATION_LIMIT, TIME_LIMIT, NUMERICAL_ERROR = range(6)
STATUS_NAMES = ["optimal", "infeasible", "unbounded", "iteration_limit", "time_limit",
                "numerical_error"]

FP64 = 0
FP32_REFINED = 1
FP32_THEN_FP64 = 2
REFERENCE = 0
ENHANCED = 1
HALPERN = 2


@dataclass
class PdlpOptions:
    """``samaya::PdlpOptions`` (src/lp/pdlp.hpp:11-16) plus the engine's precision knobs."""
    tol: float = 1e-8
    max_iterations: int = -1
    time_limit: float = float("inf")
    use_gpu: bool = True
    precision: int = FP64
    refine_max_rounds: int = 6
    inner_tol: float = 1e-4
    algorithm: int = REFERENCE
    verbose: int = 0
    autotune: bool = True
    tile_split: int = 0
    artificial_restart: float = 0.0
    keep_inert_rows: bool = False
    row_groups: int = 0
    segment_staging: int = 0
    tile_nnz: int = 0

    def to_c(self) -> _native.Opts:
        o = _native.Opts()
        _native.load().sg_pdlp_default_opts(ctypes.byref(o))
        o.tol = float(self.tol)
        o.max_iterations = int(self.max_iterations)
        o.time_limit = float(self.time_limit) if np.isfinite(self.time_limit) else 0.0
        o.precision = int(self.precision)
        o.refine_max_rounds = int(self.refine_max_rounds)
        o.inner_tol = float(self.inner_tol)
        o.algorithm = int(self.algorithm)
        o.verbose = int(self.verbose)
        o.autotune = 1 if self.autotune else 0
        o.tile_split = int(self.tile_split)
        o.artificial_restart = float(self.artificial_restart)
        o.keep_inert_rows = 1 if self.keep_inert_rows else 0
        o.row_groups = int(self.row_groups)
        o.segment_staging = int(self.segment_staging)
        o.tile_nnz = int(self.tile_nnz)
        return o


@dataclass
class PdlpResult:
    """``samaya::PdlpResult`` (src/lp/pdlp.hpp:19-30) plus engine counters."""
    status: int = NUMERICAL_ERROR
    x: np.ndarray = field(default_factory=lambda: np.zeros(0))
    y: np.ndarray = field(default_factory=lambda: np.zeros(0))
    dual_ray: np.ndarray = field(default_factory=lambda: np.zeros(0))
    primal_ray: np.ndarray = field(default_factory=lambda: np.zeros(0))
    iterations: int = 0
    primal_residual: float = 0.0
    dual_residual: float = 0.0
    gap: float = 0.0
    primal_objective: float = 0.0
    dual_objective: float = 0.0
    restarts: int = 0
    evaluations: int = 0
    refinement_rounds: int = 0
    setup_seconds: float = 0.0
    solve_seconds: float = 0.0
    step_size: float = 0.0
    primal_weight: float = 1.0
    kernel_launches: int = 0
    device_ms: float = 0.0

    @property
    def status_name(self) -> str:
        return STATUS_NAMES[self.status]


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _as_problem(lp):
    if isinstance(lp, LpProblem):
        return lp
    return LpProblem(**lp)


class PdlpSolver:
    """One uploaded LpProblem (an engine handle); ``solve()`` may be called repeatedly and
    gives the same bits each time."""

    def __init__(self, lp, options: PdlpOptions | None = None):
        self._lib = _native.load()
        self.lp = _as_problem(lp)
        self.options = options or PdlpOptions()
        self._h = ctypes.c_void_p()
        lp = self.lp
        o = self.options.to_c()
        _native.check(self._lib.sg_pdlp_create(
            ctypes.byref(self._h), lp.m, lp.n, _ptr(lp.colptr, ctypes.c_int64),
            _ptr(lp.rowidx, ctypes.c_int32), _ptr(lp.vals, ctypes.c_double),
            _ptr(lp.cost, ctypes.c_double), _ptr(lp.lower, ctypes.c_double),
            _ptr(lp.upper, ctypes.c_double), ctypes.byref(o)), "sg_pdlp_create")

    @classmethod
    def from_model(cls, model, options: PdlpOptions | None = None):
        """An engine for a model's LpProblem built on the GPU (sg_pdlp_create_model: scaling,
        computational form and the row-major copy on the device). ``solve()`` answers in the
        LpProblem's space; ``scaling`` holds the factors for ``problem.model_solution``."""
        from .problem import Scaling
        self = cls.__new__(cls)
        self._lib = _native.load()
        self.options = options or PdlpOptions()
        self._h = ctypes.c_void_p()
        m, n = int(model.m), int(model.n)
        self.lp = LpProblem(m=m, n=n, colptr=np.zeros(n + 1, dtype=np.int64),
                            rowidx=np.zeros(0, dtype=np.int32), vals=np.zeros(0),
                            cost=np.zeros(0), lower=np.zeros(0), upper=np.zeros(0))
        col, row = np.zeros(max(n, 1)), np.zeros(max(m, 1))
        o = self.options.to_c()
        D = ctypes.c_double
        _native.check(self._lib.sg_pdlp_create_model(
            ctypes.byref(self._h), m, n, _ptr(model.colptr, ctypes.c_int64),
            _ptr(model.rowidx, ctypes.c_int32), _ptr(model.vals, D), _ptr(model.obj, D),
            _ptr(model.col_lower, D), _ptr(model.col_upper, D), _ptr(model.row_lower, D),
            _ptr(model.row_upper, D), 1 if model.maximize else 0, ctypes.byref(o),
            _ptr(col, D), _ptr(row, D)), "sg_pdlp_create_model")
        self.scaling = Scaling(col=col[:n].copy(), row=row[:m].copy())
        return self

    def time_kernels(self, reps: int = 20):
        """Average device ms of one dual step, one primal step and one evaluation (CUDA events
        on the engine's stream); the next solve starts afresh."""
        a, b, c = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
        _native.check(self._lib.sg_pdlp_time_kernels(self._h, reps, ctypes.byref(a),
                                                     ctypes.byref(b), ctypes.byref(c)),
                      "sg_pdlp_time_kernels")
        return a.value, b.value, c.value

    def equilibration(self):
        """The device setup of a solve, read back: (col_scale, row_scale, operator norm of
        [A_eq -I], step size 0.99 / norm)."""
        lp = self.lp
        cs = np.zeros(max(lp.n, 1))
        rs = np.zeros(max(lp.m, 1))
        norm, eta = ctypes.c_double(0), ctypes.c_double(0)
        _native.check(self._lib.sg_pdlp_equilibration(self._h, _ptr(cs, ctypes.c_double),
                                                      _ptr(rs, ctypes.c_double),
                                                      ctypes.byref(norm), ctypes.byref(eta)),
                      "sg_pdlp_equilibration")
        return cs[:lp.n], rs[:lp.m], norm.value, eta.value

    def tile_shapes(self):
        """{"A": (nonzeros per tile, rows per short-row tile, tiles, step kernel variant,
        nonzeros per warp of a medium row's team or 0), "At": ...} in use."""
        out = {}
        for name, t in (("A", 0), ("At", 1)):
            v = [ctypes.c_int(0) for _ in range(5)]
            _native.check(self._lib.sg_pdlp_tile_shape(self._h, t, *[ctypes.byref(x) for x in v]),
                          "sg_pdlp_tile_shape")
            out[name] = (v[0].value, v[1].value, v[2].value, v[3].value, v[4].value)
        return out

    def step_rows(self) -> tuple[int, int, int, int]:
        """(rows of A the dual steps run over, their tiles, the row-group tiles among them,
        1 if the long rows' segments are staged through shared memory): m rows unless inert
        rows (empty, a logical with no cost and 0 within its bounds) are left out."""
        v = [ctypes.c_int(0) for _ in range(4)]
        _native.check(self._lib.sg_pdlp_step_rows(self._h, *[ctypes.byref(x) for x in v]),
                      "sg_pdlp_step_rows")
        return v[0].value, v[1].value, v[2].value, v[3].value

    def solve(self, x_out: np.ndarray | None = None, y_out: np.ndarray | None = None,
              download: bool = True) -> PdlpResult:
        """Solves; with ``download=False`` the answer stays on the device (x, y empty)."""
        lp = self.lp
        if not download:
            r = _native.Result()
            _native.check(self._lib.sg_pdlp_solve(self._h, ctypes.byref(r), None, None, None,
                                                  None), "sg_pdlp_solve")
            return PdlpResult(status=r.status, iterations=r.iterations,
                              primal_residual=r.primal_residual, dual_residual=r.dual_residual,
                              gap=r.gap, primal_objective=r.primal_objective,
                              dual_objective=r.dual_objective, restarts=r.restarts,
                              evaluations=r.evaluations, refinement_rounds=r.refinement_rounds,
                              setup_seconds=r.setup_seconds, solve_seconds=r.solve_seconds,
                              step_size=r.step_size, primal_weight=r.primal_weight,
                              kernel_launches=r.kernel_launches, device_ms=r.device_ms)
        # The engine writes every entry of x and y; a ray only with its flag set (copied out
        # below), so none of these needs zeroing.
        x = x_out if x_out is not None else np.empty(lp.n + lp.m)
        y = y_out if y_out is not None else np.empty(max(lp.m, 1))
        dr = np.empty(max(lp.m, 1))
        pr = np.empty(max(lp.n, 1))
        r = _native.Result()
        _native.check(self._lib.sg_pdlp_solve(self._h, ctypes.byref(r), _ptr(x, ctypes.c_double),
                                              _ptr(y, ctypes.c_double), _ptr(dr, ctypes.c_double),
                                              _ptr(pr, ctypes.c_double)), "sg_pdlp_solve")
        out = PdlpResult(status=r.status, x=x, y=y[:lp.m], iterations=r.iterations,
                         primal_residual=r.primal_residual, dual_residual=r.dual_residual,
                         gap=r.gap, primal_objective=r.primal_objective,
                         dual_objective=r.dual_objective, restarts=r.restarts,
                         evaluations=r.evaluations, refinement_rounds=r.refinement_rounds,
                         setup_seconds=r.setup_seconds, solve_seconds=r.solve_seconds,
                         step_size=r.step_size, primal_weight=r.primal_weight,
                         kernel_launches=r.kernel_launches, device_ms=r.device_ms)
        if r.has_dual_ray:
            out.dual_ray = dr[:lp.m].copy()
        if r.has_primal_ray:
            out.primal_ray = pr[:lp.n].copy()
        return out

    def close(self):
        if self._h:
            self._lib.sg_pdlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def solve_pdlp(lp, options: PdlpOptions | None = None) -> PdlpResult:
    """``samaya::solve_pdlp`` on the GPU engine (options.use_gpu is implied)."""
    with PdlpSolver(lp, options) as s:
        return s.solve()


def gpu_info() -> dict:
    """``samaya::gpu_info`` (reference src/gpu/info.cpp:12-19): built_with_cuda and device."""
    lib = _native.load()
    major, minor = ctypes.c_int(0), ctypes.c_int(0)
    name = ctypes.create_string_buffer(256)
    rc = lib.sg_pdlp_available(ctypes.byref(major), ctypes.byref(minor), name, 256)
    return {"cuda": True, "gpu": name.value.decode() if rc == 0 else None,
            "compute_capability": f"{major.value}.{minor.value}" if rc == 0 else None}


class PdhgDevice:
    """``gpu::PdhgDevice`` (reference src/gpu/pdhg_core.hpp:24-79) on the engine's kernels.
    ``which``: 0 current iterate (v_new, y_new), 1 average."""

    CURRENT = 0
    AVERAGE = 1

    def __init__(self, m, n, colptr, rowidx, vals, cost, lower, upper,
                 options: PdlpOptions | None = None):
        """``options`` (the engine's own knobs, e.g. the tile shape): None keeps the defaults
        ``sg_pdhg_create`` uses."""
        self._lib = _native.load()
        self.m, self.n = int(m), int(n)
        self._keep = [np.ascontiguousarray(colptr, dtype=np.int64),
                      np.ascontiguousarray(rowidx, dtype=np.int32),
                      np.ascontiguousarray(vals, dtype=np.float64),
                      np.ascontiguousarray(cost, dtype=np.float64),
                      np.ascontiguousarray(lower, dtype=np.float64),
                      np.ascontiguousarray(upper, dtype=np.float64)]
        k = self._keep
        self._h = ctypes.c_void_p()
        args = (ctypes.byref(self._h), self.m, self.n, _ptr(k[0], ctypes.c_int64),
                _ptr(k[1], ctypes.c_int32), _ptr(k[2], ctypes.c_double),
                _ptr(k[3], ctypes.c_double), _ptr(k[4], ctypes.c_double),
                _ptr(k[5], ctypes.c_double))
        if options is None:
            _native.check(self._lib.sg_pdhg_create(*args), "sg_pdhg_create")
        else:
            o = options.to_c()
            _native.check(self._lib.sg_pdlp_create(*args, ctypes.byref(o)), "sg_pdlp_create")

    def step_rows(self) -> tuple[int, int, int, int]:
        """As ``PdlpSolver.step_rows``: the rows, tiles, row-group tiles and segment staging of
        the dual steps."""
        v = [ctypes.c_int(0) for _ in range(4)]
        _native.check(self._lib.sg_pdlp_step_rows(self._h, *[ctypes.byref(x) for x in v]),
                      "sg_pdlp_step_rows")
        return v[0].value, v[1].value, v[2].value, v[3].value

    def set_original(self, col_scale, row_scale, cost, lower, upper):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in
                (col_scale, row_scale, cost, lower, upper)]
        _native.check(self._lib.sg_pdhg_set_original(self._h, *[_ptr(a, ctypes.c_double)
                                                                for a in arrs]),
                      "sg_pdhg_set_original")

    def step(self, tau, sigma, theta, iteration):
        _native.check(self._lib.sg_pdhg_step(self._h, tau, sigma, theta, iteration),
                      "sg_pdhg_step")

    def advance(self):
        _native.check(self._lib.sg_pdhg_advance(self._h), "sg_pdhg_advance")

    def set_state(self, v, y, v_anchor, y_anchor, precision: int = FP64):
        """The point the next single step starts from (current v, y; extrapolated point v;
        anchor / restart point; averages zero). An FP32 ``precision`` (the device must have
        been created with an FP32 precision) rounds the problem and the vectors to FP32 and
        runs the FP32 kernels from then on."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (v, y, v_anchor, y_anchor)]
        if self.m == 0:
            arrs[1] = arrs[3] = np.zeros(1)
        _native.check(self._lib.sg_pdhg_set_state(self._h, int(precision),
                                                  *[_ptr(a, ctypes.c_double) for a in arrs]),
                      "sg_pdhg_set_state")

    def halpern_step(self, tau, sigma, k):
        """One reflected Halpern iteration (weight 1 / (k + 2) toward the anchor); T(z) lands in
        the average slots."""
        _native.check(self._lib.sg_pdhg_halpern_step(self._h, tau, sigma, k),
                      "sg_pdhg_halpern_step")

    def evaluate(self, which) -> np.ndarray:
        out = np.zeros(7)
        _native.check(self._lib.sg_pdhg_evaluate(self._h, which, _ptr(out, ctypes.c_double)),
                      "sg_pdhg_evaluate")
        return out

    def restart_distance(self, which):
        dv, dy = ctypes.c_double(0), ctypes.c_double(0)
        _native.check(self._lib.sg_pdhg_restart_distance(self._h, which, ctypes.byref(dv),
                                                         ctypes.byref(dy)),
                      "sg_pdhg_restart_distance")
        return dv.value, dy.value

    def restart_to(self, which):
        _native.check(self._lib.sg_pdhg_restart_to(self._h, which), "sg_pdhg_restart_to")

    def download(self):
        nt, m = self.n + self.m, max(self.m, 1)
        v, vn, ve = np.zeros(nt), np.zeros(nt), np.zeros(nt)
        y, yn, ye = np.zeros(m), np.zeros(m), np.zeros(m)
        _native.check(self._lib.sg_pdhg_download(self._h, *[_ptr(a, ctypes.c_double) for a in
                                                           (v, vn, y, yn, ve, ye)]),
                      "sg_pdhg_download")
        return dict(v=v, v_new=vn, y=y[:self.m], y_new=yn[:self.m], v_erg=ve, y_erg=ye[:self.m])

    def spmv(self, x, transpose=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(max(self.n if transpose else self.m, 1))
        _native.check(self._lib.sg_spmv(self._h, 1 if transpose else 0, _ptr(x, ctypes.c_double),
                                        _ptr(y, ctypes.c_double)), "sg_spmv")
        return y[:(self.n if transpose else self.m)]

    def close(self):
        if self._h:
            self._lib.sg_pdlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
