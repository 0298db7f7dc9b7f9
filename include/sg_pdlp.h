/* C ABI of the GB300 PDLP engine (samaya_gb300).
 *
 * Drop-in boundary for samaya's PDLP path. Every function is extern "C", takes plain pointers
 * and sizes, never throws and returns an int status: SG_OK (0) or a negative SG_ERR_* code.
 * Host buffers belong to the caller; device memory belongs to the engine handle. One handle is
 * used by one host thread at a time; distinct handles are independent.
 *
 * The problem is samaya's LpProblem (reference src/lp/simplex.hpp:18-26): the computational form
 *     min cost'v  s.t.  [A -I] v = 0,  lower <= v <= upper,  v = (x, r),
 * with A (m x n) in CSC form (int64 column starts, int32 row indices, float64 values) and
 * cost/lower/upper of n + m entries (infinite bounds as +-INFINITY). Solutions are returned in
 * the LpProblem's space, exactly as samaya::solve_pdlp returns them.
 */
#ifndef SG_PDLP_H
#define SG_PDLP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes of a solve: the values of samaya::SimplexStatus (reference
 * src/lp/simplex.hpp:28-35). */
enum {
  SG_STATUS_OPTIMAL = 0,
  SG_STATUS_INFEASIBLE = 1,
  SG_STATUS_UNBOUNDED = 2,
  SG_STATUS_ITERATION_LIMIT = 3,
  SG_STATUS_TIME_LIMIT = 4,
  SG_STATUS_NUMERICAL_ERROR = 5
};

/* Error codes returned by the functions. */
enum {
  SG_OK = 0,
  SG_ERR_INVALID_ARGUMENT = -1,
  SG_ERR_NO_DEVICE = -2,
  SG_ERR_CUDA = -3,
  SG_ERR_OUT_OF_MEMORY = -4,
  SG_ERR_TOO_LARGE = -5,
  SG_ERR_INTERNAL = -6,
  SG_ERR_NOT_READY = -7,
  SG_ERR_PARSE = -8,       /* MPS text that free MPS rejects (sg_mps.h) */
  SG_ERR_UNSUPPORTED = -9, /* valid MPS outside what the fast reader reads (sg_mps.h) */
  SG_ERR_IO = -10          /* a file that cannot be opened or read */
};

/* Precision of the iterations. */
enum {
  SG_PRECISION_FP64 = 0,         /* FP64 storage and arithmetic (the reference's precision) */
  SG_PRECISION_FP32_REFINED = 1, /* FP32 A and iterates, FP64 residuals + outer refinement */
  SG_PRECISION_FP32_THEN_FP64 = 2 /* FP32 PDLP to inner_tol, then FP64 PDLP from that point */
};

typedef struct sg_pdlp sg_pdlp;

/* Options: the fields of samaya::PdlpOptions (reference src/lp/pdlp.hpp:11-16) plus the
 * engine's own. */
typedef struct sg_pdlp_opts {
  double tol;                /* relative primal, dual and gap tolerance (default 1e-8) */
  long long max_iterations;  /* -1: automatic, max(1e4, 1e3 (m + n)), as the reference */
  double time_limit;         /* seconds; <= 0: none */
  int precision;             /* SG_PRECISION_* */
  int refine_max_rounds;     /* outer refinement rounds of the FP32 path (default 6) */
  double inner_tol;          /* tolerance of each FP32 solve or FP32 phase (default 1e-4) */
  int verbose;               /* 0 silent */
  int algorithm;             /* SG_ALGORITHM_* (default SG_ALGORITHM_REFERENCE) */
  int autotune;              /* 1 (default): time candidate tile shapes of each large operator
                                on the device at create, keyed by its row-length statistics
                                (cached per process); 0: the built-in rule */
  int tile_split;            /* built-in rule: medium rows (more than 128 nonzeros) longer than
                                this many nonzeros are summed by a team of 2-8 warps; 0
                                (default): one warp per row */
  double artificial_restart; /* a restart is forced once the iterations since the last one
                                reach this fraction of all iterations (0, default: 0.36, the
                                reference's, with SG_ALGORITHM_REFERENCE; 0.1 with ENHANCED
                                and HALPERN); values outside (0, 1) mean the default */
  int keep_inert_rows;       /* 0 (default): rows with no nonzeros whose logical has no cost
                                and 0 within its bounds are left out of the solves' step
                                launches (their dual and logical stay 0 in every iterate, so
                                the answer is the same bits); 1: every row is stepped */
  int row_groups;            /* dual steps over runs of rows whose k-th nonzeros lie in
                                neighbouring columns (see sg_pdlp_step_rows): 0 (default) the
                                tile tuner times them, 1 the built-in shape takes them, -1
                                never */
  int segment_staging;       /* 1: the dual steps stream the segments of rows longer than a
                                tile through shared memory by bulk copies (two chunks of 2,048
                                nonzeros in flight per CTA, completing on mbarriers); 0
                                (default): the threads load them directly (measured faster on
                                the power-law LP's long rows, which are bound by their
                                scattered gathers, not by the nonzero stream) */
  int tile_nnz;              /* built-in rule: nonzeros per tile (a power of two from 256 to
                                16384); 0 (default): about 8 tiles per SM */
} sg_pdlp_opts;

/* Algorithm variants. REFERENCE follows samaya's PDLP step for step (L2 Ruiz, fixed step
 * 0.99 / ||[A -I]||, primal weight 1 updated at restarts, the 0.2 / 0.8 / 0.36 restarts);
 * ENHANCED replaces the preconditioning by infinity-norm Ruiz + Pock-Chambolle (alpha = 1)
 * and starts the primal weight at |c| / |b|; everything else is the same. HALPERN is ENHANCED
 * with the reflected Halpern iteration z+ = lambda (2 T(z) - z) + (1 - lambda) z0 in place
 * of the running average (T the PDHG map, z0 the restart point, lambda = (k+1)/(k+2));
 * termination, restarts and the answer use T(z); no infeasibility / unboundedness checks.
 * The batched engine runs HALPERN requests as ENHANCED. */
enum {
  SG_ALGORITHM_REFERENCE = 0,
  SG_ALGORITHM_ENHANCED = 1,
  SG_ALGORITHM_HALPERN = 2
};

/* Result: the scalars of samaya::PdlpResult (reference src/lp/pdlp.hpp:19-30) plus counters. */
typedef struct sg_pdlp_result {
  int status;               /* SG_STATUS_* */
  long long iterations;     /* PDHG iterations (all refinement rounds for the FP32 path) */
  double primal_residual;   /* relative, as the reference defines them (pdlp.cpp:493-519) */
  double dual_residual;
  double gap;
  double primal_objective;  /* of the LpProblem (cost'v) at the answer */
  double dual_objective;
  long long restarts;
  long long evaluations;
  int refinement_rounds;
  int has_dual_ray;         /* a Farkas certificate was written (status infeasible) */
  int has_primal_ray;       /* an improving ray was written (status unbounded) */
  double setup_seconds;
  double solve_seconds;
  double step_size;         /* 0.99 / ||[A -I]|| estimate */
  double primal_weight;     /* final omega */
  long long kernel_launches;
  double device_ms;         /* CUDA-event time of the whole solve on the engine's stream */
} sg_pdlp_result;

/* Fills the defaults (tol 1e-8, automatic iteration limit, no time limit, FP64). */
void sg_pdlp_default_opts(sg_pdlp_opts* opts);

/* Whether a usable GB300 (sm_103) is present; writes its compute capability and name.
 * Replaces gpu::gpu_available / gpu::device_name (reference src/gpu/device.hpp:34-63) behind
 * samaya::gpu_info (src/gpu/info.cpp:12-19). Returns SG_OK or SG_ERR_NO_DEVICE. */
int sg_pdlp_available(int* cc_major, int* cc_minor, char* name, size_t name_len);

/* Uploads an LpProblem and prepares the engine. Replaces gpu::PdhgDevice::create (reference
 * src/gpu/pdhg_core.cu:242-273) for the solve_pdlp path: the matrix given here is the
 * LpProblem's A before PDLP's own equilibration, which the engine performs on the device. The
 * input is checked on the host first (SG_ERR_INVALID_ARGUMENT for decreasing column starts, a
 * row index out of range, a value or cost that is not finite, a NaN bound); the row-major
 * copy of A is then built on the device (a stable sort by row: the CSR sg_csc_to_csr gives).
 * Matrices with 2^31 - 1 or more nonzeros are refused (SG_ERR_TOO_LARGE), as the reference
 * refuses them (pdhg_core.cu:176-178). */
int sg_pdlp_create(sg_pdlp** handle, int m, int n, const int64_t* a_colptr,
                   const int32_t* a_rowidx, const double* a_val, const double* cost,
                   const double* lower, const double* upper, const sg_pdlp_opts* opts);

/* Runs PDLP: samaya::solve_pdlp (reference src/lp/pdlp.cpp:228-1193) with use_gpu. Writes x
 * (n + m), y (m), and when the status carries one the Farkas ray (m) or the improving ray (n);
 * any output pointer may be NULL. Deterministic: a re-run gives the same bits. */
int sg_pdlp_solve(sg_pdlp* handle, sg_pdlp_result* result, double* x, double* y,
                  double* dual_ray, double* primal_ray);

void sg_pdlp_destroy(sg_pdlp* handle);

/* Message of an error code, and the last error message of this thread. */
const char* sg_pdlp_error_string(int code);
const char* sg_pdlp_last_error(void);

/* One-call solve of an LpProblem (create + solve + destroy). */
int sg_pdlp_solve_problem(int m, int n, const int64_t* a_colptr, const int32_t* a_rowidx,
                          const double* a_val, const double* cost, const double* lower,
                          const double* upper, const sg_pdlp_opts* opts, sg_pdlp_result* result,
                          double* x, double* y, double* dual_ray, double* primal_ray);

/* ---- Inner seam: the counterpart of the reference's gpu::PdhgDevice
 * (src/gpu/pdhg_core.hpp:24-79), for kernel-level parity. The handle must come from
 * sg_pdhg_create, whose problem is used as already equilibrated. which: 0 current (v_new,
 * y_new), 1 average. Only theta = 1 (the reference's value) is supported. */
int sg_pdhg_create(sg_pdlp** handle, int m, int n, const int64_t* a_colptr,
                   const int32_t* a_rowidx, const double* a_val, const double* cost,
                   const double* lower, const double* upper);
/* PdhgDevice::set_original (pdhg_core.cu:307-318). */
int sg_pdhg_set_original(sg_pdlp* handle, const double* col_scale, const double* row_scale,
                         const double* cost, const double* lower, const double* upper);
/* PdhgDevice::step (pdhg_core.cu:275-292). */
int sg_pdhg_step(sg_pdlp* handle, double tau, double sigma, double theta, long long iter);
/* PdhgDevice::advance (pdhg_core.cu:294-299). */
int sg_pdhg_advance(sg_pdlp* handle);
/* PdhgDevice::evaluate (pdhg_core.cu:320-346): sums[7] = primal_sq, dual_sq, primal_obj,
 * dual_obj, x_sq, r_sq, y_sq. */
int sg_pdhg_evaluate(sg_pdlp* handle, int which, double* sums);
/* PdhgDevice::restart_distance (pdhg_core.cu:348-360). */
int sg_pdhg_restart_distance(sg_pdlp* handle, int which, double* dv_sq, double* dy_sq);
/* PdhgDevice::restart_to (pdhg_core.cu:362-380). */
int sg_pdhg_restart_to(sg_pdlp* handle, int which);
/* PdhgDevice::download (pdhg_core.cu:382-402); any pointer may be NULL. */
int sg_pdhg_download(sg_pdlp* handle, double* v, double* v_new, double* y, double* y_new,
                     double* v_erg, double* y_erg);

/* The device setup of a solve, read back: the equilibration factors (col_scale n, row_scale
 * m: the reference's ruiz_equilibration, src/lp/pdlp.cpp:109-187, for SG_ALGORITHM_REFERENCE),
 * the operator-norm estimate ||[A_eq -I]|| (estimate_operator_norm, pdlp.cpp:36-103) and the
 * step size eta = 0.99 / ||[A_eq -I]|| (pdlp.cpp:311-315). Any output may be NULL. Diagnostics
 * for parity tests; the next solve starts afresh. */
int sg_pdlp_equilibration(sg_pdlp* handle, double* col_scale, double* row_scale,
                          double* operator_norm, double* step_size);

/* Seam extensions with no counterpart in the reference (whose device path is FP64 PDHG with
 * averaging only), for step-level parity of the FP32 and Halpern kernels.
 * sg_pdhg_set_state sets the point the next single step starts from: v (n + m) and y (m) as
 * the current iterate, the extrapolated point equal to v (a first step, v_prev = v), the anchor
 * / restart point (v_anchor, y_anchor), averages zero. precision SG_PRECISION_FP64 keeps the
 * FP64 set; an FP32 precision (the handle must come from sg_pdlp_create with an FP32 precision)
 * rounds the uploaded problem values, cost, bounds and the given vectors to FP32, after which
 * sg_pdhg_step, sg_pdhg_halpern_step, sg_pdhg_evaluate (then in the given problem's own space,
 * unit scales), sg_pdhg_restart_to and sg_pdhg_download (widened to FP64) run the FP32
 * kernels. Call after sg_pdhg_set_original. */
int sg_pdhg_set_state(sg_pdlp* handle, int precision, const double* v, const double* y,
                      const double* v_anchor, const double* y_anchor);
/* One reflected Halpern iteration z+ = (2 T(z) - z) + (z0 - (2 T(z) - z)) / (k + 2) (T the PDHG
 * map in primal-first order, z0 the anchor, k iterations since the anchor), with the solve's
 * two launches; T(z) is written to the average slots (v_erg, y_erg of sg_pdhg_download). Call
 * sg_pdhg_advance after it, as after sg_pdhg_step. */
int sg_pdhg_halpern_step(sg_pdlp* handle, double tau, double sigma, long long k);

/* Device time of the engine's hot kernels, measured with CUDA events on the engine's own stream
 * after a solve: the average milliseconds of one dual step (rows of A), one primal step
 * (rows of A') and one evaluation pair, over `reps` launches each. Diagnostics for the
 * roofline report; the iterate is left unusable (the next solve starts afresh). */
int sg_pdlp_time_kernels(sg_pdlp* handle, int reps, double* ms_dual, double* ms_primal,
                         double* ms_eval);

/* The tile shape in use for A (transpose 0) or A' (transpose 1): nonzeros per tile, rows per
 * short-row tile, number of tiles, the step kernel variant (0 high occupancy, 1 deep unroll
 * of medium and long rows), and the nonzeros per warp above
 * which a medium row is summed by a team of warps (0: one warp per row). Diagnostics; set by
 * the autotuner or the built-in rule. */
int sg_pdlp_tile_shape(sg_pdlp* handle, int transpose, int* cap_nnz, int* cap_rows,
                       int* ntiles, int* variant, int* split);

/* The rows of A the solves' dual steps run over (m, unless inert rows are left out: see
 * sg_pdlp_opts.keep_inert_rows), the tiles over them, how many of those tiles are row groups
 * (runs of up to 32 rows whose k-th nonzeros lie in neighbouring columns, staged so that one
 * gather reads neighbouring entries) and whether the long rows' segments are streamed through
 * shared memory (1) or not (0); a tuned shape may choose either. Diagnostics. */
int sg_pdlp_step_rows(sg_pdlp* handle, int* rows, int* tiles, int* group_tiles, int* staged);

/* The engine's partition of a CSR operator (row starts row_ptr, rows + 1) into tiles for a tile
 * shape (nonzeros per tile, rows per short-row tile, warp-per-row threshold, team split; the
 * fields sg_pdlp_tile_shape reports): nine int32 per tile in `tiles` (first row, end row, first
 * nonzero, end nonzero, kind 0 short rows / 1 segment of a long row / 2 medium rows, warps per
 * medium row, segment, segments of the row, long-row id), *ntiles and *nlong (split rows) set;
 * SG_ERR_TOO_LARGE when more than max_tiles tiles (then *ntiles tells how many). No
 * counterpart in the reference (its SpMV has no tiles); host only, no GPU needed. */
int sg_build_tiles(int rows, const int32_t* row_ptr, int cap_nnz, int cap_rows, int warp_min,
                   int split, int32_t* tiles, int max_tiles, int* ntiles, int* nlong);

/* The dual steps' partition with row groups: as sg_build_tiles, plus kind 3, a run of 8-32
 * consecutive rows longer than warp_min, each a gather neighbour of the next (neighbours[r]
 * nonzero: rows r and r + 1; `rows` entries), cut into segments of nonzero positions within
 * the rows (for kind 3 the third and fourth fields are the first and end position, the ninth
 * the group's counter when it has several segments, counted in *nlong). Host only. */
int sg_build_group_tiles(int rows, const int32_t* row_ptr, const uint8_t* neighbours,
                         int cap_nnz, int cap_rows, int warp_min, int split, int32_t* tiles,
                         int max_tiles, int* ntiles, int* nlong);

/* CSC -> CSR of an m x n matrix (the engine's row-major copy of A): row starts csr_ptr (m + 1),
 * column indices csr_idx and values csr_val (a_colptr[n] each), every row's columns in
 * increasing order, the result the reference's SparseMatrix::transpose gives
 * (src/linalg/sparse_matrix.cpp:48-78). Checks the column starts, every row index and value;
 * SG_ERR_INVALID_ARGUMENT when one is out of range or not finite. Host only (up to 16
 * threads); no GPU needed. */
int sg_csc_to_csr(int m, int n, const int64_t* a_colptr, const int32_t* a_rowidx,
                  const double* a_val, int32_t* csr_ptr, int32_t* csr_idx, double* csr_val);

/* Model -> LpProblem: samaya's power-of-two scaling and computational form, as
 * compute_scaling + make_problem compute them (reference src/linalg/scaling.cpp:130-200,
 * src/lp/lp_solver.cpp:28-51). The model is min/max obj'x s.t. row_lower <= A x <= row_upper,
 * col_lower <= x <= col_upper with A in CSC form. Writes the scaled A (lp_colptr n + 1,
 * lp_rowidx/lp_val sized by the model's nonzeros; *lp_nnz set), cost/lower/upper (n + m) and
 * the scale factors (col n, row m). Host only; no GPU needed. SG_ERR_INVALID_ARGUMENT for
 * column starts that do not begin at 0 or decrease, a row index out of range, a matrix value or
 * cost that is not finite, or a NaN bound (the checks of sg_scale_model_device). */
int sg_scale_model(int m, int n, const int64_t* a_colptr, const int32_t* a_rowidx,
                   const double* a_val, const double* obj, const double* col_lower,
                   const double* col_upper, const double* row_lower, const double* row_upper,
                   int maximize, int64_t* lp_colptr, int32_t* lp_rowidx, double* lp_val,
                   double* cost, double* lower, double* upper, double* col_scale,
                   double* row_scale, int64_t* lp_nnz);

/* sg_scale_model computed on the GPU (the reference's compute_scaling + make_problem, src/
 * linalg/scaling.cpp:79-149, src/lp/lp_solver.cpp:28-51, restated as device kernels): the same
 * arguments and the same bits as sg_scale_model (the extremes are min / max, the factors the
 * same IEEE products, square roots and quotients; a factor whose nearest power of two turns on
 * the last bit of its logarithm is finished on the host by sg_scale_model's own rule). Needs a
 * GB300 (SG_ERR_NO_DEVICE otherwise); SG_ERR_INVALID_ARGUMENT for a row index out of range or
 * a value that is not finite. */
int sg_scale_model_device(int m, int n, const int64_t* a_colptr, const int32_t* a_rowidx,
                          const double* a_val, const double* obj, const double* col_lower,
                          const double* col_upper, const double* row_lower,
                          const double* row_upper, int maximize, int64_t* lp_colptr,
                          int32_t* lp_rowidx, double* lp_val, double* cost, double* lower,
                          double* upper, double* col_scale, double* row_scale, int64_t* lp_nnz);

/* An engine handle straight from a model: compute_scaling + make_problem and the CSC -> CSR
 * transpose of the engine's row-major copy (src/linalg/sparse_matrix.cpp:48-78) run on the GPU
 * on a single upload of the model, instead of on the host before sg_pdlp_create (samaya's
 * solve_pdlp_lp setup, src/core/solver.cpp:395-405, without its presolve). The handle's
 * problem is the model's LpProblem (the one sg_scale_model gives), so sg_pdlp_solve answers in
 * its space; col_scale (n) and row_scale (m), when not NULL, receive the factors that
 * sg_unscale_solution takes to map the answer back. */
int sg_pdlp_create_model(sg_pdlp** handle, int m, int n, const int64_t* a_colptr,
                         const int32_t* a_rowidx, const double* a_val, const double* obj,
                         const double* col_lower, const double* col_upper,
                         const double* row_lower, const double* row_upper, int maximize,
                         const sg_pdlp_opts* opts, double* col_scale, double* row_scale);

/* A PDLP answer (LpProblem space, x_lp n + m, y_lp m) back to the model, as samaya's
 * solve_pdlp_lp maps it (reference src/core/solver.cpp:415-432): column values x (n), row
 * activities (m), and row duals with the convention d = c - A'y (m). Any output may be NULL. */
int sg_unscale_solution(int m, int n, const double* col_scale, const double* row_scale,
                        int maximize, const double* x_lp, const double* y_lp, double* x,
                        double* row_activity, double* row_dual);

/* y = A x (transpose = 0, x: n, y: m) or y = A'x (transpose = 1) with the engine's
 * load-balanced tile kernel on the uploaded values; replaces gpu::csr_spmv (reference
 * src/gpu/spmv.cu:91-120) for the parity tests. */
int sg_spmv(sg_pdlp* handle, int transpose, const double* x, double* y);

/* ---- Batched PDLP: many LPs in one persistent launch (no counterpart in the reference, which
 * solves one LP at a time; each instance follows samaya::solve_pdlp's algorithm,
 * src/lp/pdlp.cpp:250-1193, with per-instance restarts and termination; infeasibility and
 * unboundedness detection are not run in the batch). Matrices (nmat of them, m_g x n_g, CSC)
 * are given concatenated: mat_colptr holds n_g + 1 local column starts per matrix, mat_rowidx
 * and mat_val the nonzeros of each matrix in turn. Instance i uses matrix inst_mat[i] (several
 * instances may share one: branch-and-bound node relaxations) and its own cost/lower/upper
 * (n_g + m_g each, concatenated in instance order). x (n_g + m_g per instance) and y (m_g per
 * instance) are returned concatenated in instance order. */
typedef struct sg_batch sg_batch;

typedef struct sg_batch_result {
  int status;              /* SG_STATUS_* */
  int pad;
  long long iterations;
  double primal_residual;  /* relative, as sg_pdlp_result */
  double dual_residual;
  double gap;
  double primal_objective;
  double dual_objective;
  long long restarts;
} sg_batch_result;

int sg_batch_create(sg_batch** handle, int nmat, const int* mat_m, const int* mat_n,
                    const int64_t* mat_colptr, const int32_t* mat_rowidx, const double* mat_val,
                    int count, const int* inst_mat, const double* cost, const double* lower,
                    const double* upper, const sg_pdlp_opts* opts);
/* Solves every instance; results[count]; x, y may be NULL; *device_ms (may be NULL) gets the
 * CUDA-event time of the launch. */
int sg_batch_solve(sg_batch* handle, sg_batch_result* results, double* x, double* y,
                   double* device_ms);
void sg_batch_destroy(sg_batch* handle);
const char* sg_batch_last_error(void);

/* ---- Differentiable layer (no counterpart in the reference, whose PDLP has no adjoint).
 * sg_batch_unroll runs, for every instance of an FP64 batch, `iterations` iterations of the
 * fixed-step PDHG of the reference's step rule (src/lp/pdlp.cpp:574-641) — tau = sigma =
 * 0.99 / ||[A_eq -I]||, primal weight 1, no restarts, no averaging — from zero on the
 * instance's equilibrated problem, saving the state every `checkpoint_every` iterations, and
 * writes v_K = (x_K, r_K) in the LpProblem's space to v_out (n_i + m_i doubles per instance,
 * in instance order; may be NULL). The map is piecewise linear in cost and bounds.
 * sg_batch_unroll_adjoint takes dL/dv_K in the same layout and writes dL/dcost, dL/dlower and
 * dL/dupper (same layout; the row entries of lower/upper are the row bounds) by the
 * transposed recurrences, recomputing each checkpointed segment. Returns SG_ERR_NOT_READY
 * before an unroll, SG_ERR_INVALID_ARGUMENT for an FP32 batch. */
int sg_batch_unroll(sg_batch* handle, int iterations, int checkpoint_every, double* v_out);
int sg_batch_unroll_adjoint(sg_batch* handle, const double* grad_v, double* grad_cost,
                            double* grad_lower, double* grad_upper);

/* ---- Allocation-free SpMV. This entry point has no counterpart in the reference: it is for
 * callers that cannot call cudaMalloc (a solver running under a memory pool or budget that
 * forbids driver allocations, or a plug-in whose device memory is handed out by another
 * runtime). It computes y = A x for A in CSR form (m rows, 32-bit row starts d_row_ptr[m + 1],
 * nnz = d_row_ptr[m] nonzeros) where every array is a DEVICE pointer owned by the caller, on
 * `stream` (a cudaStream_t; NULL for the default stream), and allocates nothing: its only
 * scratch is a file-scope device array of SG_SPMV_NOALLOC_MAX_CHUNKS carry records (16 bytes
 * each, 1 MiB) that every GPU loading the library holds until the process exits. `nnz` sizes
 * the launch and must equal d_row_ptr[m] (the kernels take the bounds from the device's
 * d_row_ptr[m], so a different count still writes every row, with a launch sized for it).
 * Matrices with more than SG_SPMV_NOALLOC_MAX_CHUNKS * 2048 nonzeros are refused with
 * SG_ERR_TOO_LARGE. The first call on a device looks the scratch's device address up (once per
 * device, with that device current); make that first call before any stream capture. A
 * cudaDeviceReset makes that address stale: do not call this entry point after one. All calls
 * share the scratch, so calls that overlap on the GPU (concurrent streams, or several host
 * threads) race; serialise them. Deterministic: a re-run gives the same bits. Returns SG_OK or
 * an SG_ERR_* code (message in sg_pdlp_last_error). */
#define SG_SPMV_NOALLOC_MAX_CHUNKS 65536
int sg_spmv_noalloc(int m, long long nnz, const int* d_row_ptr, const int* d_col_idx,
                    const double* d_val, const double* d_x, double* d_y, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SG_PDLP_H */
