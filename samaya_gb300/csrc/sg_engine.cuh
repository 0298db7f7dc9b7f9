// Host side of the GB300 PDLP engine: owns the device memory of one LP, runs the device setup,
// captures one chunk of the iteration loop (kCheckFrequency fused PDHG iterations + evaluation +
// decisions + restart + detection) as a CUDA graph and replays it until the device-side status
// word says done. No exception crosses this interface; errors are negative codes.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "sg_kernels.cuh"
#include "sg_refine.cuh"

namespace sg {

enum Error : int {
  kOk = 0,
  kErrInvalidArgument = -1,
  kErrNoDevice = -2,
  kErrCuda = -3,
  kErrOutOfMemory = -4,
  kErrTooLarge = -5,
  kErrInternal = -6,
  kErrNotReady = -7,
};

struct Options {
  double tol = 1e-8;
  long long max_iterations = -1;
  double time_limit = 0.0;  // seconds; <= 0: none
  int precision = 0;        // 0 FP64, 1 FP32 storage + FP64 refinement, 2 FP32 then FP64
  int refine_max_rounds = 6;
  double inner_tol = 1e-4;
  int verbose = 0;
  int algorithm = 0;        // 0 the reference's PDLP, 1 enhanced preconditioning + weight,
                            // 2 as 1 with the reflected Halpern iteration
  bool autotune = true;     // time candidate tile shapes of large operators at create
  int tile_split = 0;       // built-in rule's team split of medium rows (0: a warp per row)
  double artificial_restart = 0.0;  // forced-restart fraction (0: 0.36 reference, 0.1 others)
  bool skip_inert_rows = true;      // leave inert rows (see DevOp::act_rows) out of the solves
  int row_groups = 0;               // kind-3 row groups: 0 tuner decides, 1 built-in, -1 never
  int segment_staging = 0;          // staged kind-1 segments: 1 always, otherwise never
  int tile_nnz = 0;                 // built-in rule's nonzeros per tile (0: ~8 tiles per SM)
};

// Tile shape of an operator: nonzeros per tile (and per long-row segment), rows per short-row
// tile, and the row length above which a row gets a warp.
struct TileShape {
  int cap_nnz = kTileNnz;
  int cap_rows = kTileRows;
  int warp_min = kWarpRowMin;
  int variant = 0;          // step kernel variant (see sg_kernels.cu)
  int split = 0;            // kind-2 rows: nonzeros per warp of a team (0: a warp per row)
  int groups = 0;           // dual steps: runs of gather-neighbour rows as kind-3 row groups
  int staged = 0;           // dual steps: kind-1 segments streamed through shared memory
};

struct SolveInfo {
  int status = kNumericalError;
  long long iterations = 0;
  double rel_primal = 0, rel_dual = 0, rel_gap = 0;
  double primal_obj = 0, dual_obj = 0;
  long long restarts = 0, evaluations = 0;
  int refinement_rounds = 0;
  double setup_seconds = 0, solve_seconds = 0;
  double omega = 1, step_size = 0, operator_norm = 0;
  int has_dual_ray = 0, has_primal_ray = 0;
  long long graph_launches = 0;
  long long kernel_launches = 0;
  double device_ms = 0;
};

// A device operator by rows with its tiles.
struct DevOp {
  int rows = 0;
  int cols = 0;
  long long nnz = 0;
  int* ptr = nullptr;
  int* idx = nullptr;
  double* val = nullptr;       // working FP64 values (equilibrated after setup)
  double* val_orig = nullptr;  // values as given
  float* val32 = nullptr;      // FP32 copy for the mixed-precision path
  Tile* tiles = nullptr;
  int ntiles = 0;
  int nlong = 0;
  double* seg_part = nullptr;
  unsigned* lcount = nullptr;
  int cap_nnz = kTileNnz;
  int cap_rows = kTileRows;
  int warp_min = kWarpRowMin;
  int variant = 0;
  int split = 0;
  int groups = 0;
  int staged = 0;
  int uniform_len = 0;  // every row of exactly this many nonzeros (0: not uniform)
  int* wait_error = nullptr;  // the engine's bounded-wait flag (staged step sets)
  std::vector<int> host_ptr;
  // The rows the solves iterate over, when some rows are inert: an empty row whose logical has
  // no cost and 0 within its bounds keeps y_i = r_i = 0 in every iterate (every iterate starts
  // at 0, and its step only ever adds 0), so the solves' launches leave it out. act_list
  // (host, increasing) and act_rows (device) hold the other rows (a step-set tile's row index
  // v stands for act_rows[v]); act_rows null: every row is in.
  std::vector<int> act_list;
  int* act_rows = nullptr;
  // host_adj[i]: rows i and i + 1 are gather neighbours (their k-th nonzeros lie 1-4 columns
  // apart: sampled at 8 positions), the runs a shape with `groups` turns into kind-3 tiles.
  std::vector<char> host_adj;
  // The step set: the tiles the solves' dual steps run (over the active rows, with the row
  // groups), when it differs from the full set (step_set).
  bool step_set = false;
  Tile* st_tiles = nullptr;
  int st_ntiles = 0;
  int st_nlong = 0;
  int st_groups = 0;
  int st_staged = 0;
  double* st_seg_part = nullptr;
  double* st_grp_part = nullptr;
  unsigned* st_lcount = nullptr;

  TileSet tileset() const {
    TileSet t;
    t.tiles = tiles;
    t.ntiles = ntiles;
    t.nlong = nlong;
    t.seg_part = seg_part;
    t.lcount = lcount;
    t.cap_nnz = cap_nnz;
    t.cap_rows = cap_rows;
    t.variant = variant;
    t.rows = nullptr;
    t.groups = 0;
    t.grp_part = nullptr;
    t.uniform_len = uniform_len;
    t.staged = 0;
    t.wait_error = wait_error;
    return t;
  }
  TileSet step_tileset() const {
    if (!step_set) return tileset();
    TileSet t = tileset();
    t.tiles = st_tiles;
    t.ntiles = st_ntiles;
    t.nlong = st_nlong;
    t.seg_part = st_seg_part;
    t.lcount = st_lcount;
    t.rows = act_rows;
    t.groups = st_groups;
    t.grp_part = st_grp_part;
    t.staged = st_staged;
    return t;
  }
  int step_tiles() const { return step_set ? st_ntiles : ntiles; }
  OpView<double> view64() const { return OpView<double>{ptr, idx, val, rows, tileset()}; }
  OpView<float> view32() const { return OpView<float>{ptr, idx, val32, rows, tileset()}; }
  // The views of the solves' dual steps (evaluation, detection and the rest take the full set).
  OpView<double> step64() const { return OpView<double>{ptr, idx, val, rows, step_tileset()}; }
  OpView<float> step32() const { return OpView<float>{ptr, idx, val32, rows, step_tileset()}; }
};

// Iterate storage of one precision.
template <typename T>
struct DevIter {
  T* V[2] = {nullptr, nullptr};
  T* Vbar = nullptr;
  T* Y[2] = {nullptr, nullptr};
  T* Verg = nullptr;
  T* Yerg = nullptr;
  T* Vrst = nullptr;
  T* Yrst = nullptr;
  T* cost = nullptr;
  T* lower = nullptr;
  T* upper = nullptr;
  T* rhs = nullptr;
};

// An LpProblem already in device memory (built there by sg_setup_device.cu): A by rows (K) and
// by columns (the rows of K'), cost / lower / upper (n + m); the row starts also on the host
// (the tile partition is built on the host).
struct DeviceLp {
  int m = 0, n = 0;
  long long nnz = 0;
  const int* kptr = nullptr;
  const int* kidx = nullptr;
  const double* kval = nullptr;
  const int* tptr = nullptr;
  const int* tidx = nullptr;
  const double* tval = nullptr;
  const double* cost = nullptr;
  const double* lower = nullptr;
  const double* upper = nullptr;
  std::vector<int> kptr_host, tptr_host;
  std::vector<char> row_inert;  // m: empty row, no cost, 0 within its bounds (may be empty)
  bool x_uniform = false;  // every structural column has the bounds [x_lo, x_hi], 0 or infinite
  double x_lo = 0.0, x_hi = 0.0;
};

class Engine {
 public:
  ~Engine();

  // Builds both operators from an LpProblem in device memory (A by columns and by rows,
  // cost/lower/upper n + m; copied device to device, the caller keeps its buffers). The host
  // entry points (create_engine_from_lp, create_engine_from_model) build that problem.
  static int create_from_device(Engine** out, const DeviceLp& lp, const Options& opt,
                                std::string* err);

  // Full PDLP solve (setup on the device, graph-replayed iterations). Outputs in the
  // LpProblem's space: x (n + m), y (m), dual_ray (m), primal_ray (n); any may be null.
  int solve(SolveInfo* info, double* x, double* y, double* dual_ray, double* primal_ray,
            std::string* err);

  // Inner GPU seam, the counterpart of the reference's gpu::PdhgDevice (pdhg_core.hpp:24-79):
  // the problem given is already equilibrated; the host drives single steps.
  int seam_set_original(const double* cs, const double* rs, const double* cost,
                        const double* lower, const double* upper);
  int seam_step(double tau, double sigma, long long iter);
  int seam_advance();
  int seam_evaluate(int which, double* sums7);
  int seam_restart_distance(int which, double* dv, double* dy);
  int seam_restart_to(int which);
  int seam_download(double* v, double* v_new, double* y, double* y_new, double* v_erg,
                    double* y_erg);
  // Seam extensions with no counterpart in the reference: the storage precision and iterate
  // state the single steps start from (current point, anchor), and one reflected Halpern
  // iteration, so that the FP32 step kernels and the Halpern kernels are checked step by step.
  int seam_set_state(int precision, const double* v, const double* y, const double* v0,
                     const double* y0);
  int seam_halpern_step(double tau, double sigma, long long k);
  // The device setup of a solve (equilibration, operator-norm estimate, step size), read
  // back: col_scale (n), row_scale (m), ||[A_eq -I]|| and eta. Any output may be null.
  int equilibration(double* col_scale, double* row_scale, double* op_norm, double* step_size);
  // y = K x (rows of A) or y = K' x through the tile kernel (FP64).
  int spmv(int transpose, const double* x, double* y);
  // Average device milliseconds of the step kernels and the evaluation (CUDA events).
  int time_kernels(int reps, double* ms_dual, double* ms_primal, double* ms_eval);
  int tile_capacity(int transpose) const { return transpose ? Kt_.cap_nnz : K_.cap_nnz; }
  // The rows of A the solves' dual steps run over, their tiles, and the row-group tiles.
  int step_rows(int* rows, int* tiles, int* group_tiles, int* staged) const {
    *rows = K_.act_rows != nullptr ? static_cast<int>(K_.act_list.size()) : m_;
    *tiles = K_.step_tiles();
    *group_tiles = K_.step_set ? K_.st_groups : 0;
    *staged = K_.step_set ? K_.st_staged : 0;
    return kOk;
  }
  int tile_shape(int transpose, int* cap_nnz, int* cap_rows, int* ntiles, int* variant,
                 int* split) const {
    const DevOp& op = transpose ? Kt_ : K_;
    *cap_nnz = op.cap_nnz;
    *cap_rows = op.cap_rows;
    *ntiles = op.ntiles;
    *variant = op.variant;
    *split = op.split;
    return 0;
  }
  bool fp32() const { return fp32_; }

  int m() const { return m_; }
  int n() const { return n_; }
  long long nnz() const { return nnz_; }

 private:
  Engine() = default;
  int alloc_all(std::string* err);
  int setup_device(const double* rhs_orig);
  int capture_chunk();
  template <typename T>
  IterView<T> iter_view(DevIter<T>& it);
  EvalView eval_view() const;
  RedView red_view() const;
  int run_loop(double deadline_s, SolveInfo* info, cudaGraphExec_t exec, Ctl* ctl,
               int kernels_per_chunk, long long max_iter);
  int capture_chunk32();
  long long max_iterations() const;
  IterView<double> master_view();
  EvalView inner_eval_view() const;
  int solve_fp64(SolveInfo* info, double* x, double* y, double* dual_ray, double* primal_ray);
  int solve_refined(SolveInfo* info, double* x, double* y, double* dual_ray, double* primal_ray);
  int solve_switched(SolveInfo* info, double* x, double* y, double* dual_ray, double* primal_ray);
  int prepare_fp32();
  IrView ir_view();
  int finish_fp64(SolveInfo* info, double t0, long long iterations_before, double* x, double* y,
                  double* dual_ray, double* primal_ray);
  void enqueue_chunk_body();
  int check(cudaError_t e, const char* what);
  TileShape default_shape(const DevOp& op) const;
  int set_tiles(DevOp* op, const TileShape& shape);
  int set_active_rows(const std::vector<char>& inert, std::string* err);
  // The seam's dual steps: the solves' tiles (row groups included) unless inert rows are left
  // out of them (a seam state may give those rows any value), else every row.
  bool seam_step_set() const { return K_.step_set && K_.act_rows == nullptr; }
  OpView<double> seam_dual64() const { return seam_step_set() ? K_.step64() : K_.view64(); }
  OpView<float> seam_dual32() const { return seam_step_set() ? K_.step32() : K_.view32(); }
  int seam_grid_k() const { return seam_step_set() ? grid_step_k_ : grid_full_k_; }
  int find_neighbours(std::string* err);
  int tune_tiles(std::string* err);
  double time_step_kernel(bool dual, int reps);

  int m_ = 0, n_ = 0;
  long long nnz_ = 0;
  Options opt_;
  int* wait_error_ = nullptr;  // device: a staged segment's bounded wait gave up
  int check_wait_error(std::string* err);
  // grid_step_k_: the dual steps of the solves (active rows); grid_full_k_: every row.
  int grid_k_ = 1, grid_t_ = 1, grid_step_k_ = 1, grid_step_t_ = 1, grid_full_k_ = 1;
  int sm_count_ = 148;
  bool fp32_ = false;
  bool switch_ = false;   // FP32 PDLP, then FP64 PDLP from its answer
  bool x_bounds_uniform_ = false;  // every structural column has the bounds [x_lo_, x_hi_]
  double x_lo_ = 0.0, x_hi_ = 0.0;
  DevOp K_, Kt_;
  DevIter<double> it64_;
  DevIter<float> it32_;
  // FP64 problem data.
  double* cost_orig_ = nullptr;   // n + m, as given (LpProblem space)
  double* lower_orig_ = nullptr;
  double* upper_orig_ = nullptr;
  double* cost_ev_ = nullptr;     // evaluation copies (the problem the iterations solve)
  double* lower_ev_ = nullptr;
  double* upper_ev_ = nullptr;
  double* rhs_ev_ = nullptr;      // m, null when zero
  double* cs_ = nullptr;
  double* rs_ = nullptr;
  double* inv_cs_ = nullptr;      // 1 / cs_, 1 / rs_ (the evaluation's multipliers)
  double* inv_rs_ = nullptr;
  double* cn_ = nullptr;
  double* rn_ = nullptr;
  double* pu_ = nullptr;          // power iteration vectors
  double* pv_ = nullptr;
  double* u0_ = nullptr;          // power iteration start (mt19937_64(12345) uniform(-1, 1))
  double* scratch_n_ = nullptr;
  double* x_out_ = nullptr;
  double* y_out_ = nullptr;
  double* ray_out_ = nullptr;
  double* partial_ = nullptr;
  unsigned* counter_ = nullptr;
  double* long_terms_ = nullptr;
  Ctl* ctl_ = nullptr;
  // One device allocation holding every buffer whose size the problem fixes (operators,
  // iterates, problem vectors, control blocks): one cudaMalloc and one cudaFree per engine.
  char* arena_ = nullptr;
  size_t arena_bytes_ = 0;
  Ctl* ctl_host_ = nullptr;       // pinned
  cudaStream_t stream_ = nullptr;
  cudaGraphExec_t chunk_exec_ = nullptr;
  cudaGraph_t chunk_graph_ = nullptr;
  int chunk_kernels_ = 0;
  long long seam_steps_ = 0;
  bool seam_mode_ = false;
  bool seam_fp32_ = false;   // the seam's steps, evaluation and download use the FP32 set
  int seam_ctl_write(double tau, double sigma, long long t, long long k, long long max_iter);
  int seam_eval_launch();
  cudaEvent_t ev_[4] = {nullptr, nullptr, nullptr, nullptr};
  // Mixed-precision path: the inner solves' control block and graph, the correction problem
  // (FP64 evaluation copy), unit scales for its evaluation, and the residual vectors.
  Ctl* ctl32_ = nullptr;
  cudaGraphExec_t chunk32_exec_ = nullptr;
  cudaGraph_t chunk32_graph_ = nullptr;
  int chunk32_kernels_ = 0;
  double* ones_n_ = nullptr;
  double* ones_m_ = nullptr;
  double* cost_in_ = nullptr;
  double* lower_in_ = nullptr;
  double* upper_in_ = nullptr;
  double* rhs_in_ = nullptr;
  double* bh_ = nullptr;
  double* dvec_ = nullptr;
};

// Builds the tile partition of a CSR operator (host). Exposed for the CPU tests.
// With adj (adj[r]: rows r and r + 1 are gather neighbours) and group_pos > 0, runs of 8-32
// neighbouring rows longer than warp_min become kind-3 row groups of group_pos positions per
// segment.
void build_tiles(const std::vector<int>& ptr, int tile_nnz, int tile_rows, int warp_min,
                 int split, std::vector<Tile>* out, int* nlong,
                 const std::vector<char>* adj = nullptr, int group_pos = 0);
// Positions per segment of a kind-3 row group for a tile capacity.
int group_positions(int cap_nnz);

// Device facts for sg_pdlp_available.
int device_info(int* major, int* minor, char* name, size_t len);

}  // namespace sg
