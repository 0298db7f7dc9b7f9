// extern "C" entry points of the GB300 PDLP engine (include/sg_pdlp.h). No exception crosses
// this layer: every error becomes a negative code plus a thread-local message.
#include <math.h>
#include <string.h>

#include <exception>
#include <new>
#include <string>
#include <vector>

#include "../../include/sg_mps.h"
#include "../../include/sg_pdlp.h"
#include "sg_engine.cuh"
#include "sg_mps.h"
#include "sg_setup_device.cuh"

struct sg_pdlp {
  sg::Engine* engine = nullptr;
};

struct sg_mps {
  sg::MpsModel model;
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& message) {
  g_last_error = message;
  return code;
}

// The C status of a read; the handle goes to *out on success and is freed otherwise.
int mps_result(sg::MpsStatus st, const sg::MpsError& e, sg_mps* h, sg_mps** out) {
  if (st == sg::MpsStatus::kOk) {
    *out = h;
    return SG_OK;
  }
  delete h;
  const std::string msg = e.line > 0 ? "line " + std::to_string(e.line) + ": " + e.message
                                     : e.message;
  switch (st) {
    case sg::MpsStatus::kParseError: return fail(SG_ERR_PARSE, msg);
    case sg::MpsStatus::kUnsupported: return fail(SG_ERR_UNSUPPORTED, msg);
    case sg::MpsStatus::kIoError: return fail(SG_ERR_IO, msg);
    case sg::MpsStatus::kTooLarge: return fail(SG_ERR_TOO_LARGE, msg);
    case sg::MpsStatus::kOutOfMemory: return fail(SG_ERR_OUT_OF_MEMORY, msg);
    default: return fail(SG_ERR_INTERNAL, msg);
  }
}

template <class V, class T>
void copy_out(const V& v, T* dst) {
  if (dst != nullptr && !v.empty()) memcpy(dst, v.data(), v.size() * sizeof(T));
}

sg::Options to_options(const sg_pdlp_opts* o) {
  sg::Options opt;
  sg_pdlp_opts d;
  sg_pdlp_default_opts(&d);
  if (o == nullptr) o = &d;
  opt.tol = o->tol > 0 ? o->tol : 1e-8;
  opt.max_iterations = o->max_iterations;
  opt.time_limit = o->time_limit;
  opt.precision = o->precision;
  opt.refine_max_rounds = o->refine_max_rounds > 0 ? o->refine_max_rounds : 6;
  opt.inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-4;
  opt.verbose = o->verbose;
  opt.algorithm = o->algorithm == SG_ALGORITHM_ENHANCED  ? 1
                  : o->algorithm == SG_ALGORITHM_HALPERN ? 2
                                                         : 0;
  opt.autotune = o->autotune != 0;
  opt.tile_split = o->tile_split > 0 ? o->tile_split : 0;
  opt.artificial_restart =
      o->artificial_restart > 0 && o->artificial_restart < 1 ? o->artificial_restart : 0.0;
  opt.skip_inert_rows = o->keep_inert_rows == 0;
  opt.row_groups = o->row_groups > 0 ? 1 : (o->row_groups < 0 ? -1 : 0);
  opt.segment_staging = o->segment_staging > 0 ? 1 : -1;
  opt.tile_nnz = 0;
  for (int c = 256; c <= 4 * sg::kTileNnz; c *= 2) {
    if (o->tile_nnz == c) opt.tile_nnz = c;
  }
  return opt;
}

// The tile partition as nine int32 per tile (sg_build_tiles, sg_build_group_tiles).
int build_tiles_c(int rows, const int32_t* row_ptr, const uint8_t* neighbours, int cap_nnz,
                  int cap_rows, int warp_min, int split, int32_t* tiles, int max_tiles,
                  int* ntiles, int* nlong) {
  if (rows < 0 || row_ptr == nullptr || ntiles == nullptr || nlong == nullptr ||
      cap_nnz < 1 || cap_rows < 1 || warp_min < 0 || split < 0 || max_tiles < 0 ||
      (max_tiles > 0 && tiles == nullptr)) {
    return SG_ERR_INVALID_ARGUMENT;
  }
  try {
    std::vector<int> ptr(row_ptr, row_ptr + rows + 1);
    for (int r = 0; r < rows; ++r) {
      if (ptr[r + 1] < ptr[r]) return SG_ERR_INVALID_ARGUMENT;
    }
    std::vector<char> adj;
    if (neighbours != nullptr) adj.assign(neighbours, neighbours + rows);
    std::vector<sg::Tile> out;
    int nl = 0;
    sg::build_tiles(ptr, cap_nnz, cap_rows, warp_min, split, &out, &nl,
                    neighbours != nullptr ? &adj : nullptr,
                    neighbours != nullptr ? sg::group_positions(cap_nnz) : 0);
    *ntiles = static_cast<int>(out.size());
    *nlong = nl;
    if (static_cast<int>(out.size()) > max_tiles) return SG_ERR_TOO_LARGE;
    for (size_t i = 0; i < out.size(); ++i) {
      const sg::Tile& t = out[i];
      int32_t* o = tiles + 9 * i;
      o[0] = t.r0;
      o[1] = t.r1;
      o[2] = t.k0;
      o[3] = t.k1;
      o[4] = t.kind;
      o[5] = t.team;
      o[6] = t.seg;
      o[7] = t.nseg;
      o[8] = t.lrow;
    }
    return SG_OK;
  } catch (...) {
    return SG_ERR_INTERNAL;
  }
}

}  // namespace

namespace sg {

// The thread's last-error text, for entry points outside this file.
void set_last_error(const char* message) { g_last_error = message ? message : ""; }

}  // namespace sg

extern "C" {

void sg_pdlp_default_opts(sg_pdlp_opts* opts) {
  if (opts == nullptr) return;
  memset(opts, 0, sizeof(*opts));
  opts->tol = 1e-8;
  opts->max_iterations = -1;
  opts->time_limit = 0.0;
  opts->precision = SG_PRECISION_FP64;
  opts->refine_max_rounds = 6;
  opts->inner_tol = 1e-4;
  opts->verbose = 0;
  opts->autotune = 1;
  opts->tile_split = 0;
}

int sg_pdlp_available(int* cc_major, int* cc_minor, char* name, size_t name_len) {
  try {
    const int rc = sg::device_info(cc_major, cc_minor, name, name_len);
    if (rc != sg::kOk) return fail(SG_ERR_NO_DEVICE, "no usable sm_103 GPU");
    return SG_OK;
  } catch (...) {
    return fail(SG_ERR_INTERNAL, "unexpected exception");
  }
}

int sg_pdlp_create(sg_pdlp** handle, int m, int n, const int64_t* a_colptr,
                   const int32_t* a_rowidx, const double* a_val, const double* cost,
                   const double* lower, const double* upper, const sg_pdlp_opts* opts) {
  if (handle == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "handle is NULL");
  *handle = nullptr;
  try {
    std::string why;
    sg::Engine* e = nullptr;
    const int rc = sg::create_engine_from_lp(&e, m, n, a_colptr, a_rowidx, a_val, cost, lower,
                                             upper, to_options(opts), &why);
    if (rc != sg::kOk) return fail(rc, why);
    *handle = new sg_pdlp{e};
    return SG_OK;
  } catch (const std::bad_alloc&) {
    return fail(SG_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (const std::exception& ex) {
    return fail(SG_ERR_INTERNAL, ex.what());
  } catch (...) {
    return fail(SG_ERR_INTERNAL, "unexpected exception");
  }
}

int sg_pdlp_create_model(sg_pdlp** handle, int m, int n, const int64_t* a_colptr,
                         const int32_t* a_rowidx, const double* a_val, const double* obj,
                         const double* col_lower, const double* col_upper,
                         const double* row_lower, const double* row_upper, int maximize,
                         const sg_pdlp_opts* opts, double* col_scale, double* row_scale) {
  if (handle == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "handle is NULL");
  *handle = nullptr;
  try {
    sg::ModelView mv;
    mv.m = m;
    mv.n = n;
    mv.colptr = a_colptr;
    mv.rowidx = a_rowidx;
    mv.val = a_val;
    mv.obj = obj;
    mv.col_lower = col_lower;
    mv.col_upper = col_upper;
    mv.row_lower = row_lower;
    mv.row_upper = row_upper;
    mv.maximize = maximize;
    std::string why;
    sg::Engine* e = nullptr;
    const int rc = sg::create_engine_from_model(&e, mv, to_options(opts), col_scale, row_scale,
                                                &why);
    if (rc != sg::kOk) return fail(rc, why);
    *handle = new sg_pdlp{e};
    return SG_OK;
  } catch (const std::bad_alloc&) {
    return fail(SG_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (const std::exception& ex) {
    return fail(SG_ERR_INTERNAL, ex.what());
  } catch (...) {
    return fail(SG_ERR_INTERNAL, "unexpected exception");
  }
}

int sg_scale_model_device(int m, int n, const int64_t* a_colptr, const int32_t* a_rowidx,
                          const double* a_val, const double* obj, const double* col_lower,
                          const double* col_upper, const double* row_lower,
                          const double* row_upper, int maximize, int64_t* lp_colptr,
                          int32_t* lp_rowidx, double* lp_val, double* cost, double* lower,
                          double* upper, double* col_scale, double* row_scale, int64_t* lp_nnz) {
  try {
    sg::ModelView mv;
    mv.m = m;
    mv.n = n;
    mv.colptr = a_colptr;
    mv.rowidx = a_rowidx;
    mv.val = a_val;
    mv.obj = obj;
    mv.col_lower = col_lower;
    mv.col_upper = col_upper;
    mv.row_lower = row_lower;
    mv.row_upper = row_upper;
    mv.maximize = maximize;
    std::string why;
    const int rc = sg::scale_model_device(mv, lp_colptr, lp_rowidx, lp_val, cost, lower, upper,
                                          col_scale, row_scale, lp_nnz, &why);
    if (rc != sg::kOk) return fail(rc, why);
    return SG_OK;
  } catch (const std::bad_alloc&) {
    return fail(SG_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (...) {
    return fail(SG_ERR_INTERNAL, "unexpected exception");
  }
}

int sg_pdlp_solve(sg_pdlp* handle, sg_pdlp_result* result, double* x, double* y,
                  double* dual_ray, double* primal_ray) {
  if (handle == nullptr || handle->engine == nullptr || result == nullptr) {
    return fail(SG_ERR_INVALID_ARGUMENT, "NULL handle or result");
  }
  try {
    memset(result, 0, sizeof(*result));
    sg::SolveInfo info;
    std::string why;
    const int rc = handle->engine->solve(&info, x, y, dual_ray, primal_ray, &why);
    if (rc != sg::kOk) {
      result->status = SG_STATUS_NUMERICAL_ERROR;
      return fail(rc, why);
    }
    result->status = info.status;
    result->iterations = info.iterations;
    result->primal_residual = info.rel_primal;
    result->dual_residual = info.rel_dual;
    result->gap = info.rel_gap;
    result->primal_objective = info.primal_obj;
    result->dual_objective = info.dual_obj;
    result->restarts = info.restarts;
    result->evaluations = info.evaluations;
    result->refinement_rounds = info.refinement_rounds;
    result->has_dual_ray = info.has_dual_ray;
    result->has_primal_ray = info.has_primal_ray;
    result->setup_seconds = info.setup_seconds;
    result->solve_seconds = info.solve_seconds;
    result->step_size = info.step_size;
    result->primal_weight = info.omega;
    result->kernel_launches = info.kernel_launches;
    result->device_ms = info.device_ms;
    return SG_OK;
  } catch (const std::bad_alloc&) {
    return fail(SG_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (const std::exception& ex) {
    return fail(SG_ERR_INTERNAL, ex.what());
  } catch (...) {
    return fail(SG_ERR_INTERNAL, "unexpected exception");
  }
}

void sg_pdlp_destroy(sg_pdlp* handle) {
  if (handle == nullptr) return;
  try {
    delete handle->engine;
  } catch (...) {
  }
  delete handle;
}

const char* sg_pdlp_error_string(int code) {
  switch (code) {
    case SG_OK: return "ok";
    case SG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SG_ERR_NO_DEVICE: return "no usable GPU";
    case SG_ERR_CUDA: return "CUDA error";
    case SG_ERR_OUT_OF_MEMORY: return "out of memory";
    case SG_ERR_TOO_LARGE: return "problem too large for 32-bit offsets";
    case SG_ERR_INTERNAL: return "internal error";
    case SG_ERR_NOT_READY: return "handle not ready for this call";
    case SG_ERR_PARSE: return "not valid free MPS";
    case SG_ERR_UNSUPPORTED: return "outside what the fast MPS reader reads";
    case SG_ERR_IO: return "file cannot be read";
    default: return "unknown error";
  }
}

const char* sg_pdlp_last_error(void) { return g_last_error.c_str(); }

int sg_pdlp_solve_problem(int m, int n, const int64_t* a_colptr, const int32_t* a_rowidx,
                          const double* a_val, const double* cost, const double* lower,
                          const double* upper, const sg_pdlp_opts* opts, sg_pdlp_result* result,
                          double* x, double* y, double* dual_ray, double* primal_ray) {
  sg_pdlp* h = nullptr;
  int rc = sg_pdlp_create(&h, m, n, a_colptr, a_rowidx, a_val, cost, lower, upper, opts);
  if (rc != SG_OK) return rc;
  rc = sg_pdlp_solve(h, result, x, y, dual_ray, primal_ray);
  sg_pdlp_destroy(h);
  return rc;
}

int sg_pdhg_create(sg_pdlp** handle, int m, int n, const int64_t* a_colptr,
                   const int32_t* a_rowidx, const double* a_val, const double* cost,
                   const double* lower, const double* upper) {
  sg_pdlp_opts o;
  sg_pdlp_default_opts(&o);
  return sg_pdlp_create(handle, m, n, a_colptr, a_rowidx, a_val, cost, lower, upper, &o);
}

#define SG_SEAM(call)                                                        \
  do {                                                                       \
    if (handle == nullptr || handle->engine == nullptr)                      \
      return fail(SG_ERR_INVALID_ARGUMENT, "NULL handle");                   \
    try {                                                                    \
      const int rc_ = (call);                                                \
      if (rc_ != sg::kOk) return fail(rc_, sg_pdlp_error_string(rc_));       \
      return SG_OK;                                                          \
    } catch (...) {                                                          \
      return fail(SG_ERR_INTERNAL, "unexpected exception");                  \
    }                                                                        \
  } while (0)

int sg_pdhg_set_original(sg_pdlp* handle, const double* col_scale, const double* row_scale,
                         const double* cost, const double* lower, const double* upper) {
  SG_SEAM(handle->engine->seam_set_original(col_scale, row_scale, cost, lower, upper));
}

int sg_pdhg_step(sg_pdlp* handle, double tau, double sigma, double theta, long long iter) {
  if (theta != 1.0) return fail(SG_ERR_INVALID_ARGUMENT, "only theta = 1 is supported");
  SG_SEAM(handle->engine->seam_step(tau, sigma, iter));
}

int sg_pdhg_advance(sg_pdlp* handle) { SG_SEAM(handle->engine->seam_advance()); }

int sg_pdhg_evaluate(sg_pdlp* handle, int which, double* sums) {
  if (sums == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "sums is NULL");
  SG_SEAM(handle->engine->seam_evaluate(which, sums));
}

int sg_pdhg_restart_distance(sg_pdlp* handle, int which, double* dv_sq, double* dy_sq) {
  if (dv_sq == nullptr || dy_sq == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "NULL output");
  SG_SEAM(handle->engine->seam_restart_distance(which, dv_sq, dy_sq));
}

int sg_pdhg_restart_to(sg_pdlp* handle, int which) {
  SG_SEAM(handle->engine->seam_restart_to(which));
}

int sg_pdhg_download(sg_pdlp* handle, double* v, double* v_new, double* y, double* y_new,
                     double* v_erg, double* y_erg) {
  SG_SEAM(handle->engine->seam_download(v, v_new, y, y_new, v_erg, y_erg));
}

int sg_pdlp_equilibration(sg_pdlp* handle, double* col_scale, double* row_scale,
                          double* operator_norm, double* step_size) {
  SG_SEAM(handle->engine->equilibration(col_scale, row_scale, operator_norm, step_size));
}

int sg_pdhg_set_state(sg_pdlp* handle, int precision, const double* v, const double* y,
                      const double* v_anchor, const double* y_anchor) {
  if (precision != SG_PRECISION_FP64 && precision != SG_PRECISION_FP32_REFINED &&
      precision != SG_PRECISION_FP32_THEN_FP64) {
    return fail(SG_ERR_INVALID_ARGUMENT, "unknown precision");
  }
  SG_SEAM(handle->engine->seam_set_state(precision, v, y, v_anchor, y_anchor));
}

int sg_pdhg_halpern_step(sg_pdlp* handle, double tau, double sigma, long long k) {
  SG_SEAM(handle->engine->seam_halpern_step(tau, sigma, k));
}

int sg_pdlp_time_kernels(sg_pdlp* handle, int reps, double* ms_dual, double* ms_primal,
                         double* ms_eval) {
  if (ms_dual == nullptr || ms_primal == nullptr || ms_eval == nullptr || reps <= 0) {
    return fail(SG_ERR_INVALID_ARGUMENT, "bad arguments");
  }
  SG_SEAM(handle->engine->time_kernels(reps, ms_dual, ms_primal, ms_eval));
}

int sg_pdlp_tile_shape(sg_pdlp* handle, int transpose, int* cap_nnz, int* cap_rows,
                       int* ntiles, int* variant, int* split) {
  if (cap_nnz == nullptr || cap_rows == nullptr || ntiles == nullptr || variant == nullptr ||
      split == nullptr) {
    return fail(SG_ERR_INVALID_ARGUMENT, "NULL output");
  }
  SG_SEAM(handle->engine->tile_shape(transpose, cap_nnz, cap_rows, ntiles, variant, split));
}

int sg_pdlp_step_rows(sg_pdlp* handle, int* rows, int* tiles, int* group_tiles, int* staged) {
  if (rows == nullptr || tiles == nullptr || group_tiles == nullptr || staged == nullptr) {
    return fail(SG_ERR_INVALID_ARGUMENT, "NULL output");
  }
  SG_SEAM(handle->engine->step_rows(rows, tiles, group_tiles, staged));
}

int sg_build_tiles(int rows, const int32_t* row_ptr, int cap_nnz, int cap_rows, int warp_min,
                   int split, int32_t* tiles, int max_tiles, int* ntiles, int* nlong) {
  return build_tiles_c(rows, row_ptr, nullptr, cap_nnz, cap_rows, warp_min, split, tiles,
                       max_tiles, ntiles, nlong);
}

int sg_build_group_tiles(int rows, const int32_t* row_ptr, const uint8_t* neighbours,
                         int cap_nnz, int cap_rows, int warp_min, int split, int32_t* tiles,
                         int max_tiles, int* ntiles, int* nlong) {
  if (neighbours == nullptr) return SG_ERR_INVALID_ARGUMENT;
  return build_tiles_c(rows, row_ptr, neighbours, cap_nnz, cap_rows, warp_min, split, tiles,
                       max_tiles, ntiles, nlong);
}

int sg_spmv(sg_pdlp* handle, int transpose, const double* x, double* y) {
  if (x == nullptr || y == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "NULL vector");
  SG_SEAM(handle->engine->spmv(transpose, x, y));
}

// ---- the fast MPS reader (include/sg_mps.h) ----

int sg_mps_read(const char* path, int threads, sg_mps** out) {
  if (out == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "NULL output");
  *out = nullptr;
  if (path == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "path is NULL");
  sg_mps* h = new (std::nothrow) sg_mps;
  if (h == nullptr) return fail(SG_ERR_OUT_OF_MEMORY, "out of host memory");
  sg::MpsError e;
  return mps_result(sg::read_mps_file(path, threads, &h->model, &e), e, h, out);
}

int sg_mps_read_text(const char* text, size_t len, int threads, sg_mps** out) {
  if (out == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "NULL output");
  *out = nullptr;
  if (text == nullptr && len > 0) return fail(SG_ERR_INVALID_ARGUMENT, "text is NULL");
  sg_mps* h = new (std::nothrow) sg_mps;
  if (h == nullptr) return fail(SG_ERR_OUT_OF_MEMORY, "out of host memory");
  sg::MpsError e;
  return mps_result(sg::read_mps_text(text, len, threads, &h->model, &e), e, h, out);
}

int sg_mps_get_info(const sg_mps* h, sg_mps_info* info) {
  if (h == nullptr || info == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "NULL argument");
  const sg::MpsModel& md = h->model;
  info->m = md.m;
  info->n = md.n;
  info->nnz = static_cast<int64_t>(md.vals.size());
  info->maximize = md.maximize ? 1 : 0;
  int32_t k = 0;
  for (const uint8_t v : md.col_integer) k += v ? 1 : 0;
  info->num_integers = k;
  info->obj_offset = md.obj_offset;
  info->name_bytes = static_cast<int64_t>(md.name.size());
  info->row_name_bytes = static_cast<int64_t>(md.row_names.size());
  info->col_name_bytes = static_cast<int64_t>(md.col_names.size());
  return SG_OK;
}

int sg_mps_get_model(const sg_mps* h, int64_t* colptr, int32_t* rowidx, double* vals,
                     double* obj, double* col_lower, double* col_upper, uint8_t* col_integer,
                     double* row_lower, double* row_upper) {
  if (h == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "NULL handle");
  const sg::MpsModel& md = h->model;
  copy_out(md.colptr, colptr);
  copy_out(md.rowidx, rowidx);
  copy_out(md.vals, vals);
  copy_out(md.obj, obj);
  copy_out(md.col_lower, col_lower);
  copy_out(md.col_upper, col_upper);
  copy_out(md.col_integer, col_integer);
  copy_out(md.row_lower, row_lower);
  copy_out(md.row_upper, row_upper);
  return SG_OK;
}

int sg_mps_get_names(const sg_mps* h, char* name, char* row_names, int64_t* row_starts,
                     char* col_names, int64_t* col_starts) {
  if (h == nullptr) return fail(SG_ERR_INVALID_ARGUMENT, "NULL handle");
  const sg::MpsModel& md = h->model;
  if (name != nullptr && !md.name.empty()) memcpy(name, md.name.data(), md.name.size());
  copy_out(md.row_names, row_names);
  copy_out(md.row_name_start, row_starts);
  copy_out(md.col_names, col_names);
  copy_out(md.col_name_start, col_starts);
  return SG_OK;
}

void sg_mps_free(sg_mps* h) { delete h; }

}  // extern "C"
