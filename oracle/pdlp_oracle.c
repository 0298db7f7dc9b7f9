/*
 * ORACLE — test infrastructure only. A plain-C restatement of the reference solver's CPU PDLP
 * path, used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the result the
 * GPU engine is compared with and as the timed CPU baseline. The product path (samaya_gb300/) never links, loads or calls it.
 *
 * Pinned: tests/test_oracle_pin.py checks this restatement bit-for-bit (iteration counts, x, y,
 * residuals, rays) against golden fixtures produced by the reference's own compiled code
 * (oracle/Makefile.ref + oracle/ref_driver.cpp -> tests/golden/make_golden.py).
 *
 * Every function follows one reference function, in the same order of floating-point
 * operations, so that the results agree to the bit when compiled with -ffp-contract=off:
 *   orc_compute_scaling   src/linalg/scaling.cpp:130-200   (power-of-two geometric + equilibration)
 *   orc_make_problem      src/lp/lp_solver.cpp:28-51       (computational form [A -I] v = 0)
 *   ruiz                  src/lp/pdlp.cpp:109-187          (10 passes of L2 Ruiz)
 *   apply_eq              src/lp/pdlp.cpp:190-209
 *   operator_norm         src/lp/pdlp.cpp:36-103           (20 power iterations, mt19937_64(12345))
 *   orc_pdlp_solve        src/lp/pdlp.cpp:250-1193         (the CPU branch of solve_pdlp_once)
 *   orc_eval_sums         src/lp/pdlp.cpp:411-488          (the seven evaluation sums)
 *   orc_pdhg_steps        src/lp/pdlp.cpp:574-651          (fixed-step PDHG, for kernel parity)
 * and one method with no reference counterpart (the engine's Halpern variant, restated from its
 * publication; its parity is by value against the engine's kernels, not pinned to the reference):
 *   orc_halpern_steps     reflected Halpern PDHG (Lu and Yang, cuPDLPx, 2025)
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define ORC_INF (1.0 / 0.0)

/* SimplexStatus values (src/lp/simplex.hpp:28-35). */
enum { ORC_OPTIMAL = 0, ORC_INFEASIBLE = 1, ORC_UNBOUNDED = 2, ORC_ITERATION_LIMIT = 3,
       ORC_TIME_LIMIT = 4, ORC_NUMERICAL_ERROR = 5 };

typedef struct {
  int rows, cols;
  int64_t* start; /* cols + 1 */
  int32_t* index; /* nnz */
  double* value;  /* nnz */
} csc_t;

static void csc_free(csc_t* a) {
  free(a->start);
  free(a->index);
  free(a->value);
  a->start = NULL;
  a->index = NULL;
  a->value = NULL;
}

static csc_t csc_copy(int rows, int cols, const int64_t* s, const int32_t* i, const double* v) {
  csc_t a;
  int64_t nnz = s[cols];
  a.rows = rows;
  a.cols = cols;
  a.start = (int64_t*)malloc(sizeof(int64_t) * (size_t)(cols + 1));
  a.index = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
  a.value = (double*)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  memcpy(a.start, s, sizeof(int64_t) * (size_t)(cols + 1));
  if (nnz > 0) {
    memcpy(a.index, i, sizeof(int32_t) * (size_t)nnz);
    memcpy(a.value, v, sizeof(double) * (size_t)nnz);
  }
  return a;
}

/* SparseMatrix::transpose (src/linalg/sparse_matrix.cpp:48-67): counting sort by row, columns
 * scattered in increasing order so the transpose's indices are sorted. */
static csc_t csc_transpose(const csc_t* a) {
  csc_t t;
  int64_t nnz = a->start[a->cols];
  t.rows = a->cols;
  t.cols = a->rows;
  t.start = (int64_t*)calloc((size_t)a->rows + 1, sizeof(int64_t));
  t.index = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
  t.value = (double*)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  for (int64_t p = 0; p < nnz; ++p) t.start[a->index[p] + 1]++;
  for (int i = 0; i < a->rows; ++i) t.start[i + 1] += t.start[i];
  int64_t* next = (int64_t*)malloc(sizeof(int64_t) * (size_t)(a->rows > 0 ? a->rows : 1));
  for (int i = 0; i < a->rows; ++i) next[i] = t.start[i];
  for (int j = 0; j < a->cols; ++j) {
    for (int64_t p = a->start[j]; p < a->start[j + 1]; ++p) {
      int64_t q = next[a->index[p]]++;
      t.index[q] = j;
      t.value[q] = a->value[p];
    }
  }
  free(next);
  return t;
}

/* The entries of a scaled copy, as SparseMatrix::from_triplets would keep them: sorted input,
 * so only exact zeros are dropped (src/linalg/sparse_matrix.cpp:15-46). */
static csc_t csc_scaled(const csc_t* a, const double* row_f, const double* col_f) {
  csc_t r;
  int64_t nnz = a->start[a->cols];
  r.rows = a->rows;
  r.cols = a->cols;
  r.start = (int64_t*)malloc(sizeof(int64_t) * (size_t)(a->cols + 1));
  r.index = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
  r.value = (double*)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  int64_t k = 0;
  r.start[0] = 0;
  for (int j = 0; j < a->cols; ++j) {
    double cf = col_f[j];
    for (int64_t p = a->start[j]; p < a->start[j + 1]; ++p) {
      double v = a->value[p] * row_f[a->index[p]] * cf;
      if (v != 0.0) {
        r.index[k] = a->index[p];
        r.value[k] = v;
        ++k;
      }
    }
    r.start[j + 1] = k;
  }
  return r;
}

/* ------------------------------------------------------------------------------------------ */
/* Power-of-two scaling (src/linalg/scaling.cpp:60-200) and make_problem (lp_solver.cpp:28-51). */

static double round_to_power_of_two(double v) {
  if (!(v > 0.0) || !isfinite(v)) return 1.0;
  return ldexp(1.0, (int)lround(log2(v)));
}

static double clamp_factor(double v) {
  const double lo = 0x1p-40, hi = 0x1p40;
  return v < lo ? lo : (hi < v ? hi : v);
}

static double magnitude_ratio(const csc_t* a, const double* row, const double* col) {
  double lo = ORC_INF, hi = 0.0;
  for (int j = 0; j < a->cols; ++j) {
    for (int64_t p = a->start[j]; p < a->start[j + 1]; ++p) {
      double v = fabs(a->value[p]) * row[a->index[p]] * col[j];
      lo = v < lo ? v : lo;
      hi = hi < v ? v : hi;
    }
  }
  return hi > 0.0 ? hi / lo : 1.0;
}

static void scan_rows(const csc_t* a, const double* col, double* row_min, double* row_max) {
  for (int i = 0; i < a->rows; ++i) {
    row_min[i] = ORC_INF;
    row_max[i] = 0.0;
  }
  for (int j = 0; j < a->cols; ++j) {
    for (int64_t p = a->start[j]; p < a->start[j + 1]; ++p) {
      double v = fabs(a->value[p]) * col[j];
      int i = a->index[p];
      row_min[i] = v < row_min[i] ? v : row_min[i];
      row_max[i] = row_max[i] < v ? v : row_max[i];
    }
  }
}

/* compute_scaling with the default ScalingOptions (10 passes, 0.9 improvement, equilibrate). */
void orc_compute_scaling(int m, int n, const int64_t* colptr, const int32_t* rowidx,
                         const double* vals, double* col, double* row) {
  csc_t a;
  a.rows = m;
  a.cols = n;
  a.start = (int64_t*)colptr;
  a.index = (int32_t*)rowidx;
  a.value = (double*)vals;
  for (int i = 0; i < m; ++i) row[i] = 1.0;
  for (int j = 0; j < n; ++j) col[j] = 1.0;
  if (colptr[n] == 0) return;
  double* row_min = (double*)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  double* row_max = (double*)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  double* prev_row = (double*)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  double* prev_col = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  double ratio = magnitude_ratio(&a, row, col);
  for (int pass = 0; pass < 10 && ratio > 1.0; ++pass) {
    memcpy(prev_row, row, sizeof(double) * (size_t)m);
    memcpy(prev_col, col, sizeof(double) * (size_t)n);
    scan_rows(&a, col, row_min, row_max);
    for (int i = 0; i < m; ++i) {
      if (row_max[i] > 0.0) row[i] = clamp_factor(1.0 / sqrt(row_min[i] * row_max[i]));
    }
    for (int j = 0; j < n; ++j) {
      double lo = ORC_INF, hi = 0.0;
      for (int64_t p = colptr[j]; p < colptr[j + 1]; ++p) {
        double v = fabs(vals[p]) * row[rowidx[p]];
        lo = v < lo ? v : lo;
        hi = hi < v ? v : hi;
      }
      if (hi > 0.0) col[j] = clamp_factor(1.0 / sqrt(lo * hi));
    }
    double new_ratio = magnitude_ratio(&a, row, col);
    if (new_ratio > ratio) {
      memcpy(row, prev_row, sizeof(double) * (size_t)m);
      memcpy(col, prev_col, sizeof(double) * (size_t)n);
      break;
    }
    int small_gain = new_ratio > 0.9 * ratio;
    ratio = new_ratio;
    if (small_gain) break;
  }
  scan_rows(&a, col, row_min, row_max);
  for (int i = 0; i < m; ++i) {
    if (row_max[i] > 0.0) row[i] = clamp_factor(1.0 / row_max[i]);
  }
  for (int j = 0; j < n; ++j) {
    double hi = 0.0;
    for (int64_t p = colptr[j]; p < colptr[j + 1]; ++p) {
      double v = fabs(vals[p]) * row[rowidx[p]];
      hi = hi < v ? v : hi;
    }
    if (hi > 0.0) col[j] = clamp_factor(1.0 / hi);
  }
  for (int i = 0; i < m; ++i) row[i] = round_to_power_of_two(row[i]);
  for (int j = 0; j < n; ++j) col[j] = round_to_power_of_two(col[j]);
  free(row_min);
  free(row_max);
  free(prev_row);
  free(prev_col);
}

/* make_problem: writes the scaled A (same sparsity; exact zeros dropped, *nnz_out set), and the
 * computational-form cost/lower/upper of n + m entries. */
void orc_make_problem(int m, int n, const int64_t* colptr, const int32_t* rowidx,
                      const double* vals, const double* obj, const double* col_lower,
                      const double* col_upper, const double* row_lower, const double* row_upper,
                      int maximize, const double* col, const double* row, int64_t* out_colptr,
                      int32_t* out_rowidx, double* out_vals, double* cost, double* lower,
                      double* upper, int64_t* nnz_out) {
  double sense = maximize ? -1.0 : 1.0;
  int64_t k = 0;
  out_colptr[0] = 0;
  for (int j = 0; j < n; ++j) {
    for (int64_t p = colptr[j]; p < colptr[j + 1]; ++p) {
      double v = vals[p] * row[rowidx[p]] * col[j];
      if (v != 0.0) {
        out_rowidx[k] = rowidx[p];
        out_vals[k] = v;
        ++k;
      }
    }
    out_colptr[j + 1] = k;
  }
  *nnz_out = k;
  for (int j = 0; j < n; ++j) {
    cost[j] = sense * obj[j] * col[j];
    lower[j] = col_lower[j] / col[j];
    upper[j] = col_upper[j] / col[j];
  }
  for (int i = 0; i < m; ++i) {
    cost[n + i] = 0.0;
    lower[n + i] = row_lower[i] * row[i];
    upper[n + i] = row_upper[i] * row[i];
  }
}

/* ------------------------------------------------------------------------------------------ */
/* std::mt19937_64 (Matsumoto & Nishimura, 64-bit Mersenne Twister, the C++ standard's
 * parameters) and std::uniform_real_distribution<double>(-1, 1) as libstdc++ computes it
 * (generate_canonical with one 64-bit draw), for the power iteration's start vector. */
typedef struct {
  uint64_t mt[312];
  int idx;
} mt64_t;

static void mt64_seed(mt64_t* s, uint64_t seed) {
  s->mt[0] = seed;
  for (int i = 1; i < 312; ++i) {
    s->mt[i] = 6364136223846793005ULL * (s->mt[i - 1] ^ (s->mt[i - 1] >> 62)) + (uint64_t)i;
  }
  s->idx = 312;
}

static uint64_t mt64_next(mt64_t* s) {
  const uint64_t upper = 0xFFFFFFFF80000000ULL, lower = 0x7FFFFFFFULL;
  if (s->idx >= 312) {
    for (int i = 0; i < 312; ++i) {
      uint64_t x = (s->mt[i] & upper) | (s->mt[(i + 1) % 312] & lower);
      uint64_t xa = x >> 1;
      if (x & 1ULL) xa ^= 0xB5026F5AA96619E9ULL;
      s->mt[i] = s->mt[(i + 156) % 312] ^ xa;
    }
    s->idx = 0;
  }
  uint64_t y = s->mt[s->idx++];
  y ^= (y >> 29) & 0x5555555555555555ULL;
  y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
  y ^= (y << 37) & 0xFFF7EEE000000000ULL;
  y ^= y >> 43;
  return y;
}

static double uniform_m1_1(mt64_t* s) {
  double r = (double)mt64_next(s) / 18446744073709551616.0;
  if (r >= 1.0) r = nextafter(1.0, 0.0);
  return r * 2.0 + -1.0;
}

/* The start vector of the power iteration (exported so the product's own setup can be
 * checked against it). */
void orc_power_start(int m, double* u) {
  mt64_t rng;
  mt64_seed(&rng, 12345ULL);
  for (int i = 0; i < m; ++i) u[i] = uniform_m1_1(&rng);
}

/* estimate_operator_norm (src/lp/pdlp.cpp:36-103). */
static double operator_norm(const csc_t* A, const csc_t* At, int max_iters) {
  int m = A->rows, n = A->cols;
  if (m == 0) return 1.0;
  double* u = (double*)malloc(sizeof(double) * (size_t)m);
  double* v = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  orc_power_start(m, u);
  double u_norm = 0.0;
  for (int i = 0; i < m; ++i) u_norm += u[i] * u[i];
  u_norm = sqrt(u_norm);
  for (int i = 0; i < m; ++i) u[i] /= u_norm;
  double sigma = 0.0;
  double result = -1.0;
  for (int it = 0; it < max_iters; ++it) {
    for (int j = 0; j < n; ++j) v[j] = 0.0;
    for (int j = 0; j < m; ++j) {
      for (int64_t p = At->start[j]; p < At->start[j + 1]; ++p) v[At->index[p]] += At->value[p] * u[j];
    }
    double v_norm = 0.0;
    for (int j = 0; j < n; ++j) v_norm += v[j] * v[j];
    v_norm = sqrt(v_norm);
    if (v_norm == 0.0) {
      result = 1.0;
      break;
    }
    for (int i = 0; i < m; ++i) u[i] = 0.0;
    for (int j = 0; j < n; ++j) {
      if (v[j] == 0.0) continue;
      for (int64_t p = A->start[j]; p < A->start[j + 1]; ++p) u[A->index[p]] += A->value[p] * v[j];
    }
    u_norm = 0.0;
    for (int i = 0; i < m; ++i) u_norm += u[i] * u[i];
    u_norm = sqrt(u_norm);
    if (u_norm == 0.0) {
      result = 1.0;
      break;
    }
    sigma = u_norm / v_norm;
    for (int i = 0; i < m; ++i) u[i] /= u_norm;
  }
  free(u);
  free(v);
  if (result > 0.0) return result;
  double la = sigma * 1.01;
  return sqrt(la * la + 1.0);
}

/* ruiz_equilibration (src/lp/pdlp.cpp:109-187). */
static void ruiz(const csc_t* A, const csc_t* At, double* rs, double* cs, int max_iters) {
  int m = A->rows, n = A->cols;
  for (int i = 0; i < m; ++i) rs[i] = 1.0;
  for (int j = 0; j < n; ++j) cs[j] = 1.0;
  if (m == 0 || n == 0) return;
  double* rn = (double*)malloc(sizeof(double) * (size_t)m);
  double* cn = (double*)malloc(sizeof(double) * (size_t)n);
  for (int it = 0; it < max_iters; ++it) {
    for (int j = 0; j < n; ++j) {
      double sum = 0.0;
      for (int64_t p = A->start[j]; p < A->start[j + 1]; ++p) {
        double v = A->value[p] * rs[A->index[p]] * cs[j];
        sum += v * v;
      }
      cn[j] = sqrt(sum);
    }
    for (int i = 0; i < m; ++i) {
      double sum = 0.0;
      for (int64_t p = At->start[i]; p < At->start[i + 1]; ++p) {
        double v = At->value[p] * rs[i] * cs[At->index[p]];
        sum += v * v;
      }
      rn[i] = sqrt(sum);
    }
    int converged = 1;
    for (int j = 0; j < n; ++j) {
      if (cn[j] > 0) {
        double s = cs[j] / cn[j];
        s = s < 1e8 ? s : 1e8;
        s = 1e-8 < s ? s : 1e-8;
        double base = fabs(cs[j]) > 1.0 ? fabs(cs[j]) : 1.0;
        if (fabs(s - cs[j]) / base > 0.1) converged = 0;
        cs[j] = s;
      }
    }
    for (int i = 0; i < m; ++i) {
      if (rn[i] > 0) {
        double s = rs[i] / rn[i];
        s = s < 1e8 ? s : 1e8;
        s = 1e-8 < s ? s : 1e-8;
        double base = fabs(rs[i]) > 1.0 ? fabs(rs[i]) : 1.0;
        if (fabs(s - rs[i]) / base > 0.1) converged = 0;
        rs[i] = s;
      }
    }
    if (converged) break;
  }
  free(rn);
  free(cn);
}

/* ------------------------------------------------------------------------------------------ */
/* The evaluation (src/lp/pdlp.cpp:402-527). */

typedef struct {
  double primal_sq, dual_sq, primal_obj, dual_obj, x_sq, r_sq, y_sq;
} sums_t;

typedef struct {
  double rel_primal, rel_dual, rel_gap, gap, primal_obj, dual_obj;
} measure_t;

typedef struct {
  int m, n;
  const csc_t* A;  /* original (pre-Ruiz) A and its transpose */
  const csc_t* At;
  const double *cost, *lower, *upper; /* original, n + m */
  const double *cs, *rs;
  double* x_orig; /* scratch n */
  double* r_orig; /* m */
  double* y_orig; /* m */
  double* ax;     /* m */
  double* aty;    /* n + m */
  double a_norm_max_col, at_norm_max_row, c_norm;
} eval_ctx;

static sums_t eval_sums(eval_ctx* e, const double* vv, const double* yy) {
  sums_t s = {0, 0, 0, 0, 0, 0, 0};
  int m = e->m, n = e->n;
  for (int j = 0; j < n; ++j) e->x_orig[j] = vv[j] * e->cs[j];
  for (int i = 0; i < m; ++i) e->r_orig[i] = vv[n + i] / e->rs[i];
  for (int i = 0; i < m; ++i) e->y_orig[i] = yy[i] * e->rs[i];
  if (m > 0) {
    for (int i = 0; i < m; ++i) e->ax[i] = 0.0;
    for (int j = 0; j < n; ++j) {
      double xj = e->x_orig[j];
      if (xj == 0.0) continue;
      for (int64_t p = e->A->start[j]; p < e->A->start[j + 1]; ++p)
        e->ax[e->A->index[p]] += e->A->value[p] * xj;
    }
    for (int i = 0; i < m; ++i) {
      double diff = e->ax[i] - e->r_orig[i];
      s.primal_sq += diff * diff;
    }
  }
  for (int k = 0; k < n + m; ++k) e->aty[k] = 0.0;
  if (m > 0) {
    for (int i = 0; i < m; ++i) {
      double yi = e->y_orig[i];
      if (yi == 0.0) continue;
      for (int64_t p = e->At->start[i]; p < e->At->start[i + 1]; ++p)
        e->aty[e->At->index[p]] += e->At->value[p] * yi;
    }
    for (int i = 0; i < m; ++i) e->aty[n + i] = -e->y_orig[i];
    for (int k = 0; k < n + m; ++k) {
      double g = e->cost[k] + e->aty[k];
      int lo = e->lower[k] > -ORC_INF, up = e->upper[k] < ORC_INF;
      double lambda = lo && up ? g : lo ? (g > 0.0 ? g : 0.0) : up ? (g < 0.0 ? g : 0.0) : 0.0;
      s.dual_sq += (g - lambda) * (g - lambda);
    }
  }
  for (int j = 0; j < n; ++j) s.primal_obj += e->cost[j] * e->x_orig[j];
  for (int i = 0; i < m; ++i) s.primal_obj += e->cost[n + i] * e->r_orig[i];
  for (int k = 0; k < n + m; ++k) {
    double g = e->cost[k] + e->aty[k];
    int lo = e->lower[k] > -ORC_INF, up = e->upper[k] < ORC_INF;
    double lambda = lo && up ? g : lo ? (g > 0.0 ? g : 0.0) : up ? (g < 0.0 ? g : 0.0) : 0.0;
    if (lambda > 0.0) s.dual_obj += lambda * e->lower[k];
    if (lambda < 0.0) s.dual_obj += lambda * e->upper[k];
  }
  for (int j = 0; j < n; ++j) s.x_sq += e->x_orig[j] * e->x_orig[j];
  for (int i = 0; i < m; ++i) s.r_sq += e->r_orig[i] * e->r_orig[i];
  for (int i = 0; i < m; ++i) s.y_sq += e->y_orig[i] * e->y_orig[i];
  return s;
}

static measure_t finish(const eval_ctx* e, sums_t s) {
  measure_t r;
  double primal_res = sqrt(s.primal_sq);
  double dual_res = sqrt(s.dual_sq);
  double gap = s.primal_obj - s.dual_obj;
  double primal_scale = 1.0 + e->a_norm_max_col * sqrt(s.x_sq) + sqrt(s.r_sq);
  double dual_scale = 1.0 + e->at_norm_max_row * sqrt(s.y_sq) + e->c_norm;
  double gap_scale = 1.0 + fabs(s.primal_obj) + fabs(s.dual_obj);
  r.rel_primal = e->m > 0 ? primal_res / primal_scale : 0.0;
  r.rel_dual = e->m > 0 ? dual_res / dual_scale : 0.0;
  r.rel_gap = gap / gap_scale;
  r.gap = gap;
  r.primal_obj = s.primal_obj;
  r.dual_obj = s.dual_obj;
  return r;
}

static double kkt_of(double omega, measure_t e) {
  return sqrt(omega * omega * e.rel_primal * e.rel_primal +
              e.rel_dual * e.rel_dual / (omega * omega) + e.rel_gap * e.rel_gap);
}

static double now_seconds(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void* xmalloc(size_t count, size_t size) {
  void* p = calloc(count > 0 ? count : 1, size);
  return p;
}

/* Farkas check on the average dual (src/lp/pdlp.cpp:723-842). Returns 1 when y_erg certifies
 * infeasibility. */
static int farkas_check(const eval_ctx* e, const double* y_erg) {
  int m = e->m, n = e->n;
  const double* lower = e->lower;
  const double* upper = e->upper;
  double* yf = (double*)xmalloc((size_t)m, sizeof(double));
  double y_max = 0.0;
  for (int i = 0; i < m; ++i) {
    yf[i] = y_erg[i] * e->rs[i];
    double a = fabs(yf[i]);
    y_max = y_max < a ? a : y_max;
  }
  int found = 0;
  if (y_max > 1e-6) {
    double* aty = (double*)xmalloc((size_t)(n + m), sizeof(double));
    for (int i = 0; i < m; ++i) {
      double yi = yf[i];
      if (yi == 0.0) continue;
      for (int64_t p = e->At->start[i]; p < e->At->start[i + 1]; ++p)
        aty[e->At->index[p]] += e->At->value[p] * yi;
    }
    for (int i = 0; i < m; ++i) aty[n + i] = -yf[i];
    double w_scale = 0.0;
    for (int j = 0; j < n; ++j) w_scale += fabs(aty[j]);
    for (int i = 0; i < m; ++i) w_scale += fabs(aty[n + i]);
    double tol = 1e-9 * w_scale;
    double min_f = 0.0, max_f = 0.0;
    for (int k = 0; k < n + m; ++k) {
      double coef = fabs(aty[k]) <= tol ? 0.0 : aty[k];
      double lo = lower[k], up = upper[k];
      if (coef > 0) {
        min_f += (lo > -ORC_INF) ? coef * lo : -ORC_INF;
        max_f += (up < ORC_INF) ? coef * up : ORC_INF;
      } else if (coef < 0) {
        min_f += (up < ORC_INF) ? coef * up : -ORC_INF;
        max_f += (lo > -ORC_INF) ? coef * lo : ORC_INF;
      }
    }
    double scale = 0.0;
    for (int j = 0; j < n; ++j) {
      double w = aty[j] / y_max;
      if (fabs(w) > 1e-9) {
        if (lower[j] > -ORC_INF) { double t = fabs(w * lower[j]); scale = scale < t ? t : scale; }
        if (upper[j] < ORC_INF) { double t = fabs(w * upper[j]); scale = scale < t ? t : scale; }
      }
    }
    for (int i = 0; i < m; ++i) {
      double coef = -aty[n + i] / y_max;
      if (fabs(coef) > 1e-9) {
        if (lower[n + i] > -ORC_INF) { double t = fabs(coef * lower[n + i]); scale = scale < t ? t : scale; }
        if (upper[n + i] < ORC_INF) { double t = fabs(coef * upper[n + i]); scale = scale < t ? t : scale; }
      }
    }
    if (!isfinite(scale)) scale = 0.0;
    double margin = 1e-8 * (1.0 + scale);
    if ((isfinite(min_f) && min_f > margin) || (isfinite(max_f) && max_f < -margin)) found = 1;
    free(aty);
  }
  free(yf);
  return found;
}

/* Improving-ray check on v_new - v (src/lp/pdlp.cpp:852-1042). Returns 1 and fills ray_x (n)
 * when the difference of consecutive iterates is a primal ray. */
static int ray_check(const eval_ctx* e, const double* v_new, const double* v, double* ray_x) {
  int m = e->m, n = e->n, nt = n + m;
  const double* lower = e->lower;
  const double* upper = e->upper;
  double* cand = (double*)xmalloc((size_t)nt, sizeof(double));
  double v_max = 0.0;
  for (int k = 0; k < nt; ++k) {
    cand[k] = v_new[k] - v[k];
    double a = fabs(cand[k]);
    v_max = v_max < a ? a : v_max;
  }
  int found = 0;
  for (int j = 0; j < n; ++j) ray_x[j] = 0.0;
  if (v_max > 1e-6) {
    double* dir = (double*)xmalloc((size_t)nt, sizeof(double));
    for (int k = 0; k < nt; ++k) dir[k] = cand[k] / v_max;
    double* res = (double*)xmalloc((size_t)m, sizeof(double));
    for (int j = 0; j < n; ++j) {
      double xj = dir[j] * e->cs[j];
      if (xj == 0.0) continue;
      for (int64_t p = e->A->start[j]; p < e->A->start[j + 1]; ++p)
        res[e->A->index[p]] += e->A->value[p] * xj;
    }
    for (int i = 0; i < m; ++i) res[i] -= dir[n + i] / e->rs[i];
    double primal_feas = 0.0;
    for (int i = 0; i < m; ++i) primal_feas += res[i] * res[i];
    primal_feas = sqrt(primal_feas);
    double cost_dir = 0.0;
    for (int j = 0; j < n; ++j) cost_dir += e->cost[j] * (dir[j] * e->cs[j]);
    for (int i = 0; i < m; ++i) cost_dir += e->cost[n + i] * (dir[n + i] / e->rs[i]);
    const double bound_tol = 1e-4, eq_tol = 1e-3;
    int ok = 1;
    for (int j = 0; j < n && ok; ++j) {
      double xj = dir[j] * e->cs[j];
      int lb = lower[j] > -ORC_INF / 2, ub = upper[j] < ORC_INF / 2;
      int fixed = lb && ub && (upper[j] - lower[j] <= 1e-10 * (1.0 + fabs(lower[j])));
      if (lb && ub) {
        double t = fixed ? eq_tol : bound_tol;
        if (fabs(xj) > t) ok = 0;
        xj = 0.0;
      } else if (lb) {
        if (xj < -bound_tol) ok = 0;
        xj = xj > 0.0 ? xj : 0.0;
      } else if (ub) {
        if (xj > bound_tol) ok = 0;
        xj = xj < 0.0 ? xj : 0.0;
      }
      ray_x[j] = xj;
    }
    double* av = (double*)xmalloc((size_t)m, sizeof(double));
    for (int j = 0; j < n; ++j) {
      double xj = ray_x[j];
      if (xj == 0.0) continue;
      for (int64_t p = e->A->start[j]; p < e->A->start[j + 1]; ++p)
        av[e->A->index[p]] += e->A->value[p] * xj;
    }
    for (int i = 0; i < m && ok; ++i) {
      double a = av[i];
      double lo = lower[n + i], up = upper[n + i];
      int lb = lo > -ORC_INF / 2, ub = up < ORC_INF / 2;
      int fixed = lb && ub && (up - lo <= 1e-10 * (1.0 + fabs(lo)));
      if (lb && ub) {
        double t = fixed ? eq_tol : bound_tol;
        if (fabs(a) > t) ok = 0;
      } else if (lb) {
        if (a < -bound_tol) ok = 0;
      } else if (ub) {
        if (a > bound_tol) ok = 0;
      }
    }
    if (primal_feas < 1e-6 && cost_dir < -1e-8 && ok) found = 1;
    free(av);
    free(res);
    free(dir);
  }
  free(cand);
  return found;
}

/* Counters for tests and logs. */
typedef struct {
  long long restarts;
  long long evaluations;
  double omega;
  double step_size; /* eta = 0.99 / L */
  double operator_norm;
  double last[3]; /* relative primal, dual, gap of the current iterate at the last evaluation */
} orc_stats_t;

/* The CPU branch of solve_pdlp_once (src/lp/pdlp.cpp:250-1193). A is the LpProblem's CSC
 * (m x n); cost/lower/upper have n + m entries. x: n + m, y: m, dual_ray: m, primal_ray: n.
 * ray_flags[0]/[1] report whether a dual/primal ray was written. Returns the SimplexStatus. */
int orc_pdlp_solve(int m, int n, const int64_t* colptr, const int32_t* rowidx, const double* vals,
                   const double* cost, const double* lower, const double* upper, double tol,
                   long long max_iterations, double time_limit, long long* iterations_out,
                   double* res3, double* x_out, double* y_out, double* dual_ray,
                   double* primal_ray, int* ray_flags, orc_stats_t* stats) {
  const double t_start = now_seconds();
  const int nt = n + m;
  const int has_limit = time_limit > 0 && isfinite(time_limit);
  int status = ORC_NUMERICAL_ERROR;
  long long result_iterations = 0;
  double r_primal = 0.0, r_dual = 0.0, r_gap = 0.0;
  ray_flags[0] = ray_flags[1] = 0;

  csc_t A = csc_copy(m, n, colptr, rowidx, vals);
  csc_t At = csc_transpose(&A);
  double* rs = (double*)xmalloc((size_t)m, sizeof(double));
  double* cs = (double*)xmalloc((size_t)n, sizeof(double));
  ruiz(&A, &At, rs, cs, 10);
  csc_t Aeq = csc_scaled(&A, rs, cs);
  csc_t Ateq = csc_scaled(&At, cs, rs);

  double* cost_eq = (double*)xmalloc((size_t)nt, sizeof(double));
  double* lower_eq = (double*)xmalloc((size_t)nt, sizeof(double));
  double* upper_eq = (double*)xmalloc((size_t)nt, sizeof(double));
  for (int k = 0; k < nt; ++k) {
    cost_eq[k] = cost[k];
    lower_eq[k] = lower[k];
    upper_eq[k] = upper[k];
  }
  for (int j = 0; j < n; ++j) {
    cost_eq[j] *= cs[j];
    lower_eq[j] /= cs[j];
    upper_eq[j] /= cs[j];
  }
  for (int i = 0; i < m; ++i) {
    cost_eq[n + i] *= rs[i];
    lower_eq[n + i] *= rs[i];
    upper_eq[n + i] *= rs[i];
  }
  const double L = operator_norm(&Aeq, &Ateq, 20);
  const double eta = 0.99 / L;
  double omega = 1.0;
  double tau = eta / omega;
  double sigma = eta * omega;
  const double theta = 1.0;
  long long k_since = 0;

  double* v = (double*)xmalloc((size_t)nt, sizeof(double));
  double* y = (double*)xmalloc((size_t)m, sizeof(double));
  double* v_prev = (double*)xmalloc((size_t)nt, sizeof(double));
  double* v_erg = (double*)xmalloc((size_t)nt, sizeof(double));
  double* y_erg = (double*)xmalloc((size_t)m, sizeof(double));
  double* residual = (double*)xmalloc((size_t)(m > 1 ? m : 1), sizeof(double));
  double* aty = (double*)xmalloc((size_t)nt, sizeof(double));
  double* v_new = (double*)xmalloc((size_t)nt, sizeof(double));
  double* v_bar = (double*)xmalloc((size_t)nt, sizeof(double));
  double* y_new = (double*)xmalloc((size_t)m, sizeof(double));
  double* v_restart = (double*)xmalloc((size_t)nt, sizeof(double));
  double* y_restart = (double*)xmalloc((size_t)m, sizeof(double));
  double* ray_x = (double*)xmalloc((size_t)n, sizeof(double));

  long long max_iter = max_iterations;
  if (max_iter <= 0) {
    max_iter = 10000LL * (long long)(m + n) / 10;
    if (max_iter < 10000LL) max_iter = 10000LL;
    if (!has_limit && max_iter > 1000000LL) max_iter = 1000000LL;
  }

  eval_ctx e;
  e.m = m;
  e.n = n;
  e.A = &A;
  e.At = &At;
  e.cost = cost;
  e.lower = lower;
  e.upper = upper;
  e.cs = cs;
  e.rs = rs;
  e.x_orig = (double*)xmalloc((size_t)n, sizeof(double));
  e.r_orig = (double*)xmalloc((size_t)m, sizeof(double));
  e.y_orig = (double*)xmalloc((size_t)m, sizeof(double));
  e.ax = (double*)xmalloc((size_t)m, sizeof(double));
  e.aty = (double*)xmalloc((size_t)nt, sizeof(double));
  e.a_norm_max_col = 0.0;
  e.at_norm_max_row = 0.0;
  if (m > 0) {
    for (int j = 0; j < n; ++j) {
      double c = 0.0;
      for (int64_t p = A.start[j]; p < A.start[j + 1]; ++p) c += A.value[p] * A.value[p];
      double s = sqrt(c);
      e.a_norm_max_col = e.a_norm_max_col < s ? s : e.a_norm_max_col;
    }
    for (int i = 0; i < m; ++i) {
      double r = 0.0;
      for (int64_t p = At.start[i]; p < At.start[i + 1]; ++p) r += At.value[p] * At.value[p];
      double s = sqrt(r);
      e.at_norm_max_row = e.at_norm_max_row < s ? s : e.at_norm_max_row;
    }
  }
  double c_norm = 0.0;
  for (int k = 0; k < nt; ++k) c_norm += cost[k] * cost[k];
  e.c_norm = sqrt(c_norm);

  double kkt_at_restart = ORC_INF, kkt_previous = ORC_INF;
  long long restarts = 0, evaluations = 0;
  measure_t last_meas = {ORC_INF, ORC_INF, ORC_INF, 0.0, 0.0, 0.0};
  int done = 0;
  for (long long iter = 0; iter < max_iter && !done; ++iter) {
    if (has_limit && now_seconds() - t_start > time_limit) {
      status = ORC_TIME_LIMIT;
      result_iterations = iter;
      break;
    }
    int evaluate = (iter + 1) % 64 == 0 || iter + 1 == max_iter;
    for (int j = 0; j < nt; ++j) v_bar[j] = v[j] + theta * (v[j] - v_prev[j]);
    for (int i = 0; i < m; ++i) residual[i] = 0.0;
    if (m > 0) {
      for (int j = 0; j < n; ++j) {
        double vj = v_bar[j];
        if (vj == 0.0) continue;
        for (int64_t p = Aeq.start[j]; p < Aeq.start[j + 1]; ++p) residual[Aeq.index[p]] += Aeq.value[p] * vj;
      }
      for (int i = 0; i < m; ++i) residual[i] -= v_bar[n + i];
      for (int i = 0; i < m; ++i) y_new[i] = y[i] + sigma * residual[i];
    }
    for (int k = 0; k < nt; ++k) aty[k] = 0.0;
    if (m > 0) {
      for (int i = 0; i < m; ++i) {
        double yi = y_new[i];
        if (yi == 0.0) continue;
        for (int64_t p = Ateq.start[i]; p < Ateq.start[i + 1]; ++p) aty[Ateq.index[p]] += Ateq.value[p] * yi;
        aty[n + i] = -yi;
      }
    }
    for (int j = 0; j < nt; ++j) {
      double grad = cost_eq[j] + aty[j];
      v_new[j] = v[j] - tau * grad;
    }
    for (int j = 0; j < nt; ++j) {
      double val = v_new[j];
      if (lower_eq[j] > -ORC_INF && val < lower_eq[j]) val = lower_eq[j];
      if (upper_eq[j] < ORC_INF && val > upper_eq[j]) val = upper_eq[j];
      v_new[j] = val;
    }
    double alpha = 1.0 / (double)(k_since + 1);
    ++k_since;
    for (int j = 0; j < nt; ++j) v_erg[j] = (1.0 - alpha) * v_erg[j] + alpha * v_new[j];
    for (int i = 0; i < m; ++i) y_erg[i] = (1.0 - alpha) * y_erg[i] + alpha * y_new[i];

    if (!evaluate) {
      double* t = v_prev; v_prev = v; v = v_new; v_new = t;
      t = y; y = y_new; y_new = t;
      continue;
    }
    ++evaluations;
    measure_t cur = finish(&e, eval_sums(&e, v_new, y_new));
    measure_t avg = finish(&e, eval_sums(&e, v_erg, y_erg));
    last_meas = cur;
    if (cur.rel_primal < tol && cur.rel_dual < tol && fabs(cur.rel_gap) < tol) {
      status = ORC_OPTIMAL;
      result_iterations = iter + 1;
      r_primal = cur.rel_primal;
      r_dual = cur.rel_dual;
      r_gap = cur.rel_gap;
      memcpy(v, v_new, sizeof(double) * (size_t)nt);
      memcpy(y, y_new, sizeof(double) * (size_t)m);
      break;
    }
    if (avg.rel_primal < tol && avg.rel_dual < tol && fabs(avg.rel_gap) < tol) {
      status = ORC_OPTIMAL;
      result_iterations = iter + 1;
      r_primal = avg.rel_primal;
      r_dual = avg.rel_dual;
      r_gap = avg.rel_gap;
      memcpy(v, v_erg, sizeof(double) * (size_t)nt);
      memcpy(y, y_erg, sizeof(double) * (size_t)m);
      break;
    }
    int detect = iter > 1000 && m > 0 && ((iter + 1) / 64) % 8 == 0;
    if (detect) {
      if (farkas_check(&e, y_erg)) {
        status = ORC_INFEASIBLE;
        result_iterations = iter + 1;
        r_primal = cur.rel_primal;
        r_dual = cur.rel_dual;
        r_gap = cur.rel_gap;
        for (int i = 0; i < m; ++i) dual_ray[i] = y_erg[i];
        ray_flags[0] = 1;
        memcpy(v, v_new, sizeof(double) * (size_t)nt);
        memcpy(y, y_new, sizeof(double) * (size_t)m);
        done = 1;
        break;
      }
      if (ray_check(&e, v_new, v, ray_x)) {
        status = ORC_UNBOUNDED;
        result_iterations = iter + 1;
        r_primal = cur.rel_primal;
        r_dual = cur.rel_dual;
        r_gap = cur.rel_gap;
        for (int j = 0; j < n; ++j) primal_ray[j] = ray_x[j];
        ray_flags[1] = 1;
        memcpy(v, v_new, sizeof(double) * (size_t)nt);
        memcpy(y, y_new, sizeof(double) * (size_t)m);
        done = 1;
        break;
      }
    }
    {
      double kkt_cur = kkt_of(omega, cur);
      double kkt_avg = kkt_of(omega, avg);
      int to_average = kkt_avg < kkt_cur;
      double kkt_cand = kkt_cur < kkt_avg ? kkt_cur : kkt_avg;
      if (!(kkt_at_restart < ORC_INF)) kkt_at_restart = kkt_cand;
      int restart = kkt_cand <= 0.2 * kkt_at_restart ||
                    (kkt_cand <= 0.8 * kkt_at_restart && kkt_cand > kkt_previous) ||
                    (double)k_since >= 0.36 * (double)(iter + 1);
      kkt_previous = kkt_cand;
      if (restart) {
        const double* vc = to_average ? v_erg : v_new;
        const double* yc = to_average ? y_erg : y_new;
        double dx = 0.0, dy = 0.0;
        for (int k = 0; k < nt; ++k) dx += (vc[k] - v_restart[k]) * (vc[k] - v_restart[k]);
        for (int i = 0; i < m; ++i) dy += (yc[i] - y_restart[i]) * (yc[i] - y_restart[i]);
        dx = sqrt(dx);
        dy = sqrt(dy);
        if (dx > 1e-10 && dy > 1e-10) {
          omega = exp(0.5 * log(dy / dx) + 0.5 * log(omega));
          tau = eta / omega;
          sigma = eta * omega;
        }
        memcpy(v_restart, vc, sizeof(double) * (size_t)nt);
        memcpy(y_restart, yc, sizeof(double) * (size_t)m);
        memcpy(v_new, v_restart, sizeof(double) * (size_t)nt);
        memcpy(v, v_restart, sizeof(double) * (size_t)nt);
        memcpy(y_new, y_restart, sizeof(double) * (size_t)m);
        k_since = 0;
        kkt_at_restart = kkt_cand;
        kkt_previous = ORC_INF;
        ++restarts;
      }
    }
    {
      double* t = v_prev; v_prev = v; v = v_new; v_new = t;
      t = y; y = y_new; y_new = t;
    }
  }
  if (status == ORC_NUMERICAL_ERROR) {
    status = ORC_ITERATION_LIMIT;
    result_iterations = max_iter;
  }
  for (int j = 0; j < n; ++j) x_out[j] = v[j] * cs[j];
  for (int i = 0; i < m; ++i) x_out[n + i] = v[n + i] / rs[i];
  for (int i = 0; i < m; ++i) y_out[i] = y[i] * rs[i];
  *iterations_out = result_iterations;
  res3[0] = r_primal;
  res3[1] = r_dual;
  res3[2] = r_gap;
  if (stats) {
    stats->restarts = restarts;
    stats->evaluations = evaluations;
    stats->omega = omega;
    stats->step_size = eta;
    stats->operator_norm = L;
    stats->last[0] = last_meas.rel_primal;
    stats->last[1] = last_meas.rel_dual;
    stats->last[2] = last_meas.rel_gap;
  }

  free(e.x_orig); free(e.r_orig); free(e.y_orig); free(e.ax); free(e.aty);
  free(v); free(y); free(v_prev); free(v_erg); free(y_erg); free(residual); free(aty);
  free(v_new); free(v_bar); free(y_new); free(v_restart); free(y_restart); free(ray_x);
  free(cost_eq); free(lower_eq); free(upper_eq); free(rs); free(cs);
  csc_free(&A); csc_free(&At); csc_free(&Aeq); csc_free(&Ateq);
  return status;
}

/* ------------------------------------------------------------------------------------------ */
/* Pieces exported for kernel-level parity tests. */

/* The Ruiz factors, A_eq (CSC) values in the order of A, and the operator-norm estimate L. */
void orc_setup(int m, int n, const int64_t* colptr, const int32_t* rowidx, const double* vals,
               double* row_scale, double* col_scale, double* aeq_vals, double* ateq_vals_csr,
               double* L_out) {
  csc_t A = csc_copy(m, n, colptr, rowidx, vals);
  csc_t At = csc_transpose(&A);
  ruiz(&A, &At, row_scale, col_scale, 10);
  csc_t Aeq = csc_scaled(&A, row_scale, col_scale);
  csc_t Ateq = csc_scaled(&At, col_scale, row_scale);
  int64_t nnz = colptr[n];
  if (aeq_vals) for (int64_t p = 0; p < nnz && p < Aeq.start[n]; ++p) aeq_vals[p] = Aeq.value[p];
  if (ateq_vals_csr) for (int64_t p = 0; p < nnz && p < Ateq.start[m]; ++p) ateq_vals_csr[p] = Ateq.value[p];
  *L_out = operator_norm(&Aeq, &Ateq, 20);
  csc_free(&A); csc_free(&At); csc_free(&Aeq); csc_free(&Ateq);
}

/* `steps` fixed-step PDHG iterations on an already equilibrated problem (A_eq as CSC m x n, its
 * transpose built here), from the state (v, v_prev, y, v_erg, y_erg) with k iterations since the
 * last restart; the state is updated in place (v_prev <- v, v <- v_new, y <- y_new). */
void orc_pdhg_steps(int m, int n, const int64_t* colptr, const int32_t* rowidx,
                    const double* vals, const double* cost, const double* lower,
                    const double* upper, double tau, double sigma, int steps, long long k,
                    double* v, double* v_prev, double* y, double* v_erg, double* y_erg) {
  const int nt = n + m;
  csc_t A = csc_copy(m, n, colptr, rowidx, vals);
  csc_t At = csc_transpose(&A);
  double* v_bar = (double*)xmalloc((size_t)nt, sizeof(double));
  double* v_new = (double*)xmalloc((size_t)nt, sizeof(double));
  double* y_new = (double*)xmalloc((size_t)m, sizeof(double));
  double* res = (double*)xmalloc((size_t)m, sizeof(double));
  double* aty = (double*)xmalloc((size_t)nt, sizeof(double));
  for (int s = 0; s < steps; ++s) {
    for (int j = 0; j < nt; ++j) v_bar[j] = v[j] + 1.0 * (v[j] - v_prev[j]);
    for (int i = 0; i < m; ++i) res[i] = 0.0;
    for (int j = 0; j < n; ++j) {
      double vj = v_bar[j];
      if (vj == 0.0) continue;
      for (int64_t p = A.start[j]; p < A.start[j + 1]; ++p) res[A.index[p]] += A.value[p] * vj;
    }
    for (int i = 0; i < m; ++i) res[i] -= v_bar[n + i];
    for (int i = 0; i < m; ++i) y_new[i] = y[i] + sigma * res[i];
    for (int q = 0; q < nt; ++q) aty[q] = 0.0;
    for (int i = 0; i < m; ++i) {
      double yi = y_new[i];
      if (yi == 0.0) continue;
      for (int64_t p = At.start[i]; p < At.start[i + 1]; ++p) aty[At.index[p]] += At.value[p] * yi;
      aty[n + i] = -yi;
    }
    for (int j = 0; j < nt; ++j) {
      double val = v[j] - tau * (cost[j] + aty[j]);
      if (lower[j] > -ORC_INF && val < lower[j]) val = lower[j];
      if (upper[j] < ORC_INF && val > upper[j]) val = upper[j];
      v_new[j] = val;
    }
    double alpha = 1.0 / (double)(k + 1);
    ++k;
    for (int j = 0; j < nt; ++j) v_erg[j] = (1.0 - alpha) * v_erg[j] + alpha * v_new[j];
    for (int i = 0; i < m; ++i) y_erg[i] = (1.0 - alpha) * y_erg[i] + alpha * y_new[i];
    memcpy(v_prev, v, sizeof(double) * (size_t)nt);
    memcpy(v, v_new, sizeof(double) * (size_t)nt);
    memcpy(y, y_new, sizeof(double) * (size_t)m);
  }
  free(v_bar); free(v_new); free(y_new); free(res); free(aty);
  csc_free(&A); csc_free(&At);
}

/* `steps` reflected Halpern PDHG iterations on an already equilibrated problem. No reference
 * counterpart: the reference runs PDHG with averaging only. This is the published restarted
 * Halpern PDHG for LP (H. Lu and J. Yang, "cuPDLPx", 2025: Halpern's iteration on the
 * reflected PDHG map) as the engine's SG_ALGORITHM_HALPERN runs it, in plain FP64 for the
 * step-level parity of its kernels. With T the PDHG map in primal-first order,
 *   v^ = proj(v - tau (cost + [A -I]'y)),   y^ = y + sigma [A -I] (2 v^ - v),
 * one iteration is z+ = R + w (z0 - R), R = 2 T(z) - z, w = 1 / (k + 2), k += 1.
 * v (n + m), y (m): the current iterate z, updated in place; v0, y0: the anchor z0;
 * v_hat, y_hat: T(z) of the last step. */
void orc_halpern_steps(int m, int n, const int64_t* colptr, const int32_t* rowidx,
                       const double* vals, const double* cost, const double* lower,
                       const double* upper, double tau, double sigma, int steps, long long k,
                       double* v, double* y, const double* v0, const double* y0, double* v_hat,
                       double* y_hat) {
  const int nt = n + m;
  csc_t A = csc_copy(m, n, colptr, rowidx, vals);
  double* refl = (double*)xmalloc((size_t)nt, sizeof(double));
  double* res = (double*)xmalloc((size_t)m, sizeof(double));
  for (int s = 0; s < steps; ++s) {
    /* Primal half: structurals from A'y (column sums), logicals from -y. */
    for (int j = 0; j < n; ++j) {
      double aty = 0.0;
      for (int64_t p = A.start[j]; p < A.start[j + 1]; ++p) aty += A.value[p] * y[A.index[p]];
      double val = v[j] - tau * (cost[j] + aty);
      if (lower[j] > -ORC_INF && val < lower[j]) val = lower[j];
      if (upper[j] < ORC_INF && val > upper[j]) val = upper[j];
      v_hat[j] = val;
    }
    for (int i = 0; i < m; ++i) {
      double val = v[n + i] - tau * (cost[n + i] - y[i]);
      if (lower[n + i] > -ORC_INF && val < lower[n + i]) val = lower[n + i];
      if (upper[n + i] < ORC_INF && val > upper[n + i]) val = upper[n + i];
      v_hat[n + i] = val;
    }
    for (int q = 0; q < nt; ++q) refl[q] = 2.0 * v_hat[q] - v[q];
    /* Dual half at the reflected primal point. */
    for (int i = 0; i < m; ++i) res[i] = 0.0;
    for (int j = 0; j < n; ++j) {
      for (int64_t p = A.start[j]; p < A.start[j + 1]; ++p) res[A.index[p]] += A.value[p] * refl[j];
    }
    const double w = 1.0 / (double)(k + 2);
    for (int i = 0; i < m; ++i) {
      y_hat[i] = y[i] + sigma * (res[i] - refl[n + i]);
      const double ry = 2.0 * y_hat[i] - y[i];
      y[i] = ry + w * (y0[i] - ry);
    }
    for (int q = 0; q < nt; ++q) v[q] = refl[q] + w * (v0[q] - refl[q]);
    ++k;
  }
  free(refl); free(res);
  csc_free(&A);
}

/* The seven evaluation sums of an iterate (scaled v: n + m, y: m) of the problem whose
 * original (pre-Ruiz) data is given, with the Ruiz factors cs (n) and rs (m). out[7] in the
 * order primal_sq, dual_sq, primal_obj, dual_obj, x_sq, r_sq, y_sq. */
void orc_eval_sums(int m, int n, const int64_t* colptr, const int32_t* rowidx, const double* vals,
                   const double* cost, const double* lower, const double* upper,
                   const double* cs, const double* rs, const double* v, const double* y,
                   double* out) {
  csc_t A = csc_copy(m, n, colptr, rowidx, vals);
  csc_t At = csc_transpose(&A);
  eval_ctx e;
  e.m = m; e.n = n; e.A = &A; e.At = &At;
  e.cost = cost; e.lower = lower; e.upper = upper; e.cs = cs; e.rs = rs;
  e.x_orig = (double*)xmalloc((size_t)n, sizeof(double));
  e.r_orig = (double*)xmalloc((size_t)m, sizeof(double));
  e.y_orig = (double*)xmalloc((size_t)m, sizeof(double));
  e.ax = (double*)xmalloc((size_t)m, sizeof(double));
  e.aty = (double*)xmalloc((size_t)(n + m), sizeof(double));
  sums_t s = eval_sums(&e, v, y);
  out[0] = s.primal_sq; out[1] = s.dual_sq; out[2] = s.primal_obj; out[3] = s.dual_obj;
  out[4] = s.x_sq; out[5] = s.r_sq; out[6] = s.y_sq;
  free(e.x_orig); free(e.r_orig); free(e.y_orig); free(e.ax); free(e.aty);
  csc_free(&A); csc_free(&At);
}

/* ------------------------------------------------------------------------------------------ */
/* The reference's independent solution check for an LP (src/verify/verify.cpp:50-249,
 * verify_primal + verify_kkt without Q, quadratic rows or integrality): bounds, row activities
 * and reduced costs d = c - A'y recomputed from the model in double-double arithmetic (sums of
 * pairs with Knuth's two-sum, products exact with fma), relative violations as there:
 *   bound / row:  (lo - v) / (1 + max(|lo|, scale)), scale = largest |a_ij x_j| of the row
 *   column dual:  sense d_j allowed only towards the bound x_j sits at, / (1 + |c_j| + sum |a_ij y_i|)
 *   row dual:     sense y_i likewise for the row activity, / (1 + |y_i|)
 * Returns 1 when every violation is within its tolerance. out[0..3] = max bound violation,
 * max row violation, max dual violation, objective (offset + c'x). */

typedef struct {
  double hi, lo;
} dd_t;

static dd_t dd_add_d(dd_t a, double b) {
  double s = a.hi + b;
  double bb = s - a.hi;
  double err = (a.hi - (s - bb)) + (b - bb);
  err += a.lo;
  double hi = s + err;
  dd_t r = {hi, err - (hi - s)};
  return r;
}

static dd_t dd_add(dd_t a, dd_t b) {
  dd_t r = dd_add_d(a, b.hi);
  return dd_add_d(r, b.lo);
}

static dd_t dd_prod(double a, double b) {
  double p = a * b;
  dd_t r = {p, fma(a, b, -p)};
  return r;
}

static double dd_val(dd_t a) { return a.hi + a.lo; }

static double bound_violation(double v, double lo, double up, double scale) {
  double viol = 0.0;
  if (v < lo) viol = (lo - v) / (1.0 + fmax(fabs(lo), scale));
  if (v > up) viol = (v - up) / (1.0 + fmax(fabs(up), scale));
  return viol;
}

static int at_bound(double v, double bound, double scale, double tol) {
  return isfinite(bound) && fabs(v - bound) <= tol * (1.0 + fmax(fabs(bound), scale));
}

int orc_verify_lp(int m, int n, const int64_t* colptr, const int32_t* rowidx, const double* vals,
                  const double* obj, double offset, const double* col_lower,
                  const double* col_upper, const double* row_lower, const double* row_upper,
                  int maximize, const double* x, const double* y, double tol_primal,
                  double tol_dual, double* out) {
  int ok = 1;
  double max_bound = 0.0, max_row = 0.0, max_dual = 0.0;
  for (int j = 0; j < n; ++j) {
    if (!isfinite(x[j])) { ok = 0; continue; }
    double v = bound_violation(x[j], col_lower[j], col_upper[j], 0.0);
    max_bound = fmax(max_bound, v);
    if (v > tol_primal) ok = 0;
  }
  dd_t* act = (dd_t*)xmalloc((size_t)(m > 0 ? m : 1), sizeof(dd_t));
  double* mag = (double*)xmalloc((size_t)(m > 0 ? m : 1), sizeof(double));
  for (int i = 0; i < m; ++i) { act[i].hi = act[i].lo = 0.0; mag[i] = 0.0; }
  const double sense = maximize ? -1.0 : 1.0;
  for (int j = 0; j < n; ++j) {
    dd_t d = {obj[j], 0.0};
    double scale = fabs(obj[j]);
    for (int64_t p = colptr[j]; p < colptr[j + 1]; ++p) {
      const int i = rowidx[p];
      dd_t t = dd_prod(vals[p], y[i]);
      t.hi = -t.hi;
      t.lo = -t.lo;
      d = dd_add(d, t);
      scale += fabs(vals[p] * y[i]);
      dd_t a = dd_prod(vals[p], x[j]);
      act[i] = dd_add(act[i], a);
      mag[i] = fmax(mag[i], fabs(vals[p] * x[j]));
    }
    const double dj = sense * dd_val(d);
    if (!isfinite(dj) || !isfinite(scale)) { ok = 0; max_dual = ORC_INF; continue; }
    const int lower = at_bound(x[j], col_lower[j], 0.0, tol_primal);
    const int upper = at_bound(x[j], col_upper[j], 0.0, tol_primal);
    double viol = 0.0;
    if (!lower) viol = fmax(viol, dj);
    if (!upper) viol = fmax(viol, -dj);
    viol /= 1.0 + scale;
    max_dual = fmax(max_dual, viol);
    if (viol > tol_dual) ok = 0;
  }
  for (int i = 0; i < m; ++i) {
    const double r = dd_val(act[i]);
    if (!isfinite(r) || !isfinite(mag[i]) || !isfinite(y[i])) { ok = 0; max_row = ORC_INF; continue; }
    double v = bound_violation(r, row_lower[i], row_upper[i], mag[i]);
    max_row = fmax(max_row, v);
    if (v > tol_primal) ok = 0;
    const double yi = sense * y[i];
    const int lower = at_bound(r, row_lower[i], mag[i], tol_primal);
    const int upper = at_bound(r, row_upper[i], mag[i], tol_primal);
    double viol = 0.0;
    if (!lower) viol = fmax(viol, yi);
    if (!upper) viol = fmax(viol, -yi);
    viol /= 1.0 + fabs(yi);
    max_dual = fmax(max_dual, viol);
    if (viol > tol_dual) ok = 0;
  }
  dd_t objective = {offset, 0.0};
  for (int j = 0; j < n; ++j) objective = dd_add(objective, dd_prod(obj[j], x[j]));
  out[0] = max_bound;
  out[1] = max_row;
  out[2] = max_dual;
  out[3] = dd_val(objective);
  free(act);
  free(mag);
  return ok;
}
