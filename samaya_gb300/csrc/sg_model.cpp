// Model -> LpProblem on the host (C++): the power-of-two scaling and the computational form that
// samaya applies before PDLP (reference src/linalg/scaling.cpp:130-200 compute_scaling and
// src/lp/lp_solver.cpp:28-51 make_problem), and the mapping of a PDLP answer back to the model
// (src/core/solver.cpp:415-432). The steps, passes and constants are samaya's so that the
// LpProblem handed to the engine is the one samaya's solve_pdlp receives.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/sg_pdlp.h"
#include "sg_transpose.h"

namespace {

double nearest_power_of_two(double v) {
  if (!(v > 0.0) || !std::isfinite(v)) return 1.0;
  return std::ldexp(1.0, static_cast<int>(std::lround(std::log2(v))));
}

double clamp_scale(double v) { return std::min(std::max(v, 0x1p-40), 0x1p40); }

struct Csc {
  int m, n;
  const int64_t* start;
  const int32_t* row;
  const double* val;
};

// max |a_ij| / min |a_ij| over the nonzeros of R A C.
double spread(const Csc& a, const std::vector<double>& r, const std::vector<double>& c) {
  double lo = INFINITY, hi = 0.0;
  for (int j = 0; j < a.n; ++j) {
    for (int64_t p = a.start[j]; p < a.start[j + 1]; ++p) {
      const double v = std::fabs(a.val[p]) * r[a.row[p]] * c[j];
      lo = std::min(lo, v);
      hi = std::max(hi, v);
    }
  }
  return hi > 0.0 ? hi / lo : 1.0;
}

void row_extremes(const Csc& a, const std::vector<double>& c, std::vector<double>& rmin,
                  std::vector<double>& rmax) {
  std::fill(rmin.begin(), rmin.end(), INFINITY);
  std::fill(rmax.begin(), rmax.end(), 0.0);
  for (int j = 0; j < a.n; ++j) {
    for (int64_t p = a.start[j]; p < a.start[j + 1]; ++p) {
      const double v = std::fabs(a.val[p]) * c[j];
      const int i = a.row[p];
      rmin[i] = std::min(rmin[i], v);
      rmax[i] = std::max(rmax[i], v);
    }
  }
}

}  // namespace

namespace {

// The model checks of sg_scale_model_device (sg_setup_device.cu, check_host): column starts
// from 0 and never decreasing, the matrix arrays present, every row index in range and every
// value finite (host threads), every cost finite and no bound NaN.
bool valid_model(int m, int n, const int64_t* colptr, const int32_t* rowidx, const double* val,
                 const double* obj, const double* col_lower, const double* col_upper,
                 const double* row_lower, const double* row_upper) {
  if (colptr[0] != 0) return false;
  for (int j = 0; j < n; ++j) {
    if (colptr[j + 1] < colptr[j]) return false;
  }
  const int64_t nnz = colptr[n];
  if (nnz > 0 && (rowidx == nullptr || val == nullptr)) return false;
  for (int j = 0; j < n; ++j) {
    if (!std::isfinite(obj[j]) || std::isnan(col_lower[j]) || std::isnan(col_upper[j])) {
      return false;
    }
  }
  for (int i = 0; i < m; ++i) {
    if (std::isnan(row_lower[i]) || std::isnan(row_upper[i])) return false;
  }
  const char* why = nullptr;
  return nnz == 0 || sg::check_nonzeros(m, nnz, rowidx, val, 16, &why) == 0;
}

}  // namespace

extern "C" {

/* See include/sg_pdlp.h. */
int sg_scale_model(int m, int n, const int64_t* a_colptr, const int32_t* a_rowidx,
                   const double* a_val, const double* obj, const double* col_lower,
                   const double* col_upper, const double* row_lower, const double* row_upper,
                   int maximize, int64_t* lp_colptr, int32_t* lp_rowidx, double* lp_val,
                   double* cost, double* lower, double* upper, double* col_scale,
                   double* row_scale, int64_t* lp_nnz) {
  if (m < 0 || n < 0 || a_colptr == nullptr || obj == nullptr || col_lower == nullptr ||
      col_upper == nullptr || lp_colptr == nullptr || cost == nullptr || lower == nullptr ||
      upper == nullptr || col_scale == nullptr || lp_nnz == nullptr) {
    return SG_ERR_INVALID_ARGUMENT;
  }
  if (m > 0 && (row_lower == nullptr || row_upper == nullptr || row_scale == nullptr)) {
    return SG_ERR_INVALID_ARGUMENT;
  }
  if (!valid_model(m, n, a_colptr, a_rowidx, a_val, obj, col_lower, col_upper, row_lower,
                   row_upper)) {
    return SG_ERR_INVALID_ARGUMENT;
  }
  const int64_t nnz = a_colptr[n];
  const Csc a{m, n, a_colptr, a_rowidx, a_val};
  std::vector<double> r(static_cast<size_t>(m), 1.0), c(static_cast<size_t>(n), 1.0);
  if (nnz > 0) {
    std::vector<double> rmin(static_cast<size_t>(m)), rmax(static_cast<size_t>(m));
    // Geometric-mean passes: rows, then columns, divided by sqrt(min * max) of their current
    // magnitudes; at most 10 passes, stop when a pass gains less than 10% or worsens the spread.
    double ratio = spread(a, r, c);
    for (int pass = 0; pass < 10 && ratio > 1.0; ++pass) {
      const std::vector<double> r_prev = r, c_prev = c;
      row_extremes(a, c, rmin, rmax);
      for (int i = 0; i < m; ++i) {
        if (rmax[i] > 0.0) r[i] = clamp_scale(1.0 / std::sqrt(rmin[i] * rmax[i]));
      }
      for (int j = 0; j < n; ++j) {
        double lo = INFINITY, hi = 0.0;
        for (int64_t p = a_colptr[j]; p < a_colptr[j + 1]; ++p) {
          const double v = std::fabs(a_val[p]) * r[a_rowidx[p]];
          lo = std::min(lo, v);
          hi = std::max(hi, v);
        }
        if (hi > 0.0) c[j] = clamp_scale(1.0 / std::sqrt(lo * hi));
      }
      const double next = spread(a, r, c);
      if (next > ratio) {
        r = r_prev;
        c = c_prev;
        break;
      }
      const bool small_gain = next > 0.9 * ratio;
      ratio = next;
      if (small_gain) break;
    }
    // Equilibration: every row and then every column maximum to about 1.
    row_extremes(a, c, rmin, rmax);
    for (int i = 0; i < m; ++i) {
      if (rmax[i] > 0.0) r[i] = clamp_scale(1.0 / rmax[i]);
    }
    for (int j = 0; j < n; ++j) {
      double hi = 0.0;
      for (int64_t p = a_colptr[j]; p < a_colptr[j + 1]; ++p) {
        hi = std::max(hi, std::fabs(a_val[p]) * r[a_rowidx[p]]);
      }
      if (hi > 0.0) c[j] = clamp_scale(1.0 / hi);
    }
    for (double& f : r) f = nearest_power_of_two(f);
    for (double& f : c) f = nearest_power_of_two(f);
  }
  // Computational form: min (sense c C)'x s.t. [R A C  -I] v = 0 with the scaled bounds.
  const double sense = maximize ? -1.0 : 1.0;
  int64_t k = 0;
  lp_colptr[0] = 0;
  for (int j = 0; j < n; ++j) {
    for (int64_t p = a_colptr[j]; p < a_colptr[j + 1]; ++p) {
      const double v = a_val[p] * r[a_rowidx[p]] * c[j];
      if (v != 0.0) {
        lp_rowidx[k] = a_rowidx[p];
        lp_val[k] = v;
        ++k;
      }
    }
    lp_colptr[j + 1] = k;
  }
  *lp_nnz = k;
  for (int j = 0; j < n; ++j) {
    cost[j] = sense * obj[j] * c[j];
    lower[j] = col_lower[j] / c[j];
    upper[j] = col_upper[j] / c[j];
    col_scale[j] = c[j];
  }
  for (int i = 0; i < m; ++i) {
    cost[n + i] = 0.0;
    lower[n + i] = row_lower[i] * r[i];
    upper[n + i] = row_upper[i] * r[i];
    row_scale[i] = r[i];
  }
  return SG_OK;
}

/* See include/sg_pdlp.h. */
int sg_unscale_solution(int m, int n, const double* col_scale, const double* row_scale,
                        int maximize, const double* x_lp, const double* y_lp, double* x,
                        double* row_activity, double* row_dual) {
  if (m < 0 || n < 0 || col_scale == nullptr || x_lp == nullptr ||
      (m > 0 && (row_activity != nullptr || row_dual != nullptr) && row_scale == nullptr)) {
    return SG_ERR_INVALID_ARGUMENT;
  }
  const double sense = maximize ? -1.0 : 1.0;
  for (int j = 0; j < n; ++j) {
    if (x) x[j] = x_lp[j] * col_scale[j];
  }
  for (int i = 0; i < m; ++i) {
    if (row_activity) row_activity[i] = x_lp[n + i] / row_scale[i];
    // PDLP's Lagrangian c'x + y'(Ax - r) gives reduced costs c + A'y: negated for d = c - A'y,
    // and the objective sense applied.
    if (row_dual && y_lp) row_dual[i] = -sense * (y_lp[i] * row_scale[i]);
  }
  return SG_OK;
}

}  // extern "C"
