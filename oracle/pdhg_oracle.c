/*
 * pdhg_oracle.c -- CPU restatement of SANKHYA's restarted PDHG (TEST INFRASTRUCTURE ONLY).
 *
 * What the checker restates, and where the reference states it, is listed in
 * pdhg_oracle.h. The arithmetic is written in the same order as the reference's so that an
 * x86-64 build of the reference and this file produce the same bits; the only deliberate
 * difference is that the iteration log and profiler scopes are not reproduced.
 */
#define _POSIX_C_SOURCE 200809L
#include "pdhg_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ---- Bound helpers: include/sankhya/types.hpp:86-96 ------------------------------------- */
static int is_infinite_value(double v) { return isinf(v) || fabs(v) >= 1e30; }
static int is_finite_bound(double v) { return !is_infinite_value(v); }

/* src/pdhg/pdhg.cpp:68-72 */
static double project(double value, double lower, double upper) {
  if (is_finite_bound(lower) && value < lower) return lower;
  if (is_finite_bound(upper) && value > upper) return upper;
  return value;
}

/* std::max / std::min / std::clamp with the standard's comparison order. */
static double dmax(double a, double b) { return (a < b) ? b : a; }
static double dmin(double a, double b) { return (b < a) ? b : a; }
static double dclamp(double v, double lo, double hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

static double now_seconds(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ---- Sparse products: src/la/sparse.cpp:232-269 ----------------------------------------- */
void orc_multiply(int32_t rows, int32_t cols, const int32_t* cs, const int32_t* ri,
                  const double* v, const double* x, double* y) {
  for (int32_t i = 0; i < rows; ++i) y[i] = 0.0;
  for (int32_t j = 0; j < cols; ++j) {
    const double xj = 1.0 * x[j];
    if (xj == 0.0) continue;
    for (int32_t k = cs[j]; k < cs[j + 1]; ++k) y[ri[k]] += v[k] * xj;
  }
}

static void transpose_multiply_add(int32_t cols, const int32_t* cs, const int32_t* ri,
                                   const double* v, const double* x, double* y) {
  /* One gather per column, so the result is the same at any thread count; the reference
   * parallelises this loop the same way (src/la/sparse.cpp:246-250). */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int32_t j = 0; j < cols; ++j) {
    double dot = 0.0;
    for (int32_t k = cs[j]; k < cs[j + 1]; ++k) dot += v[k] * x[ri[k]];
    y[j] += 1.0 * dot;
  }
}

void orc_transpose_multiply(int32_t rows, int32_t cols, const int32_t* cs, const int32_t* ri,
                            const double* v, const double* x, double* y) {
  (void)rows;
  for (int32_t j = 0; j < cols; ++j) y[j] = 0.0;
  transpose_multiply_add(cols, cs, ri, v, x, y);
}

/* src/pdhg/pdhg_evaluate.cpp:23-27 */
static double euclidean_norm(const double* v, int64_t count) {
  double s = 0.0;
  for (int64_t k = 0; k < count; ++k) s += v[k] * v[k];
  return sqrt(s);
}

/* ---- Scaling: src/la/scaling.cpp:14-159 ------------------------------------------------- */

/* apply_pass (src/la/scaling.cpp:14-40): the rebuilt matrix keeps the pattern; each entry
 * becomes (value * row_pass[i]) * col_pass[j], summed into a zero by finalize(). */
static void apply_pass(int32_t rows, int32_t cols, const int32_t* cs, const int32_t* ri,
                       double* values, const double* row_pass, const double* col_pass,
                       double* row_scale, double* col_scale) {
  for (int32_t j = 0; j < cols; ++j) {
    const double cj = col_pass[j];
    for (int32_t k = cs[j]; k < cs[j + 1]; ++k) {
      const double entry = values[k] * row_pass[ri[k]] * cj;
      double sum = 0.0;
      sum += entry;
      values[k] = sum;
    }
  }
  for (int32_t i = 0; i < rows; ++i) row_scale[i] *= row_pass[i];
  for (int32_t j = 0; j < cols; ++j) col_scale[j] *= col_pass[j];
}

/* ruiz_round (src/la/scaling.cpp:44-72) when `sum_mode` is 0, pock_chambolle_round
 * (src/la/scaling.cpp:76-100) when it is 1. */
static void scaling_round(int32_t rows, int32_t cols, const int32_t* cs, const int32_t* ri,
                          double* values, double* row_scale, double* col_scale, int sum_mode,
                          double* row_acc, double* col_acc) {
  for (int32_t i = 0; i < rows; ++i) row_acc[i] = 0.0;
  for (int32_t j = 0; j < cols; ++j) col_acc[j] = 0.0;
  for (int32_t j = 0; j < cols; ++j) {
    for (int32_t k = cs[j]; k < cs[j + 1]; ++k) {
      const double magnitude = fabs(values[k]);
      const int32_t i = ri[k];
      if (sum_mode) {
        row_acc[i] += magnitude;
        col_acc[j] += magnitude;
      } else {
        row_acc[i] = dmax(row_acc[i], magnitude);
        col_acc[j] = dmax(col_acc[j], magnitude);
      }
    }
  }
  for (int32_t i = 0; i < rows; ++i) row_acc[i] = row_acc[i] > 0.0 ? 1.0 / sqrt(row_acc[i]) : 1.0;
  for (int32_t j = 0; j < cols; ++j) col_acc[j] = col_acc[j] > 0.0 ? 1.0 / sqrt(col_acc[j]) : 1.0;
  apply_pass(rows, cols, cs, ri, values, row_acc, col_acc, row_scale, col_scale);
}

/* scale_bound (src/la/scaling.cpp:105-107) */
static double scale_bound(double bound, double multiplier) {
  return is_finite_bound(bound) ? bound * multiplier : bound;
}

void orc_build_scaling(const orc_lp* lp, const double* min_space_cost, int32_t ruiz_iterations,
                       double* scaled_values, double* row_scale, double* col_scale,
                       double* scaled_cost, double* scaled_col_lower, double* scaled_col_upper,
                       double* scaled_row_lower, double* scaled_row_upper, double* min_abs,
                       double* max_abs) {
  const int32_t rows = lp->rows, cols = lp->cols;
  const int32_t nnz = lp->col_starts[cols];
  memcpy(scaled_values, lp->values, sizeof(double) * (size_t)nnz);
  for (int32_t i = 0; i < rows; ++i) row_scale[i] = 1.0;
  for (int32_t j = 0; j < cols; ++j) col_scale[j] = 1.0;
  double* row_acc = (double*)malloc(sizeof(double) * (size_t)(rows > 0 ? rows : 1));
  double* col_acc = (double*)malloc(sizeof(double) * (size_t)(cols > 0 ? cols : 1));
  for (int32_t pass = 0; pass < ruiz_iterations; ++pass) {
    scaling_round(rows, cols, lp->col_starts, lp->row_index, scaled_values, row_scale, col_scale,
                  0, row_acc, col_acc);
  }
  scaling_round(rows, cols, lp->col_starts, lp->row_index, scaled_values, row_scale, col_scale, 1,
                row_acc, col_acc);
  free(row_acc);
  free(col_acc);

  for (int32_t j = 0; j < cols; ++j) {
    const double dc = col_scale[j];
    scaled_cost[j] = min_space_cost[j] * dc;
    scaled_col_lower[j] = scale_bound(lp->col_lower[j], 1.0 / dc);
    scaled_col_upper[j] = scale_bound(lp->col_upper[j], 1.0 / dc);
  }
  for (int32_t i = 0; i < rows; ++i) {
    const double dr = row_scale[i];
    scaled_row_lower[i] = scale_bound(lp->row_lower[i], dr);
    scaled_row_upper[i] = scale_bound(lp->row_upper[i], dr);
  }
  double mx = 0.0, mn = 0.0;
  int first = 1;
  for (int32_t k = 0; k < nnz; ++k) {
    const double magnitude = fabs(scaled_values[k]);
    mx = dmax(mx, magnitude);
    if (first || magnitude < mn) {
      mn = magnitude;
      first = 0;
    }
  }
  *min_abs = mn;
  *max_abs = mx;
}

/* ---- std::mt19937 and std::uniform_real_distribution<double>(-1, 1) ----------------------
 * MT19937 is Matsumoto & Nishimura (1998); the double is the C++ standard's
 * generate_canonical<double, 53> over two 32-bit draws as libstdc++ implements it, then
 * a + (b - a) * r. These reproduce src/la/scaling.cpp:168-171 exactly. */
typedef struct {
  uint32_t mt[624];
  int index;
} mt19937;

static void mt_seed(mt19937* g, uint32_t seed) {
  g->mt[0] = seed;
  for (int i = 1; i < 624; ++i) {
    g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
  }
  g->index = 624;
}

static uint32_t mt_next(mt19937* g) {
  if (g->index >= 624) {
    for (int i = 0; i < 624; ++i) {
      const uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
      g->mt[i] = g->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    g->index = 0;
  }
  uint32_t y = g->mt[g->index++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= (y >> 18);
  return y;
}

static double mt_uniform_pm1(mt19937* g) {
  const double r = 4294967296.0; /* 2^32 */
  double sum = 0.0, tmp = 1.0;
  for (int k = 0; k < 2; ++k) {
    sum += (double)mt_next(g) * tmp;
    tmp *= r;
  }
  double ret = sum / tmp;
  if (ret >= 1.0) ret = nextafter(1.0, 0.0);
  return ret * (1.0 - (-1.0)) + (-1.0);
}

void orc_power_start(uint32_t seed, int32_t count, double* out) {
  mt19937 g;
  mt_seed(&g, seed);
  for (int32_t k = 0; k < count; ++k) out[k] = mt_uniform_pm1(&g);
}

double orc_spectral_norm(int32_t rows, int32_t cols, const int32_t* cs, const int32_t* ri,
                         const double* values, int32_t iterations, uint32_t seed) {
  if (rows == 0 || cols == 0 || cs[cols] == 0) return 1.0;
  double* v = (double*)malloc(sizeof(double) * (size_t)cols);
  double* av = (double*)malloc(sizeof(double) * (size_t)rows);
  orc_power_start(seed, cols, v);
  double norm = 0.0;
  for (int32_t step = 0; step < iterations; ++step) {
    double length = 0.0;
    for (int32_t j = 0; j < cols; ++j) length += v[j] * v[j];
    length = sqrt(length);
    if (length == 0.0) {
      free(v);
      free(av);
      return 1.0;
    }
    for (int32_t j = 0; j < cols; ++j) v[j] /= length;
    orc_multiply(rows, cols, cs, ri, values, v, av);
    orc_transpose_multiply(rows, cols, cs, ri, values, av, v);
    double next = 0.0;
    for (int32_t j = 0; j < cols; ++j) next += v[j] * v[j];
    norm = sqrt(sqrt(next));
  }
  free(v);
  free(av);
  return norm > 0.0 ? norm * 1.01 : 1.0;
}

/* ---- Evaluation: src/pdhg/pdhg_evaluate.cpp:29-139 --------------------------------------- */
typedef struct {
  const orc_lp* lp;
  const double* cost; /* minimise-space */
  double bound_norm;
  double cost_norm;
} problem_t;

static double worst(const orc_residuals* r) {
  double w = r->primal;
  if (w < r->dual) w = r->dual;
  if (w < r->gap) w = r->gap;
  return w;
}

/* include/sankhya/tolerances.hpp:19,22,108 and src/pdhg/pdhg_evaluate.hpp:57-69 */
static int meets_request(const orc_residuals* r, double tolerance) {
  return r->primal <= tolerance && r->dual <= tolerance && r->gap <= tolerance &&
         r->absolute_primal <= 1e-7;
}
static int meets_project_standard(const orc_residuals* r) {
  return r->absolute_primal <= 1e-7 && r->absolute_dual <= 1e-7 && r->gap_as_verified <= 1e-9 &&
         r->complementarity <= 1e-6;
}

static orc_residuals evaluate(const problem_t* p, const double* x, const double* y,
                              double* activity, double* reduced) {
  const orc_lp* lp = p->lp;
  const int32_t rows = lp->rows, cols = lp->cols;
  orc_residuals r;
  memset(&r, 0, sizeof(r));

  if (rows > 0) {
    orc_multiply(rows, cols, lp->col_starts, lp->row_index, lp->values, x, activity);
  }
  double primal_violation = 0.0;
  for (int32_t i = 0; i < rows; ++i) {
    const double a = activity[i];
    double violation = 0.0;
    if (is_finite_bound(lp->row_lower[i])) violation = dmax(violation, lp->row_lower[i] - a);
    if (is_finite_bound(lp->row_upper[i])) violation = dmax(violation, a - lp->row_upper[i]);
    primal_violation += violation * violation;
  }
  r.absolute_primal = sqrt(primal_violation);
  r.primal = r.absolute_primal / (1.0 + p->bound_norm);

  for (int32_t j = 0; j < cols; ++j) reduced[j] = p->cost[j];
  if (rows > 0) transpose_multiply_add(cols, lp->col_starts, lp->row_index, lp->values, y, reduced);

  double dual_violation = 0.0;
  double bound_contribution = 0.0;
  for (int32_t j = 0; j < cols; ++j) {
    const double d = reduced[j];
    if (d > 0.0) {
      if (is_finite_bound(lp->col_lower[j])) {
        bound_contribution += d * lp->col_lower[j];
      } else {
        dual_violation += d * d;
      }
    } else if (d < 0.0) {
      if (is_finite_bound(lp->col_upper[j])) {
        bound_contribution += d * lp->col_upper[j];
      } else {
        dual_violation += d * d;
      }
    }
  }
  double support = 0.0;
  for (int32_t i = 0; i < rows; ++i) {
    const double yi = y[i];
    if (yi > 0.0) {
      if (is_finite_bound(lp->row_upper[i])) {
        support += yi * lp->row_upper[i];
      } else {
        dual_violation += yi * yi;
      }
    } else if (yi < 0.0) {
      if (is_finite_bound(lp->row_lower[i])) {
        support += yi * lp->row_lower[i];
      } else {
        dual_violation += yi * yi;
      }
    }
  }
  r.absolute_dual = sqrt(dual_violation);
  r.dual = r.absolute_dual / (1.0 + p->cost_norm);

  for (int32_t i = 0; i < rows; ++i) {
    if (lp->row_lower[i] == lp->row_upper[i]) continue;
    const double lower_slack =
        is_finite_bound(lp->row_lower[i]) ? activity[i] - lp->row_lower[i] : INFINITY;
    const double upper_slack =
        is_finite_bound(lp->row_upper[i]) ? lp->row_upper[i] - activity[i] : INFINITY;
    r.complementarity = dmax(r.complementarity, fabs(y[i]) * dmin(lower_slack, upper_slack));
  }
  for (int32_t j = 0; j < cols; ++j) {
    if (lp->col_lower[j] == lp->col_upper[j]) continue;
    const double lower_slack =
        is_finite_bound(lp->col_lower[j]) ? x[j] - lp->col_lower[j] : INFINITY;
    const double upper_slack =
        is_finite_bound(lp->col_upper[j]) ? lp->col_upper[j] - x[j] : INFINITY;
    r.complementarity = dmax(r.complementarity, fabs(reduced[j]) * dmin(lower_slack, upper_slack));
  }

  double primal_objective = 0.0;
  for (int32_t j = 0; j < cols; ++j) primal_objective += p->cost[j] * x[j];
  r.primal_objective = primal_objective;
  r.dual_objective = bound_contribution - support;
  const double absolute_gap = fabs(r.primal_objective - r.dual_objective);
  r.gap = absolute_gap / (1.0 + fabs(r.primal_objective) + fabs(r.dual_objective));
  r.gap_as_verified = absolute_gap / dmax(1.0, fabs(r.primal_objective));
  return r;
}

orc_residuals orc_evaluate(const orc_lp* lp, const double* x, const double* y, double* activity,
                           double* reduced) {
  const int32_t rows = lp->rows, cols = lp->cols;
  double* cost = (double*)malloc(sizeof(double) * (size_t)(cols > 0 ? cols : 1));
  for (int32_t j = 0; j < cols; ++j) cost[j] = lp->sense * lp->col_cost[j];
  problem_t p;
  p.lp = lp;
  p.cost = cost;
  p.cost_norm = euclidean_norm(cost, cols);
  double bound_square = 0.0;
  for (int32_t i = 0; i < rows; ++i) {
    const double b = is_finite_bound(lp->row_lower[i])
                         ? lp->row_lower[i]
                         : (is_finite_bound(lp->row_upper[i]) ? lp->row_upper[i] : 0.0);
    bound_square += b * b;
  }
  p.bound_norm = sqrt(bound_square);
  orc_residuals r = evaluate(&p, x, y, activity, reduced);
  free(cost);
  return r;
}

/* Model::validate's numeric checks (src/core/model.cpp:127-240): every matrix value finite
 * (:178), no NaN bound and no crossed bound (:210-224), no NaN cost (:214) and no NaN
 * objective offset (:228). An infinite cost passes, as it does there. */
static int model_is_valid(const orc_lp* lp) {
  const int32_t nnz = lp->col_starts[lp->cols];
  for (int32_t k = 0; k < nnz; ++k) {
    if (!isfinite(lp->values[k])) return 0;
  }
  for (int32_t j = 0; j < lp->cols; ++j) {
    if (isnan(lp->col_lower[j]) || isnan(lp->col_upper[j])) return 0;
    if (lp->col_lower[j] > lp->col_upper[j]) return 0;
    if (isnan(lp->col_cost[j])) return 0;
  }
  for (int32_t i = 0; i < lp->rows; ++i) {
    if (isnan(lp->row_lower[i]) || isnan(lp->row_upper[i])) return 0;
    if (lp->row_lower[i] > lp->row_upper[i]) return 0;
  }
  if (isnan(lp->objective_offset)) return 0;
  return 1;
}

/* ---- The engine: src/pdhg/pdhg.cpp:76-568 ----------------------------------------------- */
#define ALLOC(T, count) ((T*)calloc((size_t)((count) > 0 ? (count) : 1), sizeof(T)))

int32_t orc_solve_pdhg(const orc_lp* lp, const orc_params* params, orc_result* result,
                       double* col_value, double* col_dual, double* row_dual) {
  const double t0 = now_seconds();
  memset(result, 0, sizeof(*result));
  const int32_t rows = lp->rows, cols = lp->cols;
  const int32_t nnz = lp->col_starts[cols];
  const double sense = lp->sense;

  if (!model_is_valid(lp)) {
    result->status = ORC_MODEL_ERROR;
    return result->status;
  }

  /* Unscaled minimise-space problem, pdhg.cpp:95-111. */
  double* cost = ALLOC(double, cols);
  for (int32_t j = 0; j < cols; ++j) cost[j] = sense * lp->col_cost[j];
  problem_t problem;
  problem.lp = lp;
  problem.cost = cost;
  problem.cost_norm = euclidean_norm(cost, cols);
  double bound_square = 0.0;
  for (int32_t i = 0; i < rows; ++i) {
    const double b = is_finite_bound(lp->row_lower[i])
                         ? lp->row_lower[i]
                         : (is_finite_bound(lp->row_upper[i]) ? lp->row_upper[i] : 0.0);
    bound_square += b * b;
  }
  problem.bound_norm = sqrt(bound_square);

  /* Preconditioning, pdhg.cpp:114-117. */
  double* sv = ALLOC(double, nnz);
  double* dr = ALLOC(double, rows);
  double* dc = ALLOC(double, cols);
  double* sc = ALLOC(double, cols);
  double* sl = ALLOC(double, cols);
  double* su = ALLOC(double, cols);
  double* srl = ALLOC(double, rows);
  double* sru = ALLOC(double, rows);
  orc_build_scaling(lp, cost, 10, sv, dr, dc, sc, sl, su, srl, sru, &result->scaled_min_abs,
                    &result->scaled_max_abs);
  const double spectral_norm = orc_spectral_norm(rows, cols, lp->col_starts, lp->row_index, sv, 30,
                                                 (uint32_t)params->random_seed + 1u);
  result->spectral_norm = spectral_norm;

  const double tolerance = params->tolerance;
  const int64_t iteration_limit = params->iteration_limit < 0 ? 1000000 : params->iteration_limit;
  const int use_restarts = params->restart != 0;
  const int stop_at_request = params->stop_at_request != 0;
  const double time_limit = params->time_limit;

  const int32_t* cs = lp->col_starts;
  const int32_t* ri = lp->row_index;

  double* x = ALLOC(double, cols);
  double* y = ALLOC(double, rows);
  for (int32_t j = 0; j < cols; ++j) x[j] = project(0.0, sl[j], su[j]);
  double* x_next = ALLOC(double, cols);
  double* y_next = ALLOC(double, rows);
  double* extrapolated = ALLOC(double, cols);
  double* at_y = ALLOC(double, cols);
  double* a_x = ALLOC(double, rows);
  double* x_sum = ALLOC(double, cols);
  double* y_sum = ALLOC(double, rows);
  int64_t averaged = 0;
  double* x_restart = ALLOC(double, cols);
  double* y_restart = ALLOC(double, rows);
  memcpy(x_restart, x, sizeof(double) * (size_t)cols);
  memcpy(y_restart, y, sizeof(double) * (size_t)rows);
  double* activity = ALLOC(double, rows);
  double* reduced = ALLOC(double, cols);
  double* dxv = ALLOC(double, cols);
  double* adx = ALLOC(double, rows);
  double* dyv = ALLOC(double, rows);
  double* cur_x = ALLOC(double, cols);
  double* cur_y = ALLOC(double, rows);
  double* avg_x = ALLOC(double, cols);
  double* avg_y = ALLOC(double, rows);
  double* best_x = ALLOC(double, cols);
  double* best_y = ALLOC(double, rows);
  memcpy(best_x, x, sizeof(double) * (size_t)cols);
  memcpy(best_y, y, sizeof(double) * (size_t)rows);

  double eta = spectral_norm > 0.0 ? 1.0 / spectral_norm : 1.0;
  double omega = 1.0;
  int64_t iteration = 0, restarts = 0, last_restart = 0;
  double restart_kkt = INFINITY;
  orc_residuals best;
  memset(&best, 0, sizeof(best));
  best.primal = best.dual = best.gap = INFINITY;
  int converged = 0;
  int32_t stop_status = ORC_ITERATION_LIMIT;

  for (;;) {
    /* pdhg.cpp:202-205 with ResourceLimits::time_exhausted (src/core/resource_limits.cpp:72-78):
     * a limit of 1e300 or more is the "no limit" sentinel. */
    if (time_limit < 1e300 && (time_limit <= 0.0 || now_seconds() - t0 > time_limit)) {
      stop_status = ORC_TIME_LIMIT;
      break;
    }
    if (iteration >= iteration_limit) break;

    const double tau = eta / omega;
    const double sigma = eta * omega;

    /* Primal step, pdhg.cpp:226-236. */
    for (int32_t j = 0; j < cols; ++j) at_y[j] = 0.0;
    if (rows > 0) orc_transpose_multiply(rows, cols, cs, ri, sv, y, at_y);
    for (int32_t j = 0; j < cols; ++j) {
      const double gradient = sc[j] + at_y[j];
      x_next[j] = project(x[j] - tau * gradient, sl[j], su[j]);
      extrapolated[j] = 2.0 * x_next[j] - x[j];
    }
    /* Dual step, pdhg.cpp:239-247. */
    if (rows > 0) orc_multiply(rows, cols, cs, ri, sv, extrapolated, a_x);
    for (int32_t i = 0; i < rows; ++i) {
      const double v = y[i] + sigma * a_x[i];
      y_next[i] = v - sigma * project(v / sigma, srl[i], sru[i]);
    }

    /* Adaptive step, pdhg.cpp:252-335. */
    double movement = 0.0;
    for (int32_t j = 0; j < cols; ++j) {
      const double d = x_next[j] - x[j];
      movement += 0.5 * omega * d * d;
    }
    for (int32_t i = 0; i < rows; ++i) {
      const double d = y_next[i] - y[i];
      movement += 0.5 * d * d / omega;
    }
    double interaction = 0.0;
    if (rows > 0) {
      for (int32_t j = 0; j < cols; ++j) dxv[j] = x_next[j] - x[j];
      orc_multiply(rows, cols, cs, ri, sv, dxv, adx);
      for (int32_t i = 0; i < rows; ++i) interaction += (y_next[i] - y[i]) * adx[i];
      interaction = fabs(interaction);
    }
    const int no_information = interaction <= 0.0;
    const double limit = no_information ? INFINITY : movement / interaction;
    const double exponent = (double)(iteration + 1 > 2 ? iteration + 1 : 2);
    const double shrink = 1.0 - pow(exponent, -0.3);
    const double grow = 1.0 + pow(exponent, -0.6);
    const double proposed = dmin(shrink * limit, grow * eta);

    if (eta <= limit) {
      double* t = x;
      x = x_next;
      x_next = t;
      t = y;
      y = y_next;
      y_next = t;
      for (int32_t j = 0; j < cols; ++j) x_sum[j] += x[j];
      for (int32_t i = 0; i < rows; ++i) y_sum[i] += y[i];
      ++averaged;
      ++iteration;
    }
    const double eta_ceiling = 1.0e3 / dmax(spectral_norm, 1e-12);
    if (!no_information) eta = dclamp(proposed, 1e-12, eta_ceiling);

    /* Evaluation, pdhg.cpp:341-384. */
    if (iteration == 0) continue;
    if (iteration % 40 != 0 && !no_information) continue;
    result->evaluations++;

    for (int32_t j = 0; j < cols; ++j) cur_x[j] = x[j] * dc[j];
    for (int32_t i = 0; i < rows; ++i) cur_y[i] = y[i] * dr[i];
    const orc_residuals current = evaluate(&problem, cur_x, cur_y, activity, reduced);
    const orc_residuals* chosen = &current;
    const double* chosen_x = cur_x;
    const double* chosen_y = cur_y;
    orc_residuals average;
    if (averaged > 0) {
      const double count = (double)averaged;
      for (int32_t j = 0; j < cols; ++j) avg_x[j] = (x_sum[j] / count) * dc[j];
      for (int32_t i = 0; i < rows; ++i) avg_y[i] = (y_sum[i] / count) * dr[i];
      average = evaluate(&problem, avg_x, avg_y, activity, reduced);
      if (worst(&average) < worst(&current)) {
        chosen = &average;
        chosen_x = avg_x;
        chosen_y = avg_y;
      }
    }
    if (worst(chosen) < worst(&best)) {
      best = *chosen;
      memcpy(best_x, chosen_x, sizeof(double) * (size_t)cols);
      memcpy(best_y, chosen_y, sizeof(double) * (size_t)rows);
    }

    /* Stop test, pdhg.cpp:424-436. */
    if (meets_request(chosen, tolerance) && (stop_at_request || meets_project_standard(chosen))) {
      best = *chosen;
      memcpy(best_x, chosen_x, sizeof(double) * (size_t)cols);
      memcpy(best_y, chosen_y, sizeof(double) * (size_t)rows);
      converged = 1;
      break;
    }

    /* Restart and primal weight, pdhg.cpp:438-483. */
    if (use_restarts) {
      const double kkt = worst(chosen);
      const int64_t since = iteration - last_restart;
      const int sufficient = kkt <= 0.2 * restart_kkt;
      const int64_t floor_36 = (int64_t)(0.36 * (double)iteration);
      const int artificial = since >= (floor_36 > 40 ? floor_36 : 40);
      if (sufficient || artificial) {
        for (int32_t j = 0; j < cols; ++j) dxv[j] = x[j] - x_restart[j];
        for (int32_t i = 0; i < rows; ++i) dyv[i] = y[i] - y_restart[i];
        const double dx_norm = euclidean_norm(dxv, cols);
        const double dy_norm = euclidean_norm(dyv, rows);
        if (dx_norm > 1e-12 && dy_norm > 1e-12) {
          const double theta = 0.5;
          omega = exp(theta * log(dy_norm / dx_norm) + (1.0 - theta) * log(omega));
          omega = dclamp(omega, 1e-6, 1e6);
        }
        memset(x_sum, 0, sizeof(double) * (size_t)cols);
        memset(y_sum, 0, sizeof(double) * (size_t)rows);
        averaged = 0;
        memcpy(x_restart, x, sizeof(double) * (size_t)cols);
        memcpy(y_restart, y, sizeof(double) * (size_t)rows);
        restart_kkt = kkt;
        last_restart = iteration;
        ++restarts;
      }
    }
  }

  /* Report, pdhg.cpp:487-567. */
  const orc_residuals final_residuals = evaluate(&problem, best_x, best_y, activity, reduced);
  if (col_value) memcpy(col_value, best_x, sizeof(double) * (size_t)cols);
  if (col_dual) {
    for (int32_t j = 0; j < cols; ++j) col_dual[j] = sense * reduced[j];
  }
  if (row_dual) {
    for (int32_t i = 0; i < rows; ++i) row_dual[i] = sense * (-best_y[i]);
  }
  result->iterations = iteration;
  result->restarts = restarts;
  result->final_residuals = final_residuals;
  const int verifiable = converged && meets_project_standard(&final_residuals);
  if (verifiable) {
    result->status = ORC_OPTIMAL;
  } else if (converged) {
    result->status = ORC_FEASIBLE;
  } else {
    result->status = (stop_status == ORC_TIME_LIMIT || stop_status == ORC_INTERRUPTED)
                         ? stop_status
                         : ORC_ITERATION_LIMIT;
  }
  if (verifiable) {
    result->dual_bound = sense * final_residuals.dual_objective + lp->objective_offset;
  } else {
    result->dual_bound = sense < 0.0 ? INFINITY : -INFINITY;
  }
  /* Model::evaluate_objective, src/core/model.cpp:101-107. */
  double linear = lp->objective_offset;
  for (int32_t j = 0; j < cols; ++j) linear += lp->col_cost[j] * best_x[j];
  result->objective = linear;
  result->solve_seconds = now_seconds() - t0;

  free(cost); free(sv); free(dr); free(dc); free(sc); free(sl); free(su); free(srl); free(sru);
  free(x); free(y); free(x_next); free(y_next); free(extrapolated); free(at_y); free(a_x);
  free(x_sum); free(y_sum); free(x_restart); free(y_restart); free(activity); free(reduced);
  free(dxv); free(adx); free(dyv); free(cur_x); free(cur_y); free(avg_x); free(avg_y);
  free(best_x); free(best_y);
  return result->status;
}
