/*
 * qp_oracle.c -- CPU restatement of SANKHYA's convex-QP engine (Condat-Vu). TEST
 * INFRASTRUCTURE: a checker for the GPU QP engine, never part of it. See qp_oracle.h for the
 * functions, the reference lines each one follows and how the restatement is pinned.
 */
#include "qp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static int qp_finite_bound(double v) { return !(isinf(v) || fabs(v) >= 1e30); }

/* src/qp/qp_condat_vu.cpp:60-64 */
static double qp_project(double value, double lower, double upper) {
  if (qp_finite_bound(lower) && value < lower) return lower;
  if (qp_finite_bound(upper) && value > upper) return upper;
  return value;
}

/* std::max semantics: a NaN second argument leaves the first. */
static double qp_max(double a, double b) { return (a < b) ? b : a; }

static double qp_now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int64_t hessian_nonzeros(const orc_qp* qp) {
  if (qp->hessian_starts == NULL) return 0;
  return qp->hessian_starts[qp->lp.cols];
}

/* y += A x, the column scatter of SparseMatrix::multiply_add (src/la/sparse.cpp:232-242):
 * columns in order, a zero x_j skipped, each entry added to its row in storage order. */
static void multiply_add(const orc_lp* lp, const double* x, double* y) {
  for (int32_t j = 0; j < lp->cols; ++j) {
    const double xj = 1.0 * x[j];
    if (xj == 0.0) continue;
    for (int32_t k = lp->col_starts[j]; k < lp->col_starts[j + 1]; ++k) {
      y[lp->row_index[k]] += lp->values[k] * xj;
    }
  }
}

/* y += A^T x, the per-column gather of SparseMatrix::transpose_multiply_add
 * (src/la/sparse.cpp:244-259). */
static void transpose_multiply_add(const orc_lp* lp, const double* x, double* y) {
  for (int32_t j = 0; j < lp->cols; ++j) {
    double dot = 0.0;
    for (int32_t k = lp->col_starts[j]; k < lp->col_starts[j + 1]; ++k) {
      dot += lp->values[k] * x[lp->row_index[k]];
    }
    y[j] += 1.0 * dot;
  }
}

double orc_qp_spectral_norm(int32_t rows, int32_t cols, const int32_t* col_starts,
                            const int32_t* row_index, const double* values, uint32_t seed) {
  if (rows == 0 || cols == 0 || col_starts[cols] == 0) return 0.0;
  orc_lp a;
  memset(&a, 0, sizeof(a));
  a.rows = rows;
  a.cols = cols;
  a.col_starts = col_starts;
  a.row_index = row_index;
  a.values = values;
  double* v = (double*)malloc(sizeof(double) * (size_t)cols);
  double* av = (double*)malloc(sizeof(double) * (size_t)rows);
  orc_power_start(26119u + seed, cols, v);
  double estimate = 0.0;
  for (int iteration = 0; iteration < 20; ++iteration) {
    double norm = 0.0;
    for (int32_t j = 0; j < cols; ++j) norm += v[j] * v[j];
    norm = sqrt(norm);
    if (norm <= 0.0) {
      estimate = 0.0;
      break;
    }
    for (int32_t j = 0; j < cols; ++j) v[j] /= norm;
    for (int32_t i = 0; i < rows; ++i) av[i] = 0.0;
    multiply_add(&a, v, av);
    for (int32_t j = 0; j < cols; ++j) v[j] = 0.0;
    transpose_multiply_add(&a, av, v);
    double next = 0.0;
    for (int32_t j = 0; j < cols; ++j) next += v[j] * v[j];
    estimate = sqrt(sqrt(next));
  }
  free(v);
  free(av);
  return estimate;
}

void orc_qp_hessian_multiply(const orc_qp* qp, const double* x, double* out) {
  const int32_t n = qp->lp.cols;
  for (int32_t j = 0; j < n; ++j) out[j] = 0.0;
  if (qp->hessian_starts == NULL) return;
  for (int32_t j = 0; j < n; ++j) {
    for (int32_t k = qp->hessian_starts[j]; k < qp->hessian_starts[j + 1]; ++k) {
      const int32_t i = qp->hessian_index[k];
      const double value = qp->hessian_values[k];
      out[i] += value * x[j];
      if (i != j) out[j] += value * x[i];
    }
  }
}

double orc_qp_hessian_norm(const orc_qp* qp, uint32_t seed) {
  const int32_t n = qp->lp.cols;
  if (hessian_nonzeros(qp) == 0 || n == 0) return 0.0;
  double* v = (double*)malloc(sizeof(double) * (size_t)n);
  double* qv = (double*)malloc(sizeof(double) * (size_t)n);
  orc_power_start(20260826u + seed, n, v);
  double estimate = 0.0;
  for (int iteration = 0; iteration < 20; ++iteration) {
    double norm = 0.0;
    for (int32_t j = 0; j < n; ++j) norm += v[j] * v[j];
    norm = sqrt(norm);
    if (norm <= 0.0) {
      estimate = 0.0;
      break;
    }
    for (int32_t j = 0; j < n; ++j) v[j] /= norm;
    orc_qp_hessian_multiply(qp, v, qv);
    double next = 0.0;
    for (int32_t i = 0; i < n; ++i) next += qv[i] * v[i];
    estimate = fabs(next);
    memcpy(v, qv, sizeof(double) * (size_t)n);
  }
  free(v);
  free(qv);
  return estimate;
}

double orc_qp_objective(const orc_qp* qp, const double* x) {
  const orc_lp* lp = &qp->lp;
  double linear = lp->objective_offset;
  for (int32_t j = 0; j < lp->cols; ++j) linear += lp->col_cost[j] * x[j];
  if (hessian_nonzeros(qp) == 0) return linear;
  double quadratic = 0.0;
  for (int32_t j = 0; j < lp->cols; ++j) {
    for (int32_t k = qp->hessian_starts[j]; k < qp->hessian_starts[j + 1]; ++k) {
      const int32_t i = qp->hessian_index[k];
      const double v = qp->hessian_values[k];
      quadratic += (i == j) ? 0.5 * v * x[i] * x[j] : v * x[i] * x[j];
    }
  }
  return linear + quadratic;
}

int32_t orc_solve_qp(const orc_qp* qp, const orc_qp_params* params, orc_qp_result* result,
                     double* col_value, double* col_dual, double* row_dual) {
  const double t0 = qp_now();
  const orc_lp* lp = &qp->lp;
  const int32_t n = lp->cols, m = lp->rows;
  const double sense = lp->sense;
  memset(result, 0, sizeof(*result));
  result->primal_residual = -1.0;
  result->dual_residual = -1.0;

  /* Step sizes: src/qp/qp_condat_vu.cpp:195-208. */
  const uint32_t seed = (uint32_t)params->random_seed;
  const double norm_a = orc_qp_spectral_norm(m, n, lp->col_starts, lp->row_index, lp->values,
                                             seed);
  const double norm_q = orc_qp_hessian_norm(qp, seed);
  const double margin = 1.05;
  const double l = margin * norm_q;
  const double a2 = margin * margin * qp_max(norm_a * norm_a, 1e-12);
  const double tau = 1.0 / (l / 2.0 + sqrt(a2) + 1e-12);
  const double sigma = (m > 0) ? (1.0 / tau - l / 2.0) / (2.0 * a2) : 0.0;
  result->norm_a = norm_a;
  result->norm_q = norm_q;
  result->tau = tau;
  result->sigma = sigma;

  /* Iterates: src/qp/qp_condat_vu.cpp:213-225. */
  double* x = (double*)calloc((size_t)n + 1, sizeof(double));
  double* x_next = (double*)calloc((size_t)n + 1, sizeof(double));
  double* extrapolated = (double*)calloc((size_t)n + 1, sizeof(double));
  double* qx = (double*)calloc((size_t)n + 1, sizeof(double));
  double* at_y = (double*)calloc((size_t)n + 1, sizeof(double));
  double* y = (double*)calloc((size_t)m + 1, sizeof(double));
  double* ax = (double*)calloc((size_t)m + 1, sizeof(double));
  for (int32_t j = 0; j < n; ++j) x[j] = qp_project(0.0, lp->col_lower[j], lp->col_upper[j]);

  const double tolerance = params->tolerance;
  const int64_t limit = params->iteration_limit;
  const int64_t ceiling = 1000000;
  const double time_limit = params->time_limit;
  int64_t iterations = 0;
  int32_t status = ORC_ITERATION_LIMIT;

  /* The loop: src/qp/qp_condat_vu.cpp:236-335. */
  for (;;) {
    if (time_limit < 1e300 && (time_limit <= 0.0 || qp_now() - t0 > time_limit)) {
      status = ORC_TIME_LIMIT;
      break;
    }
    if ((limit >= 0 && iterations >= limit) || (limit < 0 && iterations >= ceiling)) {
      status = ORC_ITERATION_LIMIT;
      result->ceiling = limit < 0;
      break;
    }
    ++iterations;
    orc_qp_hessian_multiply(qp, x, qx);
    for (int32_t j = 0; j < n; ++j) at_y[j] = 0.0;
    if (m > 0) transpose_multiply_add(lp, y, at_y);
    for (int32_t j = 0; j < n; ++j) {
      const double gradient = sense * lp->col_cost[j] + sense * qx[j] + at_y[j];
      x_next[j] = qp_project(x[j] - tau * gradient, lp->col_lower[j], lp->col_upper[j]);
      extrapolated[j] = 2.0 * x_next[j] - x[j];
    }
    if (m > 0) {
      for (int32_t i = 0; i < m; ++i) ax[i] = 0.0;
      multiply_add(lp, extrapolated, ax);
      for (int32_t i = 0; i < m; ++i) {
        const double v = y[i] + sigma * ax[i];
        y[i] = v - sigma * qp_project(v / sigma, lp->row_lower[i], lp->row_upper[i]);
      }
    }
    double* t = x;
    x = x_next;
    x_next = t;

    if (iterations % 50 != 0) continue;
    /* The stop controller's time test (src/core/stop_controller.hpp:47-56). */
    if (time_limit < 1e300 && (time_limit <= 0.0 || qp_now() - t0 > time_limit)) {
      status = ORC_TIME_LIMIT;
      break;
    }
    double primal_residual = 0.0;
    if (m > 0) {
      for (int32_t i = 0; i < m; ++i) ax[i] = 0.0;
      multiply_add(lp, x, ax);
      for (int32_t i = 0; i < m; ++i) {
        const double projected = qp_project(ax[i], lp->row_lower[i], lp->row_upper[i]);
        primal_residual = qp_max(primal_residual, fabs(ax[i] - projected));
      }
    }
    orc_qp_hessian_multiply(qp, x, qx);
    for (int32_t j = 0; j < n; ++j) at_y[j] = 0.0;
    if (m > 0) transpose_multiply_add(lp, y, at_y);
    double dual_residual = 0.0;
    for (int32_t j = 0; j < n; ++j) {
      const double gradient = sense * lp->col_cost[j] + sense * qx[j] + at_y[j];
      const double stepped = qp_project(x[j] - gradient, lp->col_lower[j], lp->col_upper[j]);
      dual_residual = qp_max(dual_residual, fabs(x[j] - stepped));
    }
    result->primal_residual = primal_residual;
    result->dual_residual = dual_residual;
    if (primal_residual <= tolerance && dual_residual <= tolerance) {
      status = ORC_OPTIMAL;
      break;
    }
  }

  /* The reported point: src/qp/qp_condat_vu.cpp:341-361. */
  result->status = status;
  result->iterations = iterations;
  orc_qp_hessian_multiply(qp, x, qx);
  for (int32_t j = 0; j < n; ++j) at_y[j] = 0.0;
  if (m > 0) transpose_multiply_add(lp, y, at_y);
  if (col_value != NULL) memcpy(col_value, x, sizeof(double) * (size_t)n);
  if (row_dual != NULL) {
    for (int32_t i = 0; i < m; ++i) row_dual[i] = -sense * y[i];
  }
  if (col_dual != NULL) {
    for (int32_t j = 0; j < n; ++j) col_dual[j] = lp->col_cost[j] + qx[j] + sense * at_y[j];
  }
  result->objective = orc_qp_objective(qp, x);
  result->solve_seconds = qp_now() - t0;
  free(x);
  free(x_next);
  free(extrapolated);
  free(qx);
  free(at_y);
  free(y);
  free(ax);
  return status;
}
