// ref_capi.cpp -- a C entry layer over the REFERENCE's own PDHG sources, for tests only.
//
// oracle/Makefile compiles this file together with the reference's unmodified sources
// (src/pdhg, src/la/{scaling,sparse}.cpp, src/core/{model,resource_limits}.cpp, src/util/*)
// into oracle/_ref/libsankhya_ref.so. The functions mirror pdhg_oracle.h one for one so that a
// test can run the restatement and the reference on identical inputs and compare the bits.
// Nothing here is linked into the GPU engine.
//
// Two more groups hand Models that the reference's own code builds to the tests: one read by
// its MPS/LP reader (sankhya::io::read_model, src/io/lp_reader.cpp:650), one made by its test
// generator of LPs with an exact, analytically known optimum (sankhya::oracle::kkt_lp,
// tests/oracles/lp_generator.cpp:122, turned into a Model by
// tests/oracles/rational_simplex.cpp:252).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <string>
#include <vector>

#include "la/scaling.hpp"
#include "oracles/lp_generator.hpp"
#include "oracles/rational_simplex.hpp"
#include "pdhg/pdhg_evaluate.hpp"
#include "sankhya/io.hpp"
#include "sankhya/logging.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"
#include "sankhya/pdhg.hpp"
#include "sankhya/qp.hpp"
#include "qp/convexity.hpp"

#include "../pdhg_oracle.h"
#include "../qp_oracle.h"

namespace {

sankhya::Model to_model(const orc_lp* lp) {
  sankhya::Model model;
  const auto n = static_cast<std::size_t>(lp->cols);
  const auto m = static_cast<std::size_t>(lp->rows);
  model.sense = lp->sense < 0.0 ? sankhya::ObjSense::kMaximize : sankhya::ObjSense::kMinimize;
  model.objective_offset = lp->objective_offset;
  model.col_cost.assign(lp->col_cost, lp->col_cost + n);
  model.col_lower.assign(lp->col_lower, lp->col_lower + n);
  model.col_upper.assign(lp->col_upper, lp->col_upper + n);
  model.col_type.assign(n, sankhya::VarType::kContinuous);
  model.row_lower.assign(lp->row_lower, lp->row_lower + m);
  model.row_upper.assign(lp->row_upper, lp->row_upper + m);
  model.matrix.reset(lp->rows, lp->cols);
  model.matrix.reserve(static_cast<std::size_t>(lp->col_starts[lp->cols]));
  for (int32_t j = 0; j < lp->cols; ++j) {
    for (int32_t k = lp->col_starts[j]; k < lp->col_starts[j + 1]; ++k) {
      model.matrix.add_entry(lp->row_index[k], j, lp->values[k]);
    }
  }
  // Drop tolerance zero keeps every entry the caller passed, explicit zeros included, so the
  // pattern matches the CSC arrays one for one.
  model.matrix.finalize(0.0);
  return model;
}

// The Model of a QP: the LP part as to_model builds it, and the Hessian's stored triangle as
// Model::hessian (n x n CSC), entries kept one for one.
sankhya::Model to_qp_model(const orc_qp* qp) {
  sankhya::Model model = to_model(&qp->lp);
  model.hessian.reset(qp->lp.cols, qp->lp.cols);
  if (qp->hessian_starts != nullptr) {
    for (int32_t j = 0; j < qp->lp.cols; ++j) {
      for (int32_t k = qp->hessian_starts[j]; k < qp->hessian_starts[j + 1]; ++k) {
        model.hessian.add_entry(qp->hessian_index[k], j, qp->hessian_values[k]);
      }
    }
  }
  model.hessian.finalize(0.0);
  return model;
}

int32_t status_code(sankhya::SolveStatus s) {
  using S = sankhya::SolveStatus;
  switch (s) {
    case S::kNotSolved: return ORC_NOT_SOLVED;
    case S::kOptimal: return ORC_OPTIMAL;
    case S::kFeasible: return ORC_FEASIBLE;
    case S::kInfeasible: return ORC_INFEASIBLE;
    case S::kIterationLimit: return ORC_ITERATION_LIMIT;
    case S::kTimeLimit: return ORC_TIME_LIMIT;
    case S::kNumericalError: return ORC_NUMERICAL_ERROR;
    case S::kModelError: return ORC_MODEL_ERROR;
    case S::kInterrupted: return ORC_INTERRUPTED;
    default: return 100 + static_cast<int32_t>(s);
  }
}

orc_residuals to_c(const sankhya::pdhg::Residuals& r) {
  orc_residuals c;
  c.primal = r.primal;
  c.dual = r.dual;
  c.gap = r.gap;
  c.primal_objective = r.primal_objective;
  c.dual_objective = r.dual_objective;
  c.absolute_primal = r.absolute_primal;
  c.absolute_dual = r.absolute_dual;
  c.gap_as_verified = r.gap_as_verified;
  c.complementarity = r.complementarity;
  return c;
}

// The restart count is not a Solution field; the engine's message carries it
// ("... after N iterations and R restarts ...", src/pdhg/pdhg.cpp:519-548).
long long restarts_from_message(const std::string& message) {
  const std::size_t at = message.find(" iterations and ");
  if (at == std::string::npos) return -1;
  return std::atoll(message.c_str() + at + std::strlen(" iterations and "));
}

}  // namespace

extern "C" {

int32_t ref_solve_pdhg(const orc_lp* lp, const orc_params* params, orc_result* result,
                       double* col_value, double* col_dual, double* row_dual, char* message,
                       int32_t message_capacity) {
  std::memset(result, 0, sizeof(*result));
  const sankhya::Model model = to_model(lp);
  sankhya::Options options;
  options.set_bool("log_to_console", false);
  options.set_double("pdhg_tolerance", params->tolerance);
  options.set_int("iteration_limit", params->iteration_limit);
  if (params->time_limit < 1e300) options.set_double("time_limit", params->time_limit);
  options.set_bool("pdhg_restart", params->restart != 0);
  options.set_bool("pdhg_stop_at_request", params->stop_at_request != 0);
  options.set_int("random_seed", params->random_seed);
  sankhya::Logger logger(nullptr);
  const sankhya::Solution s = sankhya::pdhg::solve_pdhg(model, options, logger, nullptr);
  result->status = status_code(s.status);
  result->iterations = s.iterations;
  result->restarts = restarts_from_message(s.message);
  result->objective = s.objective;
  result->dual_bound = s.dual_bound;
  result->solve_seconds = s.solve_seconds;
  const auto n = static_cast<std::size_t>(lp->cols);
  const auto m = static_cast<std::size_t>(lp->rows);
  if (col_value != nullptr && s.col_value.size() == n) {
    std::memcpy(col_value, s.col_value.data(), n * sizeof(double));
  }
  if (col_dual != nullptr && s.col_dual.size() == n) {
    std::memcpy(col_dual, s.col_dual.data(), n * sizeof(double));
  }
  if (row_dual != nullptr && s.row_dual.size() == m) {
    std::memcpy(row_dual, s.row_dual.data(), m * sizeof(double));
  }
  if (message != nullptr && message_capacity > 0) {
    std::snprintf(message, static_cast<std::size_t>(message_capacity), "%s", s.message.c_str());
  }
  return result->status;
}

// The reference's convex-QP engine, convexity gate included (src/qp/qp_condat_vu.cpp:164-362).
// result->primal_residual / dual_residual are not Solution fields and stay -1.
int32_t ref_solve_qp(const orc_qp* qp, const orc_qp_params* params, orc_qp_result* result,
                     double* col_value, double* col_dual, double* row_dual, char* message,
                     int32_t message_capacity) {
  std::memset(result, 0, sizeof(*result));
  result->primal_residual = -1.0;
  result->dual_residual = -1.0;
  const sankhya::Model model = to_qp_model(qp);
  sankhya::Options options;
  options.set_bool("log_to_console", false);
  options.set_double("qp_tolerance", params->tolerance);
  options.set_int("iteration_limit", params->iteration_limit);
  if (params->time_limit < 1e300) options.set_double("time_limit", params->time_limit);
  options.set_int("random_seed", params->random_seed);
  sankhya::Logger logger(nullptr);
  const sankhya::Solution s = sankhya::qp::solve_convex_qp(model, options, logger, nullptr);
  result->status = status_code(s.status);
  result->iterations = s.iterations;
  result->objective = s.objective;
  result->solve_seconds = s.solve_seconds;
  const auto n = static_cast<std::size_t>(qp->lp.cols);
  const auto m = static_cast<std::size_t>(qp->lp.rows);
  if (col_value != nullptr && s.col_value.size() == n) {
    std::memcpy(col_value, s.col_value.data(), n * sizeof(double));
  }
  if (col_dual != nullptr && s.col_dual.size() == n) {
    std::memcpy(col_dual, s.col_dual.data(), n * sizeof(double));
  }
  if (row_dual != nullptr && s.row_dual.size() == m) {
    std::memcpy(row_dual, s.row_dual.data(), m * sizeof(double));
  }
  if (message != nullptr && message_capacity > 0) {
    std::snprintf(message, static_cast<std::size_t>(message_capacity), "%s", s.message.c_str());
  }
  return result->status;
}

// The reference's convexity decision (src/qp/convexity.cpp:177-210): 0 convex, 1 indefinite,
// 2 unverified; `detail` receives its text.
int32_t ref_check_convexity(const orc_qp* qp, char* detail, int32_t detail_capacity) {
  const sankhya::Model model = to_qp_model(qp);
  const sankhya::qp::ConvexityResult r = sankhya::qp::check_convexity(model);
  if (detail != nullptr && detail_capacity > 0) {
    std::snprintf(detail, static_cast<std::size_t>(detail_capacity), "%s", r.detail.c_str());
  }
  switch (r.verdict) {
    case sankhya::qp::Convexity::kConvex: return 0;
    case sankhya::qp::Convexity::kIndefinite: return 1;
    default: return 2;
  }
}

void ref_build_scaling(const orc_lp* lp, const double* min_space_cost, int32_t ruiz_iterations,
                       double* scaled_values, double* row_scale, double* col_scale,
                       double* scaled_cost, double* scaled_col_lower, double* scaled_col_upper,
                       double* scaled_row_lower, double* scaled_row_upper, double* min_abs,
                       double* max_abs) {
  const sankhya::Model model = to_model(lp);
  const std::vector<double> cost(min_space_cost, min_space_cost + lp->cols);
  const sankhya::Scaling s = sankhya::build_scaling(model, cost, ruiz_iterations);
  std::memcpy(scaled_values, s.matrix.values().data(), s.matrix.values().size() * sizeof(double));
  std::memcpy(row_scale, s.row.data(), s.row.size() * sizeof(double));
  std::memcpy(col_scale, s.column.data(), s.column.size() * sizeof(double));
  std::memcpy(scaled_cost, s.cost.data(), s.cost.size() * sizeof(double));
  std::memcpy(scaled_col_lower, s.col_lower.data(), s.col_lower.size() * sizeof(double));
  std::memcpy(scaled_col_upper, s.col_upper.data(), s.col_upper.size() * sizeof(double));
  std::memcpy(scaled_row_lower, s.row_lower.data(), s.row_lower.size() * sizeof(double));
  std::memcpy(scaled_row_upper, s.row_upper.data(), s.row_upper.size() * sizeof(double));
  *min_abs = s.min_abs;
  *max_abs = s.max_abs;
}

double ref_spectral_norm(const orc_lp* lp, int32_t iterations, uint32_t seed) {
  const sankhya::Model model = to_model(lp);
  return sankhya::estimate_spectral_norm(model.matrix, iterations, seed);
}

orc_residuals ref_evaluate(const orc_lp* lp, const double* x, const double* y, double* activity,
                           double* reduced) {
  const sankhya::Model model = to_model(lp);
  sankhya::pdhg::Problem problem;
  problem.model = &model;
  const auto n = static_cast<std::size_t>(lp->cols);
  const auto m = static_cast<std::size_t>(lp->rows);
  problem.cost.resize(n);
  for (std::size_t j = 0; j < n; ++j) problem.cost[j] = lp->sense * lp->col_cost[j];
  problem.cost_norm = sankhya::pdhg::euclidean_norm(problem.cost);
  double bound_square = 0.0;
  for (std::size_t i = 0; i < m; ++i) {
    const double rl = lp->row_lower[i], ru = lp->row_upper[i];
    const double b = sankhya::is_finite_bound(rl) ? rl : (sankhya::is_finite_bound(ru) ? ru : 0.0);
    bound_square += b * b;
  }
  problem.bound_norm = std::sqrt(bound_square);
  std::vector<double> xs(x, x + n), ys(y, y + m), act, red;
  const sankhya::pdhg::Residuals r = sankhya::pdhg::evaluate(problem, xs, ys, act, red);
  if (activity != nullptr) std::memcpy(activity, act.data(), m * sizeof(double));
  if (reduced != nullptr) std::memcpy(reduced, red.data(), n * sizeof(double));
  return to_c(r);
}

// The reference's sparse products on the LP's matrix: y = A x (SparseMatrix::multiply,
// src/la/sparse.cpp:232-242,261-264) and x = A^T y (transpose_multiply, :244-259,266-269).
void ref_multiply(const orc_lp* lp, const double* x, double* y) {
  const sankhya::Model model = to_model(lp);
  model.matrix.multiply(x, y);
}

void ref_transpose_multiply(const orc_lp* lp, const double* y, double* x) {
  const sankhya::Model model = to_model(lp);
  model.matrix.transpose_multiply(y, x);
}

// ---- Models built by the reference's own code ------------------------------------------

struct ref_model {
  sankhya::Model model;
  int64_t optimal_objective = 0;
};

// Reads an MPS or LP file with the reference's reader. Returns NULL (and the reader's message
// in `error`) when the file does not parse or the Model does not validate.
void* ref_model_read(const char* path, char* error, int32_t error_capacity) {
  auto* h = new ref_model;
  const sankhya::io::ReadResult r = sankhya::io::read_model(path, &h->model);
  std::string message = r.ok ? h->model.validate() : r.error;
  if (!r.ok || !message.empty()) {
    if (error != nullptr && error_capacity > 0) {
      std::snprintf(error, static_cast<std::size_t>(error_capacity), "%s", message.c_str());
    }
    delete h;
    return nullptr;
  }
  return h;
}

// The `trial`-th instance (counting from 0) that kkt_lp draws from one mt19937_64 seeded with
// `seed`, with the generator's default configuration except the row and column maxima, as
// the reference's PDHG-against-simplex test draws them (tests/unit/test_pdhg.cpp:181-190).
void* ref_model_kkt_lp(uint64_t seed, int32_t trial, int32_t max_rows, int32_t max_cols) {
  std::mt19937_64 rng(seed);
  sankhya::oracle::GeneratorConfig config;
  config.max_rows = max_rows;
  config.max_cols = max_cols;
  sankhya::oracle::KktInstance instance;
  for (int32_t t = 0; t <= trial; ++t) instance = sankhya::oracle::kkt_lp(rng, config);
  auto* h = new ref_model;
  h->model = sankhya::oracle::to_model(instance.lp);
  h->optimal_objective = instance.optimal_objective;
  return h;
}

void ref_model_shape(const void* handle, int32_t* rows, int32_t* cols, int64_t* nonzeros,
                     double* sense, double* objective_offset, int64_t* optimal_objective) {
  const auto* h = static_cast<const ref_model*>(handle);
  *rows = h->model.num_rows();
  *cols = h->model.num_cols();
  *nonzeros = h->model.matrix.num_nonzeros();
  *sense = h->model.sense == sankhya::ObjSense::kMaximize ? -1.0 : 1.0;
  *objective_offset = h->model.objective_offset;
  *optimal_objective = h->optimal_objective;
}

// Copies the Model into caller arrays sized by ref_model_shape (CSC, ascending rows).
void ref_model_arrays(const void* handle, int32_t* col_starts, int32_t* row_index,
                      double* values, double* col_cost, double* col_lower, double* col_upper,
                      double* row_lower, double* row_upper) {
  const auto* h = static_cast<const ref_model*>(handle);
  const sankhya::Model& m = h->model;
  const auto& starts = m.matrix.column_starts();
  const auto& index = m.matrix.row_indices();
  const auto& vals = m.matrix.values();
  for (std::size_t k = 0; k < starts.size(); ++k) col_starts[k] = static_cast<int32_t>(starts[k]);
  for (std::size_t k = 0; k < index.size(); ++k) row_index[k] = static_cast<int32_t>(index[k]);
  std::memcpy(values, vals.data(), vals.size() * sizeof(double));
  std::memcpy(col_cost, m.col_cost.data(), m.col_cost.size() * sizeof(double));
  std::memcpy(col_lower, m.col_lower.data(), m.col_lower.size() * sizeof(double));
  std::memcpy(col_upper, m.col_upper.data(), m.col_upper.size() * sizeof(double));
  std::memcpy(row_lower, m.row_lower.data(), m.row_lower.size() * sizeof(double));
  std::memcpy(row_upper, m.row_upper.data(), m.row_upper.size() * sizeof(double));
}

// The Hessian of a read Model (its stored lower triangle, CSC): the count of stored entries,
// then the arrays (cols + 1 starts, that many row indices and values).
int64_t ref_model_hessian_nonzeros(const void* handle) {
  return static_cast<const ref_model*>(handle)->model.hessian.num_nonzeros();
}

void ref_model_hessian(const void* handle, int32_t* starts, int32_t* index, double* values) {
  const sankhya::Model& m = static_cast<const ref_model*>(handle)->model;
  const int32_t n = m.num_cols();
  int32_t at = 0;
  for (int32_t j = 0; j < n; ++j) {
    starts[j] = at;
    if (j < m.hessian.num_cols()) {
      const sankhya::ColumnView c = m.hessian.column(j);
      for (sankhya::Index k = 0; k < c.size; ++k) {
        index[at] = static_cast<int32_t>(c.rows[k]);
        values[at] = c.values[k];
        ++at;
      }
    }
  }
  starts[n] = at;
}

void ref_model_free(void* handle) { delete static_cast<ref_model*>(handle); }

}  // extern "C"
