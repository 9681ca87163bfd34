// lp_gradients.cpp -- gradients of an LP's optimum from SANKHYA's own types (see
// lp_gradients.hpp). Compiles inside SANKHYA's tree beside seam/pdhg_gpu.cpp and links
// against libsankhya_gb300.so.
#include "lp_gradients.hpp"

#include <cstdio>
#include <memory>
#include <mutex>

#include "sankhya_gb300.h"

namespace sankhya::gpu {
namespace {

// The batched engine is created per call (one LP); calls run one after another.
std::mutex use;

struct BatchHandle {
  sankhya_gb300_batch* h = nullptr;
  ~BatchHandle() {
    if (h != nullptr) sankhya_gb300_batch_destroy(h);
  }
};

std::string option_or(const Options& options, const char* name, const char* fallback) {
  return Options::exists(name) ? options.get_string(name) : std::string(fallback);
}

SolveStatus status_of(int code) {
  switch (code) {
    case SANKHYA_GB300_OPTIMAL: return SolveStatus::kOptimal;
    case SANKHYA_GB300_FEASIBLE: return SolveStatus::kFeasible;
    case SANKHYA_GB300_INFEASIBLE: return SolveStatus::kInfeasible;
    case SANKHYA_GB300_ITERATION_LIMIT: return SolveStatus::kIterationLimit;
    default: return SolveStatus::kNumericalError;
  }
}

}  // namespace

std::pair<Solution, LpGradients> solve_pdhg_gpu_with_gradients(const Model& model,
                                                                const Options& options,
                                                                Logger& logger,
                                                                const LossGradient& loss) {
  Solution solution;
  solution.allocate_for(model);
  solution.algorithm = "pdhg-gpu-batch";
  LpGradients g;
  const auto n = static_cast<std::size_t>(model.num_cols());
  const auto m = static_cast<std::size_t>(model.num_rows());
  const auto fail = [&](SolveStatus status, const std::string& message) {
    solution.status = status;
    solution.message = message;
    g.message = message;
    return std::make_pair(solution, g);
  };
  const std::string problem_text = model.validate();
  if (!problem_text.empty()) return fail(SolveStatus::kModelError, problem_text);
  if ((!loss.by_x.empty() && loss.by_x.size() != n) ||
      (!loss.by_y.empty() && loss.by_y.size() != m)) {
    return fail(SolveStatus::kModelError, "the loss gradient's lengths do not match the model");
  }

  std::lock_guard<std::mutex> held(use);
  BatchHandle batch;
  if (sankhya_gb300_batch_create(0, &batch.h) != SANKHYA_GB300_OK) {
    return fail(SolveStatus::kNumericalError,
                std::string("GB300 batched engine unavailable: ") + sankhya_gb300_last_error());
  }
  sankhya_gb300_lp lp{};
  lp.rows = model.num_rows();
  lp.cols = model.num_cols();
  lp.col_starts = model.matrix.column_starts().data();
  lp.row_index = model.matrix.row_indices().data();
  lp.values = model.matrix.values().data();
  lp.col_cost = model.col_cost.data();
  lp.col_lower = model.col_lower.data();
  lp.col_upper = model.col_upper.data();
  lp.row_lower = model.row_lower.data();
  lp.row_upper = model.row_upper.data();
  lp.sense = model.sense_multiplier();
  lp.objective_offset = model.objective_offset;
  sankhya_gb300_params params{};
  params.tolerance = options.get_double("pdhg_tolerance");
  params.iteration_limit = options.get_int("iteration_limit");
  params.time_limit = 1e308;
  params.restart = options.get_bool("pdhg_restart") ? 1 : 0;
  params.stop_at_request = options.get_bool("pdhg_stop_at_request") ? 1 : 0;
  params.random_seed = options.get_int("random_seed");
  params.precision = option_or(options, "pdhg_precision", "fp64") == "mixed"
                         ? SANKHYA_GB300_MIXED
                         : SANKHYA_GB300_FP64;
  params.stop_rule = option_or(options, "pdhg_stop_rule", "standard") == "relative"
                         ? SANKHYA_GB300_STOP_RELATIVE
                         : SANKHYA_GB300_STOP_STANDARD;
  sankhya_gb300_batch_item item{};
  sankhya_gb300_adjoint_info info{};
  double seconds = 0.0;
  int code = sankhya_gb300_batch_load(batch.h, 1, &lp);
  if (code == SANKHYA_GB300_OK) code = sankhya_gb300_batch_solve(batch.h, &params, &item, &seconds);
  const bool solved = code == SANKHYA_GB300_OK && (item.status == SANKHYA_GB300_OPTIMAL ||
                                                   item.status == SANKHYA_GB300_FEASIBLE);
  if (solved) code = sankhya_gb300_batch_polish(batch.h, &item, &info);
  if (code == SANKHYA_GB300_OK) {
    code = sankhya_gb300_batch_solution(batch.h, 0, solution.col_value.data(),
                                        solution.col_dual.data(), solution.row_dual.data());
  }
  if (code != SANKHYA_GB300_OK) {
    return fail(code == SANKHYA_GB300_ERROR_MODEL ? SolveStatus::kModelError
                                                  : SolveStatus::kNumericalError,
                std::string("GB300 batched PDHG: ") + sankhya_gb300_last_error());
  }
  solution.status = status_of(item.status);
  solution.iterations = item.iterations;
  solution.dual_bound = item.dual_bound;
  solution.solve_seconds = seconds;
  solution.recompute_quality(model);
  if (!solved || info.status != 0) {
    char text[160];
    std::snprintf(text, sizeof(text),
                  "%s after %lld iterations; polish status %d: no gradients",
                  to_string(solution.status), static_cast<long long>(item.iterations),
                  static_cast<int>(info.status));
    solution.message = text;
    g.status = solved ? (info.status == 1 ? 1 : 3) : 3;
    g.message = text;
    return {solution, g};
  }
  solution.message = "batched PDHG polished onto its vertex";

  for (auto* v : {&g.cost, &g.col_lower, &g.col_upper}) v->assign(n, 0.0);
  for (auto* v : {&g.row_lower, &g.row_upper}) v->assign(m, 0.0);
  const double* gx = loss.by_x.empty() ? nullptr : loss.by_x.data();
  const double* gy = loss.by_y.empty() ? nullptr : loss.by_y.data();
  double* dc = g.cost.data();
  double* drl = g.row_lower.data();
  double* dru = g.row_upper.data();
  double* dl = g.col_lower.data();
  double* du = g.col_upper.data();
  sankhya_gb300_adjoint_info adj{};
  code = sankhya_gb300_batch_adjoint(batch.h, &gx, &gy, &loss.by_f, &dc, &drl, &dru, &dl, &du,
                                     &adj);
  if (code != SANKHYA_GB300_OK) {
    g.status = 3;
    g.message = std::string("GB300 adjoint: ") + sankhya_gb300_last_error();
    return {solution, g};
  }
  g.status = adj.status;
  char text[160];
  std::snprintf(text, sizeof(text),
                "adjoint status %d, |B| = %d, |R| = %d, conjugate-gradient iterations %d and %d",
                static_cast<int>(adj.status), static_cast<int>(adj.basic_cols),
                static_cast<int>(adj.active_rows), static_cast<int>(adj.iterations[0]),
                static_cast<int>(adj.iterations[1]));
  g.message = text;
  logger.info("GPU gradients: {}", g.message);
  return {solution, g};
}

bool write_gradients(const std::string& path, const Model& model, const LpGradients& g,
                     std::string* error) {
  const auto n = static_cast<std::size_t>(model.num_cols());
  const auto m = static_cast<std::size_t>(model.num_rows());
  if (g.cost.size() != n || g.col_lower.size() != n || g.col_upper.size() != n ||
      g.row_lower.size() != m || g.row_upper.size() != m) {
    if (error != nullptr) *error = "the gradients do not match the model";
    return false;
  }
  std::unique_ptr<std::FILE, int (*)(std::FILE*)> f(std::fopen(path.c_str(), "w"), &std::fclose);
  if (!f) {
    if (error != nullptr) *error = "cannot open " + path;
    return false;
  }
  std::fprintf(f.get(), "# dL/dc dL/d(col_lower) dL/d(col_upper) per column; "
                        "dL/d(row_lower) dL/d(row_upper) per row\n");
  for (std::size_t j = 0; j < n; ++j) {
    const std::string name = j < model.col_names.size() ? model.col_names[j]
                                                        : "c" + std::to_string(j);
    std::fprintf(f.get(), "col %s %.17g %.17g %.17g\n", name.c_str(), g.cost[j], g.col_lower[j],
                 g.col_upper[j]);
  }
  for (std::size_t i = 0; i < m; ++i) {
    const std::string name = i < model.row_names.size() ? model.row_names[i]
                                                        : "r" + std::to_string(i);
    std::fprintf(f.get(), "row %s %.17g %.17g\n", name.c_str(), g.row_lower[i], g.row_upper[i]);
  }
  if (std::ferror(f.get()) != 0) {
    if (error != nullptr) *error = "write error on " + path;
    return false;
  }
  return true;
}

}  // namespace sankhya::gpu
