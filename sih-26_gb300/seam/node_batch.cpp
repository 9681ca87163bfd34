// node_batch.cpp -- branch-and-bound node relaxations on the GB300 batched engine (see
// node_batch.hpp). Compiles inside SANKHYA's tree beside seam/pdhg_gpu.cpp and links against
// libsankhya_gb300.so.
#include "node_batch.hpp"

#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "sankhya/types.hpp"
#include "sankhya_gb300.h"

namespace sankhya::gpu {
namespace {

SolveStatus node_status(int code) {
  switch (code) {
    case SANKHYA_GB300_OPTIMAL: return SolveStatus::kOptimal;
    case SANKHYA_GB300_FEASIBLE: return SolveStatus::kFeasible;
    case SANKHYA_GB300_INFEASIBLE: return SolveStatus::kInfeasible;
    case SANKHYA_GB300_ITERATION_LIMIT: return SolveStatus::kIterationLimit;
    default: return SolveStatus::kNumericalError;
  }
}

std::string option_or(const Options& options, const char* name, const char* fallback) {
  return Options::exists(name) ? options.get_string(name) : std::string(fallback);
}

// Neumaier's compensated sum: the host check below must not depend on the order the terms
// come in, nor lose the small difference that decides it.
struct Sum {
  double s = 0.0, c = 0.0;
  void add(double v) {
    const double t = s + v;
    c += std::fabs(s) >= std::fabs(v) ? (s - t) + v : (v - t) + s;
    s = t;
  }
  double value() const { return s + c; }
};

// The Farkas value of the dual direction d for the node (the model with bounds lo / up):
//   sum_j min over [lo_j, up_j] of (A'd)_j x_j  -  sum_i max over [rl_i, ru_i] of d_i s_i,
// over the sum of its terms' magnitudes. A positive value proves the node infeasible; a term
// that needs an absent bound gives -1 (no proof).
double farkas_share(const Model& model, const std::vector<double>& lo,
                    const std::vector<double>& up, const std::vector<double>& d) {
  const auto& starts = model.matrix.column_starts();
  const auto& rows = model.matrix.row_indices();
  const auto& values = model.matrix.values();
  Sum value, size;
  for (Index j = 0; j < model.num_cols(); ++j) {
    Sum r;
    for (Index k = starts[j]; k < starts[j + 1]; ++k) r.add(values[k] * d[rows[k]]);
    const double rj = r.value();
    if (rj == 0.0) continue;
    const double bound = rj > 0.0 ? lo[j] : up[j];
    if (!is_finite_bound(bound)) return -1.0;
    value.add(rj * bound);
    size.add(std::fabs(rj * bound));
  }
  for (Index i = 0; i < model.num_rows(); ++i) {
    const double di = d[i];
    if (di == 0.0) continue;
    const double side = di > 0.0 ? model.row_upper[i] : model.row_lower[i];
    if (!is_finite_bound(side)) return -1.0;
    value.add(-di * side);
    size.add(std::fabs(di * side));
  }
  return size.value() > 0.0 ? value.value() / size.value() : -1.0;
}

// One batched engine per process, created on first use; a caller holds `use` from its load
// until it has read every node back.
std::mutex use;

sankhya_gb300_batch* shared_batch(std::string* error) {
  static sankhya_gb300_batch* batch = nullptr;
  if (batch == nullptr && sankhya_gb300_batch_create(0, &batch) != SANKHYA_GB300_OK) {
    *error = sankhya_gb300_last_error();
    batch = nullptr;
  }
  return batch;
}

}  // namespace

std::vector<Solution> solve_node_relaxations_gpu(const Model& model,
                                                 const std::vector<NodeBounds>& nodes,
                                                 const Options& options, Logger& logger) {
  std::vector<Solution> out(nodes.size());
  for (Solution& s : out) {
    s.allocate_for(model);
    s.algorithm = "pdhg-gpu-batch";
  }
  if (nodes.empty()) return out;
  const auto fail_all = [&](SolveStatus status, const std::string& message) {
    for (Solution& s : out) {
      s.status = status;
      s.message = message;
    }
    return out;
  };
  const std::string problem_text = model.validate();
  if (!problem_text.empty()) return fail_all(SolveStatus::kModelError, problem_text);
  const auto n = static_cast<std::size_t>(model.num_cols());
  for (const NodeBounds& node : nodes) {
    if (node.col_lower.size() != n || node.col_upper.size() != n) {
      return fail_all(SolveStatus::kModelError,
                      "a node's column bounds do not match the model's columns");
    }
  }

  std::string error;
  std::unique_lock<std::mutex> held(use);
  sankhya_gb300_batch* batch = shared_batch(&error);
  if (batch == nullptr) {
    return fail_all(SolveStatus::kNumericalError, "GB300 batched engine unavailable: " + error);
  }
  // Every node points at the model's own matrix arrays, so the engine keeps one device copy.
  std::vector<sankhya_gb300_lp> lps(nodes.size());
  for (std::size_t k = 0; k < nodes.size(); ++k) {
    sankhya_gb300_lp& lp = lps[k];
    lp.rows = model.num_rows();
    lp.cols = model.num_cols();
    lp.col_starts = model.matrix.column_starts().data();
    lp.row_index = model.matrix.row_indices().data();
    lp.values = model.matrix.values().data();
    lp.col_cost = model.col_cost.data();
    lp.col_lower = nodes[k].col_lower.data();
    lp.col_upper = nodes[k].col_upper.data();
    lp.row_lower = model.row_lower.data();
    lp.row_upper = model.row_upper.data();
    lp.sense = model.sense_multiplier();
    lp.objective_offset = model.objective_offset;
  }
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
  std::vector<sankhya_gb300_batch_item> items(nodes.size());
  double device_seconds = 0.0;
  int code = sankhya_gb300_batch_load(batch, static_cast<int32_t>(lps.size()), lps.data());
  if (code == SANKHYA_GB300_OK) {
    code = sankhya_gb300_batch_solve(batch, &params, items.data(), &device_seconds);
  }
  std::vector<std::vector<double>> rays(nodes.size());
  for (std::size_t k = 0; k < nodes.size() && code == SANKHYA_GB300_OK; ++k) {
    Solution& s = out[k];
    code = sankhya_gb300_batch_solution(batch, static_cast<int32_t>(k), s.col_value.data(),
                                        s.col_dual.data(), s.row_dual.data());
    if (code == SANKHYA_GB300_OK && items[k].status == SANKHYA_GB300_INFEASIBLE) {
      rays[k].assign(static_cast<std::size_t>(model.num_rows()), 0.0);
      code = sankhya_gb300_batch_ray(batch, static_cast<int32_t>(k), rays[k].data());
    }
  }
  if (code != SANKHYA_GB300_OK) {
    return fail_all(code == SANKHYA_GB300_ERROR_MODEL ? SolveStatus::kModelError
                                                      : SolveStatus::kNumericalError,
                    std::string("GB300 batched PDHG: ") + sankhya_gb300_last_error());
  }
  held.unlock();

  // recompute_quality judges each point against its own node's bounds.
  Model node_model = model;
  for (std::size_t k = 0; k < nodes.size(); ++k) {
    Solution& s = out[k];
    const sankhya_gb300_batch_item& it = items[k];
    s.status = node_status(it.status);
    s.iterations = it.iterations;
    s.dual_bound = it.dual_bound;
    s.solve_seconds = device_seconds;
    char text[192];
    if (s.status == SolveStatus::kInfeasible) {
      const double share =
          farkas_share(model, nodes[k].col_lower, nodes[k].col_upper, rays[k]);
      if (share > 0.0) {
        std::snprintf(text, sizeof(text),
                      "infeasible: Farkas certificate after %lld iterations, value %.3e of its "
                      "terms' magnitude (checked on the host)",
                      static_cast<long long>(it.iterations), share);
      } else {
        s.status = SolveStatus::kNumericalError;
        std::snprintf(text, sizeof(text),
                      "the engine reported infeasible after %lld iterations, but its "
                      "certificate does not check on the host (value %.3e)",
                      static_cast<long long>(it.iterations), share);
      }
    } else {
      std::snprintf(text, sizeof(text),
                    "batched PDHG: %s after %lld iterations, relative primal %.3e, dual %.3e, "
                    "gap %.3e",
                    to_string(s.status), static_cast<long long>(it.iterations),
                    it.final_residuals.primal, it.final_residuals.dual, it.final_residuals.gap);
    }
    s.message = text;
    node_model.col_lower = nodes[k].col_lower;
    node_model.col_upper = nodes[k].col_upper;
    s.recompute_quality(node_model);
  }
  logger.info("Batched PDHG: {} node relaxations in {:.3f}s on the GPU", nodes.size(),
              device_seconds);
  return out;
}

}  // namespace sankhya::gpu
