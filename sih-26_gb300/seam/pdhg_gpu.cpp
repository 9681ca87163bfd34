// pdhg_gpu.cpp -- the drop-in for SANKHYA's src/gpu/pdhg_gpu.cu.
//
// Implements the unchanged seam
//     Solution sankhya::gpu::solve_pdhg_gpu(const Model&, const Options&, Logger&, SolveControl*)
// declared in src/gpu/pdhg_gpu.hpp:19-20 and called from src/core/solve.cpp:802, on top of
// the GB300 engine's C ABI (include/sankhya_gb300.h). It compiles inside SANKHYA's tree in
// place of pdhg_gpu.cu and links against libsankhya_gb300.so.
//
// What it keeps from the reference's contract (src/pdhg/pdhg.cpp:487-567 and the seam's
// header): the Solution is filled exactly as solve_pdhg fills it -- col_value, col_dual =
// sense * reduced cost, row_dual = sense * (-y), iterations, status, message, dual_bound --
// and recompute_quality() runs last; the options are the registry's own rows
// (pdhg_tolerance, iteration_limit, time_limit, pdhg_restart, pdhg_stop_at_request,
// random_seed) plus the engine's pdhg_precision / pdhg_stop_rule rows where registered; the
// iteration table goes through Logger::iteration; SolveControl is polled at every status
// snapshot. What it changes, as the engine's contract requires: there is NO CPU fallback --
// a device failure is kNumericalError with the engine's message, never a silent
// pdhg::solve_pdhg (the reference falls back, src/gpu/pdhg_gpu.cu:300-303,746-758).
#include "gpu/pdhg_gpu.hpp"

#include <cmath>
#include <mutex>
#include <string>

#include "sankhya/solve_control.hpp"
#include "sankhya_gb300.h"
#include "util/profiler.hpp"

namespace sankhya::gpu {
namespace {

SolveStatus to_status(int code) {
  switch (code) {
    case SANKHYA_GB300_OPTIMAL: return SolveStatus::kOptimal;
    case SANKHYA_GB300_FEASIBLE: return SolveStatus::kFeasible;
    case SANKHYA_GB300_INFEASIBLE: return SolveStatus::kInfeasible;
    case SANKHYA_GB300_ITERATION_LIMIT: return SolveStatus::kIterationLimit;
    case SANKHYA_GB300_TIME_LIMIT: return SolveStatus::kTimeLimit;
    case SANKHYA_GB300_INTERRUPTED: return SolveStatus::kInterrupted;
    case SANKHYA_GB300_MODEL_ERROR: return SolveStatus::kModelError;
    default: return SolveStatus::kNumericalError;
  }
}

// An option row the registry may not carry in an older build: the default is used then.
// Options' typed getters abort on a name the registry does not know (they treat it as a bug,
// include/sankhya/options.hpp:82-86), so the row is looked up first.
std::string string_option(const Options& options, const char* name, const char* fallback) {
  return Options::exists(name) ? options.get_string(name) : std::string(fallback);
}

struct Hooks {
  Logger* logger;
  SolveControl* control;
  bool table = false;
};

void log_row(void* user, long long iteration, double objective, double primal, double dual,
             double seconds) {
  auto* h = static_cast<Hooks*>(user);
  if (!h->table) {
    h->logger->begin_iteration_table();
    h->table = true;
  }
  h->logger->iteration(iteration, objective, primal, dual, seconds);
}

int poll(void* user, long long iteration, double objective) {
  auto* h = static_cast<Hooks*>(user);
  if (h->control == nullptr) return 0;
  if (h->control->interruption_requested()) return 1;
  if (h->control->progress_callback && h->control->callback_due()) {
    Progress p;
    p.phase = Progress::Phase::kLp;
    p.iterations = iteration;
    p.objective = objective;
    if (h->control->progress_callback(p) != 0) return 1;
  }
  return 0;
}

// One engine per process, created on first use (device memory is reused across solves).
// SANKHYA's solve() may be called from several threads at once, and an engine holds one LP,
// so a caller keeps `use` locked from its load until it has read its solution back: solves
// from different threads run one after another on the one GPU. The lock is held while the
// engine calls the caller's log and poll hooks, so a progress callback must not itself call
// solve() with the GPU path on.
std::mutex use;

sankhya_gb300_pdhg* shared_engine(std::string* error) {
  static sankhya_gb300_pdhg* engine = nullptr;
  if (engine == nullptr && sankhya_gb300_pdhg_create(0, &engine) != SANKHYA_GB300_OK) {
    *error = sankhya_gb300_last_error();
    engine = nullptr;
  }
  return engine;
}

}  // namespace

Solution solve_pdhg_gpu(const Model& model, const Options& options, Logger& logger,
                        SolveControl* control) {
  Solution solution;
  solution.allocate_for(model);
  solution.algorithm = "pdhg-gpu";
  const std::string problem_text = model.validate();
  if (!problem_text.empty()) {
    solution.status = SolveStatus::kModelError;
    solution.message = problem_text;
    return solution;
  }
  std::string error;
  std::unique_lock<std::mutex> held(use);
  sankhya_gb300_pdhg* engine = shared_engine(&error);
  if (engine == nullptr) {
    solution.status = SolveStatus::kNumericalError;
    solution.message = "GB300 PDHG engine unavailable: " + error;
    return solution;
  }

  const auto& starts = model.matrix.column_starts();
  const auto& rows = model.matrix.row_indices();
  const auto& values = model.matrix.values();
  sankhya_gb300_lp lp{};
  lp.rows = model.num_rows();
  lp.cols = model.num_cols();
  lp.col_starts = starts.data();
  lp.row_index = rows.data();
  lp.values = values.data();
  lp.col_cost = model.col_cost.data();
  lp.col_lower = model.col_lower.data();
  lp.col_upper = model.col_upper.data();
  lp.row_lower = model.row_lower.data();
  lp.row_upper = model.row_upper.data();
  lp.sense = model.sense_multiplier();
  lp.objective_offset = model.objective_offset;

  Hooks hooks{&logger, control};
  sankhya_gb300_params params{};
  params.tolerance = options.get_double("pdhg_tolerance");
  params.iteration_limit = options.get_int("iteration_limit");
  params.time_limit = options.get_double("time_limit");
  params.restart = options.get_bool("pdhg_restart") ? 1 : 0;
  params.stop_at_request = options.get_bool("pdhg_stop_at_request") ? 1 : 0;
  params.random_seed = options.get_int("random_seed");
  params.precision = string_option(options, "pdhg_precision", "fp64") == "mixed"
                         ? SANKHYA_GB300_MIXED
                         : SANKHYA_GB300_FP64;
  params.stop_rule = string_option(options, "pdhg_stop_rule", "standard") == "relative"
                         ? SANKHYA_GB300_STOP_RELATIVE
                         : SANKHYA_GB300_STOP_STANDARD;
  params.log = log_row;
  params.log_user = &hooks;
  params.poll = poll;
  params.poll_user = &hooks;

  sankhya_gb300_result result{};
  int code = sankhya_gb300_pdhg_load(engine, &lp);
  if (code == SANKHYA_GB300_OK) code = sankhya_gb300_pdhg_solve(engine, &params, &result);
  if (code == SANKHYA_GB300_OK) {
    code = sankhya_gb300_pdhg_solution(engine, solution.col_value.data(),
                                       solution.col_dual.data(), solution.row_dual.data());
  }
  if (code != SANKHYA_GB300_OK) {
    solution.status = code == SANKHYA_GB300_ERROR_MODEL ? SolveStatus::kModelError
                                                        : SolveStatus::kNumericalError;
    solution.message = std::string("GB300 PDHG: ") + sankhya_gb300_last_error();
    return solution;
  }
  held.unlock();
  solution.status = to_status(result.status);
  solution.message = result.message;
  solution.iterations = result.iterations;
  solution.dual_bound = result.dual_bound;
  solution.solve_seconds = result.solve_seconds;
  solution.recompute_quality(model);
  // The profile SANKHYA keeps when its `profile` option is on (src/util/profiler.hpp): the
  // restart counter the CPU engine keeps (src/pdhg/pdhg.cpp:479), and the GPU solve's two
  // phases as regions the engine timed itself. The CPU engine's per-step "primal step" and
  // "dual step" scopes have no host-side counterpart: the steps run inside CUDA graphs.
  if (Profiler* profiler = logger.profiler(); profiler != nullptr) {
    if (result.restarts > 0) profiler->count("pdhg restarts", result.restarts);
    profiler->record("pdhg setup (gpu)", result.setup_seconds);
    profiler->record("pdhg iterations (gpu)", result.loop_seconds, result.attempts);
  }
  logger.info("");
  logger.info("Status: {}   objective {:.10e}   iterations {}   restarts {}   time {:.3f}s",
              to_string(solution.status), solution.objective, solution.iterations,
              result.restarts, solution.solve_seconds);
  if (!solution.message.empty()) logger.info("{}", solution.message);
  return solution;
}

}  // namespace sankhya::gpu
