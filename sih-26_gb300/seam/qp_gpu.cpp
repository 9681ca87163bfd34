// qp_gpu.cpp -- sankhya::gpu::solve_convex_qp_gpu on the GB300 engine's C ABI. Compiles
// inside SANKHYA's tree beside seam/pdhg_gpu.cpp and links against libsankhya_gb300.so.
//
// Kept from the reference's solve_convex_qp (src/qp/qp_condat_vu.cpp:164-362): the convexity
// gate and its messages (the reference's own check_convexity runs first), the option rows
// (qp_tolerance, iteration_limit, time_limit, random_seed, read through ResourceLimits as the
// CPU engine reads them), the stop messages (ResourceLimits::describe, and the engine's own
// ceiling when no iteration limit is set), the iteration table every 5,000 iterations, the
// Solution's fields (col_value = x, col_dual = c + Qx + sense A'y, row_dual = -sense y,
// dual_bound only when optimal) and recompute_quality() last. Changed: the clock, the interrupt
// and the progress callback are tested after every CUDA graph (a multiple of 50 iterations)
// rather than before every iteration; and there is no CPU fallback: a device failure is
// kNumericalError with the engine's message.
#include "qp_gpu.hpp"

#include <cmath>
#include <limits>
#include <mutex>
#include <string>

#include <fmt/format.h>

#include "core/resource_limits.hpp"
#include "qp/convexity.hpp"
#include "sankhya/timer.hpp"
#include "sankhya/tolerances.hpp"
#include "sankhya_gb300.h"

namespace sankhya::gpu {
namespace {

constexpr long long kIterationCeiling = 1000000;  // src/qp/qp_condat_vu.cpp:232

struct QpHooks {
  Logger* logger;
  SolveControl* control;
};

void qp_log(void* user, long long iteration, double objective, double primal, double dual,
            double seconds) {
  static_cast<QpHooks*>(user)->logger->iteration(iteration, objective, primal, dual, seconds);
}

int qp_poll(void* user, long long iteration, double objective) {
  auto* h = static_cast<QpHooks*>(user);
  if (h->control == nullptr) return 0;
  if (h->control->interruption_requested()) return 1;
  if (h->control->progress_callback && h->control->callback_due()) {
    Progress p;
    p.phase = Progress::Phase::kLp;
    p.iterations = iteration;
    p.objective = kInfinity;  // as the CPU engine reports it mid-loop
    p.best_bound = -kInfinity;
    (void)objective;
    if (h->control->progress_callback(p) != 0) {
      h->control->interrupt();
      return 1;
    }
    if (h->control->interruption_requested()) return 1;
  }
  return 0;
}

// One QP engine per process, created on first use; solves from several threads run one after
// another on it (the lock is held from load to the solution read-back).
std::mutex qp_use;

sankhya_gb300_qp* shared_qp_engine(std::string* error) {
  static sankhya_gb300_qp* engine = nullptr;
  if (engine == nullptr && sankhya_gb300_qp_create(0, &engine) != SANKHYA_GB300_OK) {
    *error = sankhya_gb300_last_error();
    engine = nullptr;
  }
  return engine;
}

}  // namespace

Solution solve_convex_qp_gpu(const Model& model, const Options& options, Logger& logger,
                             SolveControl* control) {
  Timer timer;
  Solution solution;
  solution.allocate_for(model);
  solution.algorithm = "qp-condat-vu-gpu";

  // The convexity gate, word for word the CPU engine's (src/qp/qp_condat_vu.cpp:170-186).
  const qp::ConvexityResult convexity = qp::check_convexity(model);
  if (convexity.verdict != qp::Convexity::kConvex) {
    solution.status = SolveStatus::kModelError;
    solution.message =
        convexity.verdict == qp::Convexity::kIndefinite
            ? fmt::format(
                  "the quadratic objective is not convex: {}. A non-convex QP has "
                  "local minima and saddle points, and this engine would return one "
                  "of them labelled optimal, so it is refused instead",
                  convexity.detail)
            : fmt::format("convexity could not be established: {}", convexity.detail);
    logger.warning("{}", solution.message);
    solution.solve_seconds = timer.elapsed_seconds();
    return solution;
  }
  const std::string problem_text = model.validate();
  if (!problem_text.empty()) {
    solution.status = SolveStatus::kModelError;
    solution.message = problem_text;
    solution.solve_seconds = timer.elapsed_seconds();
    return solution;
  }

  const ResourceLimits limits(options, logger);
  const auto n = static_cast<std::size_t>(model.num_cols());
  sankhya_gb300_qp_problem problem{};
  sankhya_gb300_lp& lp = problem.lp;
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
  if (model.hessian.num_nonzeros() > 0 && static_cast<std::size_t>(model.hessian.num_cols()) == n) {
    problem.hessian_starts = model.hessian.column_starts().data();
    problem.hessian_index = model.hessian.row_indices().data();
    problem.hessian_values = model.hessian.values().data();
  }

  QpHooks hooks{&logger, control};
  sankhya_gb300_qp_params params{};
  params.tolerance = options.get_double("qp_tolerance");
  params.iteration_limit = limits.iteration_limit();
  params.time_limit = limits.has_time_limit()
                          ? limits.time_limit() - timer.elapsed_seconds()
                          : std::numeric_limits<double>::max();
  if (limits.has_time_limit() && params.time_limit <= 0.0) params.time_limit = 0.0;
  params.random_seed = options.get_int("random_seed");
  params.log = qp_log;
  params.log_user = &hooks;
  params.poll = qp_poll;
  params.poll_user = &hooks;

  std::string error;
  std::unique_lock<std::mutex> held(qp_use);
  sankhya_gb300_qp* engine = shared_qp_engine(&error);
  if (engine == nullptr) {
    solution.status = SolveStatus::kNumericalError;
    solution.message = "GB300 QP engine unavailable: " + error;
    solution.solve_seconds = timer.elapsed_seconds();
    return solution;
  }
  sankhya_gb300_qp_result result{};
  int code = sankhya_gb300_qp_load(engine, &problem);
  if (code == SANKHYA_GB300_OK) code = sankhya_gb300_qp_solve(engine, &params, &result);
  if (code == SANKHYA_GB300_OK) {
    code = sankhya_gb300_qp_solution(engine, solution.col_value.data(), solution.col_dual.data(),
                                     solution.row_dual.data());
  }
  if (code != SANKHYA_GB300_OK) {
    solution.status = code == SANKHYA_GB300_ERROR_MODEL ? SolveStatus::kModelError
                                                        : SolveStatus::kNumericalError;
    solution.message = std::string("GB300 QP: ") + sankhya_gb300_last_error();
    solution.solve_seconds = timer.elapsed_seconds();
    return solution;
  }
  held.unlock();

  const double elapsed = timer.elapsed_seconds();
  const long long iterations = result.iterations;
  switch (result.status) {
    case SANKHYA_GB300_OPTIMAL: solution.status = SolveStatus::kOptimal; break;
    case SANKHYA_GB300_TIME_LIMIT:
      solution.status = SolveStatus::kTimeLimit;
      solution.message = limits.describe(LimitReason::kTime, elapsed, iterations, 0);
      break;
    case SANKHYA_GB300_INTERRUPTED:
      solution.status = SolveStatus::kInterrupted;
      solution.message = limits.describe(LimitReason::kInterrupt, elapsed, iterations, 0);
      break;
    default:
      solution.status = SolveStatus::kIterationLimit;
      solution.message =
          limits.iteration_limit() >= 0
              ? limits.describe(LimitReason::kIterations, elapsed, iterations, 0)
              : fmt::format(
                    "stopped at this engine's own ceiling of {} iterations, no "
                    "iteration_limit having been set",
                    kIterationCeiling);
      break;
  }
  solution.iterations = iterations;
  solution.solve_seconds = elapsed;
  // An unfinished run has proven nothing about the bound (src/qp/qp_condat_vu.cpp:355-359).
  solution.dual_bound = solution.status == SolveStatus::kOptimal
                            ? model.evaluate_objective(solution.col_value.data())
                            : (model.sense == ObjSense::kMaximize ? kInfinity : -kInfinity);
  solution.recompute_quality(model);
  return solution;
}

}  // namespace sankhya::gpu
