// ref_gpu_capi.cpp -- a C entry to the REFERENCE's own CUDA PDHG, for measurement only.
//
// oracle/Makefile (`ref-gpu`) compiles this file with the reference's unmodified
// src/gpu/pdhg_gpu.cu and src/gpu/device.cu (cuSPARSE products and its own elementwise
// kernels) and the PDHG sources libsankhya_ref.so is built from, into
// oracle/_ref/libsankhya_ref_gpu.so. bench.py times it as the existing-GPU bar beside this
// engine. It takes the same arguments as ref_solve_pdhg (ref_capi.cpp) and calls
// sankhya::gpu::solve_pdhg_gpu (src/gpu/pdhg_gpu.hpp:19-20). That function falls back to the
// reference's CPU PDHG when it finds no device or a CUDA call fails (src/gpu/pdhg_gpu.cu:300,
// 757); `algorithm` receives the name the answer carries ("pdhg-cuda" only when the CUDA
// path ran to the end), so the caller can tell.
#include <cstdio>
#include <cstring>
#include <string>

#include "gpu/pdhg_gpu.hpp"
#include "sankhya/logging.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"

#include "../pdhg_oracle.h"

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
  model.matrix.finalize(0.0);
  return model;
}

}  // namespace

extern "C" {

// Returns the reference's SolveStatus as its enum value (include/sankhya/model.hpp:64).
// iterations, objective and solve_seconds come from the Solution; residuals3 receives its
// primal infeasibility, dual infeasibility and relative gap; algorithm (capacity bytes)
// receives Solution::algorithm and message its message.
int32_t ref_gpu_solve_pdhg(const orc_lp* lp, double tolerance, int64_t iteration_limit,
                           double time_limit, int64_t* iterations, double* objective,
                           double* solve_seconds, double* residuals3, char* algorithm,
                           int32_t capacity, char* message, int32_t message_capacity) {
  const sankhya::Model model = to_model(lp);
  sankhya::Options options;
  options.set_bool("log_to_console", false);
  options.set_double("pdhg_tolerance", tolerance);
  options.set_int("iteration_limit", iteration_limit);
  if (time_limit < 1e300) options.set_double("time_limit", time_limit);
  sankhya::Logger logger(nullptr);
  const sankhya::Solution s = sankhya::gpu::solve_pdhg_gpu(model, options, logger, nullptr);
  if (iterations != nullptr) *iterations = s.iterations;
  if (objective != nullptr) *objective = s.objective;
  if (solve_seconds != nullptr) *solve_seconds = s.solve_seconds;
  if (residuals3 != nullptr) {
    residuals3[0] = s.primal_infeasibility;
    residuals3[1] = s.dual_infeasibility;
    residuals3[2] = s.relative_gap;
  }
  if (algorithm != nullptr && capacity > 0) {
    std::snprintf(algorithm, static_cast<std::size_t>(capacity), "%s", s.algorithm.c_str());
  }
  if (message != nullptr && message_capacity > 0) {
    std::snprintf(message, static_cast<std::size_t>(message_capacity), "%s", s.message.c_str());
  }
  return static_cast<int32_t>(s.status);
}

}  // extern "C"
