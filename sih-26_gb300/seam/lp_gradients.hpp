// lp_gradients.hpp -- gradients of an LP's optimum from SANKHYA's own types, on the GB300
// engine.
//
// No counterpart in the reference, which does not differentiate. For a loss
// L(x*, y*, f*) of an LP's optimal point x* (col_value), multipliers y* (row_dual) and value
// f* (objective), this gives dL/dc, dL/d(row_lower), dL/d(row_upper), dL/d(col_lower) and
// dL/d(col_upper) by implicit differentiation at the optimum's active set
// (include/sankhya_gb300.h, sankhya_gb300_batch_adjoint), after solving the LP on the batched
// engine and polishing it onto its vertex (sankhya_gb300_batch_polish). It is the C++ face of
// what sankhya_gb300/autograd.py gives torch.
#pragma once

#include <string>
#include <vector>

#include "sankhya/logging.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"

namespace sankhya::gpu {

// Upstream gradients of L: by x* (num_cols entries, or empty for zero), by y* (num_rows, or
// empty) and by f*.
struct LossGradient {
  std::vector<double> by_x, by_y;
  double by_f = 0.0;
};

struct LpGradients {
  std::vector<double> cost, row_lower, row_upper, col_lower, col_upper;
  // 0: the gradients hold; 1: the optimum is degenerate (the basic columns and active rows
  // differ in number) and the gradients are zero; 2: a square solve did not converge; 3: the
  // LP was not solved to optimality, or its point could not be polished onto a vertex.
  int status = 3;
  std::string message;
};

// Solves `model` (options as solve_pdhg_gpu reads them; pdhg_tolerance is the PDHG stage's,
// the polish then lands on the vertex), and returns the polished Solution and the gradients
// of L at it.
[[nodiscard]] std::pair<Solution, LpGradients> solve_pdhg_gpu_with_gradients(
    const Model& model, const Options& options, Logger& logger, const LossGradient& loss);

// One line per column ("col <name> <dL/dc> <dL/dl> <dL/du>") and per row ("row <name>
// <dL/drl> <dL/dru>"), names as the model holds them (index when it holds none), values in
// %.17g. Returns false with *error set when the file cannot be written.
bool write_gradients(const std::string& path, const Model& model, const LpGradients& g,
                     std::string* error);

}  // namespace sankhya::gpu
