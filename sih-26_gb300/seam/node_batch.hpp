// node_batch.hpp -- branch-and-bound node relaxations on the GB300 batched engine.
//
// No counterpart in the reference, which solves each node relaxation on its own with a
// warm-started dual simplex (src/mip/branch_and_bound_node.cpp: solve_node, and its strong
// branching's probe of both children of every candidate). This is the call a search makes to
// hand a whole set of them to the GPU at once: every node shares the model's matrix, costs
// and rows and differs only in its column bounds, so the matrix goes to the device once and
// every node is solved from scratch by one thread block of one persistent launch
// (include/sankhya_gb300.h, sankhya_gb300_batch_*).
#pragma once

#include <vector>

#include "sankhya/logging.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"

namespace sankhya::gpu {

// The column bounds of one node: the model with col_lower / col_upper replaced.
struct NodeBounds {
  std::vector<double> col_lower, col_upper;
};

// One Solution per node, filled as solve_pdhg_gpu fills one (col_value, col_dual =
// sense * reduced cost, row_dual = sense * (-y), iterations, status, message, dual_bound,
// recompute_quality against the node's own bounds), with algorithm "pdhg-gpu-batch".
// Options: pdhg_tolerance, iteration_limit, pdhg_restart, pdhg_stop_at_request, random_seed,
// and pdhg_precision / pdhg_stop_rule where registered; time_limit is not used by batches.
// A node the engine reports infeasible keeps kInfeasible only if its Farkas certificate
// (sankhya_gb300_batch_ray) also checks on the host, in compensated FP64 sums; otherwise it is
// kNumericalError, saying so. A node whose bounds do not match the model's column count is
// kModelError; no engine, or an engine failure, makes every node kNumericalError with the
// engine's message (there is no CPU fallback).
[[nodiscard]] std::vector<Solution> solve_node_relaxations_gpu(
    const Model& model, const std::vector<NodeBounds>& nodes, const Options& options,
    Logger& logger);

}  // namespace sankhya::gpu
