// qp_gpu.hpp -- the GB300 face of SANKHYA's convex-QP engine.
//
// Same contract as sankhya::qp::solve_convex_qp (include/sankhya/qp.hpp:20, implemented in
// src/qp/qp_condat_vu.cpp): minimise offset + c'x + 0.5 x'Qx over row_lower <= Ax <= row_upper
// and the column bounds, a Hessian that is not provably convex refused with kModelError before
// any arithmetic, the Solution filled as the CPU engine fills it. The iterations run on the
// GPU (sankhya_gb300_qp_*, include/sankhya_gb300.h). For SANKHYA's solve() to route a QP
// here when its `gpu` option is on, its QP branch (src/core/solve.cpp:975-981) calls
//     options.get_bool("gpu") ? gpu::solve_convex_qp_gpu(target, opts, logger, control)
//                             : qp::solve_convex_qp(target, opts, logger, control)
// with opts = with_the_time_that_is_left(options).
#pragma once

#include "sankhya/logging.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"
#include "sankhya/solve_control.hpp"

namespace sankhya::gpu {

[[nodiscard]] Solution solve_convex_qp_gpu(const Model& model, const Options& options,
                                           Logger& logger, SolveControl* control = nullptr);

}  // namespace sankhya::gpu
