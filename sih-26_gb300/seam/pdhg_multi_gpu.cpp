// pdhg_multi_gpu.cpp -- the drop-in for SANKHYA's src/gpu/pdhg_multi_gpu.cu.
//
// The reference splits the rows of one LP over several devices and sums the partial A^T y
// through the host every iteration (src/gpu/pdhg_multi_gpu.cu:596-617). The GB300 engine
// keeps an LP on ONE device -- one GB300 holds a 2e7-nonzero LP dozens of times over -- so
// this entry point solves on the first listed device, exactly as the reference itself does
// when device_ids has one entry (src/gpu/pdhg_multi_gpu.hpp:19-24). Several GPUs are used by
// solving several LPs at once (one engine per device), not by partitioning one.
#include "gpu/pdhg_multi_gpu.hpp"

#include "gpu/pdhg_gpu.hpp"

namespace sankhya::gpu {

Solution solve_pdhg_multi_gpu(const Model& model, const Options& options,
                              const std::vector<int>& device_ids, Logger& logger,
                              SolveControl* control) {
  (void)device_ids;
  return solve_pdhg_gpu(model, options, logger, control);
}

}  // namespace sankhya::gpu
