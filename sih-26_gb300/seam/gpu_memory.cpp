// gpu_memory.cpp -- the drop-in for SANKHYA's src/gpu/gpu_memory.cpp.
//
// The VRAM gate of src/core/solve.cpp:751-773 asks estimate_pdhg_gpu_memory() for the bytes
// the engine will allocate. The reference's estimate counted its own GpuState (9 n-vectors,
// 8 m-vectors, one CSR copy and a cuSPARSE allowance, src/gpu/gpu_memory.cpp:18-46); the GB300
// engine holds CSR and CSC copies of the scaled and unscaled values, its own vector set and
// the mixed method's FP32 copies, so the estimate comes from the engine itself
// (sankhya_gb300_estimate_memory, pure arithmetic, callable without a GPU). The mixed
// method's share is included so the gate never admits a solve that runs out of memory.
// tests/unit/test_gpu_memory.cpp:52-64 pins the old formula and is revised with it.
#include "gpu/gpu_memory.hpp"

#include <algorithm>

#include "sankhya_gb300.h"

namespace sankhya::gpu {

bool is_supported_compute_capability(int major, int minor) noexcept {
  return major * 10 + minor >= kMinComputeArch;
}

std::size_t estimate_pdhg_gpu_memory(Index rows, Index cols, Count nonzeros) {
  return sankhya_gb300_estimate_memory(rows < 0 ? 0 : rows, cols < 0 ? 0 : cols,
                                       nonzeros < 0 ? 0 : nonzeros, SANKHYA_GB300_MIXED);
}

std::size_t vram_reserve(std::size_t total_bytes) {
  // Unchanged policy (src/gpu/gpu_memory.cpp:48-55): the larger of 10% and 256 MiB.
  constexpr std::size_t kMinReserve = 256ULL * 1024 * 1024;
  return std::max(kMinReserve, total_bytes / 10);
}

}  // namespace sankhya::gpu
