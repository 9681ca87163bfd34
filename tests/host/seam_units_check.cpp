// seam_units_check.cpp -- the reference's unit tests of the pieces the seam replaces, restated
// against the seam, on the CPU.
//
// Linked with seam/gpu_memory.cpp and the engine library itself (libsankhya_gb300.so), whose
// memory estimate is plain arithmetic and runs without a GPU. Built with
// SANKHYA_MIN_COMPUTE_ARCH=103, as a build with the GB300 engine is.
//
// tests/unit/test_gpu_memory.cpp: every assertion holds except SmallModelFormula, which pins
// the reference engine's own buffer list (its GpuState) and changes with the engine:
//   - an empty model still needs the 16 MiB fixed allowance (:20-24), and so do negative
//     sizes, which are clamped (:46-50);
//   - the estimate grows with the nonzeros, the rows and the columns (:26-44);
//   - 100,000 x 200,000 with 1e6 nonzeros needs more than 40 MiB (:66-74);
//   - the reserve is the larger of 256 MiB and a tenth of the device (:77-98).
// tests/unit/test_gpu_device.cpp, with the minimum architecture this engine needs (10.3, the
// GB300): kMinComputeArch is positive (:18-22); 10.3 and above are supported; every earlier
// architecture the reference's tests name is not (B200 10.0, Hopper 9.0, Ada 8.9, Ampere 8.6,
// Turing 7.5, Volta 7.0, Pascal 6.1), nor are 0.0 and negative capabilities (:24-66).
#include <cstdio>
#include <string>

#include "gpu/device.hpp"
#include "gpu/gpu_memory.hpp"

namespace {

int g_failures = 0;

void check(bool ok, const std::string& what) {
  if (!ok) {
    std::printf("FAIL: %s\n", what.c_str());
    ++g_failures;
  }
}

}  // namespace

int main() {
  using sankhya::gpu::estimate_pdhg_gpu_memory;
  using sankhya::gpu::is_supported_compute_capability;
  using sankhya::gpu::kMinComputeArch;
  using sankhya::gpu::vram_reserve;
  constexpr std::size_t kMiB = 1024ULL * 1024;

  check(estimate_pdhg_gpu_memory(0, 0, 0) >= 16 * kMiB, "empty model: fixed allowance");
  check(estimate_pdhg_gpu_memory(-1, -1, -1) >= 16 * kMiB, "negative sizes: clamped");
  check(estimate_pdhg_gpu_memory(100, 200, 0) < estimate_pdhg_gpu_memory(100, 200, 1000) &&
            estimate_pdhg_gpu_memory(100, 200, 1000) < estimate_pdhg_gpu_memory(100, 200, 100000),
        "grows with the nonzeros");
  check(estimate_pdhg_gpu_memory(1000, 500, 5000) < estimate_pdhg_gpu_memory(10000, 500, 5000),
        "grows with the rows");
  check(estimate_pdhg_gpu_memory(500, 1000, 5000) < estimate_pdhg_gpu_memory(500, 5000, 5000),
        "grows with the columns");
  check(estimate_pdhg_gpu_memory(100000, 200000, 1000000) > 40 * kMiB, "large model");

  check(vram_reserve(0) >= 256 * kMiB, "reserve floor");
  check(vram_reserve(10240 * kMiB) == 10240 * kMiB / 10, "reserve: a tenth of 10 GiB");
  check(vram_reserve(1024 * kMiB) == 256 * kMiB, "reserve: the floor under 1 GiB");
  check(vram_reserve(6144 * kMiB) == 6144 * kMiB / 10, "reserve: a tenth of 6 GiB");

  check(kMinComputeArch == 103, "minimum architecture 10.3");
  check(is_supported_compute_capability(10, 3), "GB300 (10.3) supported");
  check(is_supported_compute_capability(12, 0), "a later architecture supported");
  const int older[][2] = {{10, 0}, {9, 0}, {8, 9}, {8, 6}, {7, 5}, {7, 0}, {6, 1}, {0, 0}, {-1, 0}};
  for (const auto& cc : older) {
    check(!is_supported_compute_capability(cc[0], cc[1]),
          "compute " + std::to_string(cc[0]) + "." + std::to_string(cc[1]) + " unsupported");
  }

  if (g_failures == 0) std::printf("OK\n");
  return g_failures == 0 ? 0 : 1;
}
