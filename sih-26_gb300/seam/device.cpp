// device.cpp -- the drop-in for SANKHYA's src/gpu/device.cu (src/gpu/device.hpp:19-29),
// answering the same three probes through the GB300 engine's C ABI.
#include "gpu/device.hpp"

#include "sankhya_gb300.h"

namespace sankhya::gpu {

bool device_available(std::string* description) {
  char buf[256] = {0};
  const int code = sankhya_gb300_device_available(buf, sizeof(buf));
  if (description != nullptr) *description = buf;
  return code == SANKHYA_GB300_OK;
}

bool device_free_memory(std::size_t* free_bytes, std::size_t* total_bytes) {
  return sankhya_gb300_device_free_memory(free_bytes, total_bytes) == SANKHYA_GB300_OK;
}

bool device_compute_capability(int* major, int* minor) {
  int32_t a = 0, b = 0;
  if (sankhya_gb300_device_compute_capability(&a, &b) != SANKHYA_GB300_OK) return false;
  if (major != nullptr) *major = a;
  if (minor != nullptr) *minor = b;
  return true;
}

}  // namespace sankhya::gpu
