// checkpoint_stub.cpp -- stands in for the reference's src/mip/checkpoint.cpp in the seam's
// front-end test library. That file needs the full nlohmann::json, which the reference's
// CMake fetches over the network, so it is not compiled here. Branch and bound only calls
// these when a checkpoint path is set; the front-end test solves LPs and never does. Each
// reports failure with a reason instead of pretending to have written or read anything.
#include <string>

#include "mip/checkpoint.hpp"

namespace sankhya::mip {

bool write_checkpoint(const std::string& path, const TreeCheckpoint& checkpoint,
                      std::string* error) {
  (void)checkpoint;
  if (error != nullptr) *error = path + ": checkpoints are not built into this test library";
  return false;
}

bool read_checkpoint(const std::string& path, TreeCheckpoint* checkpoint, std::string* error) {
  (void)checkpoint;
  if (error != nullptr) *error = path + ": checkpoints are not built into this test library";
  return false;
}

}  // namespace sankhya::mip
