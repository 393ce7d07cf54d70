// Permanent kernel instantiations for matrix sizes 33..36 (split across
// translation units so the build compiles them in parallel).
#include "permanent_kernel.cuh"

namespace pcvl {
int launch_perm_bin_33_36(int n, const PermBinArgs& a, PermNode* node) {
  return launch_perm_bin_range<33, 36>(n, a, node);
}
}  // namespace pcvl
