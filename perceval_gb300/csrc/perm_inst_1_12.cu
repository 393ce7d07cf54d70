// Permanent kernel instantiations for matrix sizes 1..12 (split across
// translation units so the build compiles them in parallel).
#include "permanent_kernel.cuh"

namespace pcvl {
int launch_perm_bin_1_12(int n, const PermBinArgs& a, PermNode* node) {
  return launch_perm_bin_range<1, 12>(n, a, node);
}
}  // namespace pcvl
