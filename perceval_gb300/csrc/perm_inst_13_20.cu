// Permanent kernel instantiations for matrix sizes 13..20 (split across
// translation units so the build compiles them in parallel).
#include "permanent_kernel.cuh"

namespace pcvl {
int launch_perm_bin_13_20(int n, const PermBinArgs& a, PermNode* node) {
  return launch_perm_bin_range<13, 20>(n, a, node);
}
}  // namespace pcvl
