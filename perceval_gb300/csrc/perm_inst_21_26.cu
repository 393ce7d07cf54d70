// Permanent kernel instantiations for matrix sizes 21..26 (split across
// translation units so the build compiles them in parallel).
#include "permanent_kernel.cuh"

namespace pcvl {
int launch_perm_bin_21_26(int n, const PermBinArgs& a, PermNode* node) {
  return launch_perm_bin_range<21, 26>(n, a, node);
}
}  // namespace pcvl
