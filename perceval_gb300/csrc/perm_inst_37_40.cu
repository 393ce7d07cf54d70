// Permanent kernel instantiations for matrix sizes 37..40 (split across
// translation units so the build compiles them in parallel).
#include "permanent_kernel.cuh"

namespace pcvl {
int launch_perm_bin_37_40(int n, const PermBinArgs& a, PermNode* node) {
  return launch_perm_bin_range<37, 40>(n, a, node);
}
}  // namespace pcvl
