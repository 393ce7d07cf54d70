// Permanent kernel instantiations for matrix sizes 27..32 (split across
// translation units so the build compiles them in parallel).
#include "permanent_kernel.cuh"

namespace pcvl {
int launch_perm_bin_27_32(int n, const PermBinArgs& a, PermNode* node) {
  return launch_perm_bin_range<27, 32>(n, a, node);
}
}  // namespace pcvl
