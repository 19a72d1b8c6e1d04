// heal_ntt_fwd64_gdec.cu — forward pass kernels for int64_t tensors that
// extract g_decomposition digits on load (the first pass of
// heal_g_decomposition_ntt); their own translation unit so that they compile
// in parallel with the plain kernels.  See heal_ntt_kernels.cuh.
#include "heal_ntt_launch.cuh"

namespace heal {
int launch_ntt_pass_fwd64_gdec(const NttArgs &a, int64_t nblocks, int mode) {
  return launch_direction_typed<int64_t, false, true>(a, nblocks, mode);
}
}  // namespace heal
