// heal_ntt_inv64.cu — inverse (Gentleman-Sande) pass kernels for int64_t tensors
// (one translation unit per direction and element type so they compile in
// parallel); see heal_ntt_kernels.cuh.
#include "heal_ntt_launch.cuh"

namespace heal {
int launch_ntt_pass_inv64(const NttArgs &a, int64_t nblocks, int mode) {
  return launch_direction_typed<int64_t, true>(a, nblocks, mode);
}
}  // namespace heal
