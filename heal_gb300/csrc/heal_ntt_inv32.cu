// heal_ntt_inv32.cu — inverse (Gentleman-Sande) pass kernels for int32_t tensors
// (one translation unit per direction and element type so they compile in
// parallel); see heal_ntt_kernels.cuh.
#include "heal_ntt_launch.cuh"

namespace heal {
int launch_ntt_batch_inv32(const NttBatchArgs &b, int64_t nblocks, int mode, int p, int threads, size_t smem) {
  return launch_batch_direction<int32_t, true>(b, nblocks, mode, p, threads, smem);
}
int launch_ntt_staged_inv32(const NttArgs &a, int mode) { return launch_staged_direction<int32_t, true>(a, mode); }
int launch_ntt_pass_inv32(const NttArgs &a, int64_t nblocks, int mode) {
  return launch_direction_typed<int32_t, true>(a, nblocks, mode);
}
}  // namespace heal
