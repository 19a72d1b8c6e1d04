// heal_ntt_launch.cuh — instantiates and launches the pass kernels of one
// direction (included once by heal_ntt_fwd.cu and once by heal_ntt_inv.cu,
// so the two directions compile in parallel).
#pragma once
#include <algorithm>

#include "heal_ntt_kernels.cuh"
#include "heal_ntt_staged.cuh"

namespace heal {

// ---------------------------------------------------------- staged kernel
// One persistent launch of ntt_staged_kernel over the pass's tiles, at the
// resident CTAs per SM the occupancy calculator gives (rounded to whole
// shares of every limb group).  The tile decomposition is redone for the
// kernel's own tile width C.
template <typename T, int MODE, bool INV, int LOGP, int C, int MINB>
static int launch_staged_typed(const NttArgs &a0) {
  typedef StagedShape<T, MODE, INV, LOGP, C, MINB> S;
  static int per_sm = 0;
  auto kern = ntt_staged_kernel<T, MODE, INV, LOGP, C, MINB>;
  if (!per_sm) {
    HEAL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM_BYTES));
    int nb = 0;
    HEAL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, S::THREADS, S::SMEM_BYTES));
    per_sm = std::max(nb, 1);
  }
  NttArgs a = a0;
  a.C = C;
  a.logC = S::LOGC;
  a.ngroups_t = (a.k + C - 1) / C;
  a.fast_bid = a.ngroups_t < (int64_t)UINT32_MAX && a.l * a.r < (int64_t)UINT32_MAX && a.r < (int64_t)UINT32_MAX;
  if (a.fast_bid) {
    a.fd_groups = fastdiv_make((uint32_t)a.ngroups_t);
    a.fd_nij = fastdiv_make((uint32_t)(a.l * a.r));
    a.fd_r = fastdiv_make((uint32_t)a.r);
  }
  const int64_t nunits = a.nsets * a.l * a.r;  // tiles per limb group
  if (nunits < 1 || nunits * a.ngroups_t > 0x7FFFFFFF)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT: more than 2^31 - 1 tiles in one call");
  // every limb group gets the same number of CTAs (shares), each a contiguous run of its tiles
  const int64_t shares =
      std::max<int64_t>(1, std::min<int64_t>(nunits, (int64_t)per_sm * device_sm_count() / a.ngroups_t));
  const int64_t grid = shares * a.ngroups_t;
  if (grid > 0x7FFFFFFF) return set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT: too many limb groups in one call");
  kern<<<(unsigned)grid, S::THREADS, S::SMEM_BYTES, stream()>>>(a, (uint32_t)nunits);
  return check_launch("ntt_staged_pass");
}

// the staged form (int32 tensors: 256-point passes in the 32-bit modes,
// tiles of 8 limbs, 16 points per thread: 128-thread CTAs, 4 per SM)
template <typename T, bool INV>
static int launch_staged_direction(const NttArgs &a, int mode) {
  if constexpr (sizeof(T) == 4) {
    constexpr int C = 8;
    if (mode == MODE_N32_LAZY) return launch_staged_typed<T, MODE_N32_LAZY, INV, 8, C, 4>(a);
    if (mode == MODE_N32) return launch_staged_typed<T, MODE_N32, INV, 8, C, 4>(a);
  }
  return set_error(HEAL_ERR_RUNTIME, "NTT: no staged kernel for this element type and mode");
}

template <typename Kern>
static int launch_with_smem(Kern kern, const NttArgs &a, int64_t nblocks, int threads, size_t smem, bool &attr_set) {
  if (!attr_set) {
    HEAL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    attr_set = true;
  }
  if (nblocks < 1 || nblocks > 0x7FFFFFFF)  // one CTA per tile along grid x; the tile index is 31-bit
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT: more than 2^31 - 1 tiles in one call");
  kern<<<(unsigned)nblocks, threads, smem, stream()>>>(a);
  return check_launch("ntt_pass");
}

template <typename T, int MODE, bool INV, int LOGP, bool GDEC>
static int launch_reg(const NttArgs &a, int64_t nblocks) {
  static bool attr = false;
  const int threads = ((1 << LOGP) >> lpt_of(MODE, INV)) * a.C;
  const size_t smem = (size_t)(1 << LOGP) * a.C * sizeof(int64_t);
  if constexpr (!INV && !GDEC && mode_wide(MODE) && LOGP == 8)
    return launch_with_smem(ntt_reg_kernel_fwd64_r16<T, MODE, LOGP>, a, nblocks,
                            ((1 << LOGP) >> kFwd64R16Lpt) * a.C, smem, attr);
  if constexpr (!INV && !GDEC && mode_wide(MODE))
    return launch_with_smem(ntt_reg_kernel_fwd64<T, MODE, INV, LOGP, GDEC>, a, nblocks, threads, smem, attr);
  return launch_with_smem(ntt_reg_kernel<T, MODE, INV, LOGP, GDEC>, a, nblocks, threads, smem, attr);
}

template <typename T, bool WIDE, bool INV, bool GDEC>
static int launch_small(const NttArgs &a, int64_t nblocks) {
  static bool attr = false;
  const size_t smem = (size_t)(1 << a.p) * a.C * sizeof(int64_t);
  return launch_with_smem(ntt_small_kernel<T, WIDE, INV, GDEC>, a, nblocks, 256, smem, attr);
}

template <typename T, int MODE, bool INV, bool GDEC>
static int launch_typed(const NttArgs &a, int64_t nblocks) {
  switch (a.p) {
    case 3:
      if constexpr (lpt_of(MODE, INV) <= 3) return launch_reg<T, MODE, INV, 3, GDEC>(a, nblocks);
      return launch_small<T, mode_wide(MODE), INV, GDEC>(a, nblocks);
    case 4: return launch_reg<T, MODE, INV, 4, GDEC>(a, nblocks);
    case 5: return launch_reg<T, MODE, INV, 5, GDEC>(a, nblocks);
    case 6: return launch_reg<T, MODE, INV, 6, GDEC>(a, nblocks);
    case 7: return launch_reg<T, MODE, INV, 7, GDEC>(a, nblocks);
    case 8: return launch_reg<T, MODE, INV, 8, GDEC>(a, nblocks);
    case 9: return launch_reg<T, MODE, INV, 9, GDEC>(a, nblocks);
    case 10: return launch_reg<T, MODE, INV, 10, GDEC>(a, nblocks);
    case 11: return launch_reg<T, MODE, INV, 11, GDEC>(a, nblocks);
    case 12: return launch_reg<T, MODE, INV, 12, GDEC>(a, nblocks);
    default: return launch_small<T, mode_wide(MODE), INV, GDEC>(a, nblocks);
  }
}

// one batched launch of register-kernel passes of one class (pass length p)
template <typename T, int MODE, bool INV>
static int launch_batch_typed(const NttBatchArgs &b, int64_t nblocks, int p, int threads, size_t smem) {
  switch (p) {
#define HEAL_NTT_BATCH_CASE(LP)                                                                          \
  case LP:                                                                                               \
    if constexpr (LP > 3 || lpt_of(MODE, INV) <= 3) {                                                    \
      static bool attr = false;                                                                          \
      if (!attr) {                                                                                       \
        HEAL_TRY_CUDA(cudaFuncSetAttribute(ntt_reg_batch_kernel<T, MODE, INV, LP>,                       \
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));      \
        attr = true;                                                                                     \
      }                                                                                                  \
      ntt_reg_batch_kernel<T, MODE, INV, LP><<<(unsigned)nblocks, threads, smem, stream()>>>(b);         \
      return check_launch("ntt_batch_pass");                                                             \
    }                                                                                                    \
    break;
    HEAL_NTT_BATCH_CASE(3)
    HEAL_NTT_BATCH_CASE(4)
    HEAL_NTT_BATCH_CASE(5)
    HEAL_NTT_BATCH_CASE(6)
    HEAL_NTT_BATCH_CASE(7)
    HEAL_NTT_BATCH_CASE(8)
    HEAL_NTT_BATCH_CASE(9)
    HEAL_NTT_BATCH_CASE(10)
    HEAL_NTT_BATCH_CASE(11)
    HEAL_NTT_BATCH_CASE(12)
#undef HEAL_NTT_BATCH_CASE
  }
  return set_error(HEAL_ERR_RUNTIME, "NTT batch: pass length without a register kernel");
}

template <typename T, bool INV>
static int launch_batch_direction(const NttBatchArgs &b, int64_t nblocks, int mode, int p, int threads, size_t smem) {
  if constexpr (sizeof(T) == 8) {
    if (mode == MODE_W64_GROW) return launch_batch_typed<T, MODE_W64_GROW, INV>(b, nblocks, p, threads, smem);
    if (mode == MODE_W64_LAZY) return launch_batch_typed<T, MODE_W64_LAZY, INV>(b, nblocks, p, threads, smem);
  }
  if (mode == MODE_N32_LAZY) return launch_batch_typed<T, MODE_N32_LAZY, INV>(b, nblocks, p, threads, smem);
  return launch_batch_typed<T, MODE_N32, INV>(b, nblocks, p, threads, smem);
}

// int32 tensors hold q < 2^31, so they only need the 32-bit modes
template <typename T, bool INV, bool GDEC = false>
static int launch_direction_typed(const NttArgs &a, int64_t nblocks, int mode) {
  if constexpr (sizeof(T) == 8) {
    if (mode == MODE_W64_GROW) return launch_typed<T, MODE_W64_GROW, INV, GDEC>(a, nblocks);
    if (mode == MODE_W64_LAZY) return launch_typed<T, MODE_W64_LAZY, INV, GDEC>(a, nblocks);
  }
  if (mode == MODE_N32_LAZY) return launch_typed<T, MODE_N32_LAZY, INV, GDEC>(a, nblocks);
  return launch_typed<T, MODE_N32, INV, GDEC>(a, nblocks);
}

}  // namespace heal
