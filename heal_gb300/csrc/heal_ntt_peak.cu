// heal_ntt_peak.cu — the arithmetic ceiling of the NTT's 64-bit butterfly.
//
// heal_ntt_butterfly_peak times the forward growing-range butterfly of the
// register kernel (heal_ntt_kernels.cuh: u + t, u - t + 4q with t the
// growing-range Shoup product) on operands that never leave registers: each thread holds 8
// words and the 7 twiddle pairs of one radix-8 group and runs `groups` groups
// of 12 butterflies, with one load and one store per word.  The measured
// rate is the integer-pipe roofline that an NTT pass, which also moves its
// points through HBM and shared memory and loads its twiddles, is compared
// with.
#include <cuda_runtime.h>

#include "heal_internal.h"
#include "heal_ntt_kernels.cuh"

namespace heal {

__global__ void __launch_bounds__(128) butterfly_peak_kernel(uint64_t *data, const ulonglong2 *tw, uint64_t q,
                                                             int groups, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t v[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) v[e] = data[(size_t)i * 8 + e];
  ulonglong2 t[7];
#pragma unroll
  for (int e = 0; e < 7; ++e) t[e] = tw[(i + e) & 63];
  const uint64_t q4 = 4 * q;
  for (int it = 0; it < groups; ++it) {
#pragma unroll
    for (int kk = 0; kk < 3; ++kk) {
      const int dist = 4 >> kk;
#pragma unroll
      for (int gl = 0; gl < (1 << kk); ++gl) {
        const ulonglong2 pr = t[(1 << kk) - 1 + gl];
#pragma unroll
        for (int off = 0; off < dist; ++off) {
          const int a = gl * 2 * dist + off, b = a + dist;
          const uint64_t u = v[a];
          const uint64_t tv = mulw_grow(v[b], pr, q);
          v[a] = u + tv;
          v[b] = u - tv + q4;
        }
      }
    }
  }
#pragma unroll
  for (int e = 0; e < 8; ++e) data[(size_t)i * 8 + e] = v[e];
}

}  // namespace heal

using namespace heal;

extern "C" int heal_ntt_butterfly_peak(int groups, double *butterflies_per_s) {
  clear_error();
  HEAL_CHECK(ensure_init());
  if (capturing()) return set_error(HEAL_ERR_RUNTIME, "heal_ntt_butterfly_peak: not allowed while a graph is being captured");
  if (groups < 1 || groups > (1 << 16) || !butterflies_per_s)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_ntt_butterfly_peak: groups must be in 1 .. 65536, the output non-null");
  const uint32_t n = (uint32_t)device_sm_count() * 8u * 128u;  // 8 CTAs of 128 threads per SM
  void *data = nullptr, *tw = nullptr;
  HEAL_CHECK(scratch_alloc((size_t)n * 8 * sizeof(uint64_t), &data));
  int rc = scratch_alloc(64 * sizeof(ulonglong2), &tw);
  cudaEvent_t a = nullptr, b = nullptr;
  if (!rc) rc = cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess
                    ? HEAL_OK : set_error(HEAL_ERR_RUNTIME, "heal_ntt_butterfly_peak: cudaEventCreate failed");
  const uint64_t q = 1125899906826241ull;  // a 50-bit NTT prime; the rate does not depend on the values
  if (!rc && cudaMemsetAsync(data, 0x11, (size_t)n * 8 * sizeof(uint64_t), stream()) != cudaSuccess)
    rc = set_error(HEAL_ERR_RUNTIME, "heal_ntt_butterfly_peak: memset failed");
  if (!rc && cudaMemsetAsync(tw, 0x22, 64 * sizeof(ulonglong2), stream()) != cudaSuccess)
    rc = set_error(HEAL_ERR_RUNTIME, "heal_ntt_butterfly_peak: memset failed");
  float ms = 0.f;
  for (int rep = 0; !rc && rep < 2; ++rep) {  // the first launch warms up
    cudaEventRecord(a, stream());
    butterfly_peak_kernel<<<n / 128, 128, 0, stream()>>>((uint64_t *)data, (const ulonglong2 *)tw, q, groups, n);
    rc = check_launch("butterfly_peak");
    cudaEventRecord(b, stream());
    if (!rc && cudaEventSynchronize(b) != cudaSuccess) rc = set_error(HEAL_ERR_RUNTIME, "heal_ntt_butterfly_peak: sync failed");
    if (!rc) cudaEventElapsedTime(&ms, a, b);
  }
  if (!rc) *butterflies_per_s = (double)n * groups * 12 / (ms / 1e3);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  scratch_free(data);
  scratch_free(tw);
  return rc;
}
