// heal_tail.cuh — the keyswitch tail (modmul -> axis_modsum -> permute for a
// short reduced axis) as a device function, shared by heal_fused.cu
// (heal_modmul_axis_sum_permute's lean kernel) and heal_keyswitch.cu (the
// persistent keyswitch batch), and the per-modulus helpers it uses.
#pragma once
#include <cuda_runtime.h>

#include "heal_internal.h"

namespace heal {

template <typename T> struct FusedMG;
template <> struct FusedMG<int32_t> { typedef MG32 type; };
template <> struct FusedMG<int64_t> { typedef MG64 type; };

// one term's element of modmul then one step of axis_modsum's running sum,
// as the separate kernels compute them
template <typename T>
__device__ __forceinline__ int64_t exact_step(int64_t sum, int64_t a, int64_t b, int64_t q,
                                              const typename FusedMG<T>::type &c) {
  int64_t v;
  if (a >= 0 && b >= 0 && q > 0) {
    if (sizeof(T) == 4) v = (int64_t)(T)mg32_mod((uint64_t)a * (uint64_t)b, (const MG32 &)c);
    else v = (int64_t)(T)mg64_mulmod((uint64_t)a, (uint64_t)b, (const MG64 &)c);
  } else {
    v = (int64_t)(T)((i128)a * (i128)b % (i128)q);
  }
  if (sum >= 0 && v >= 0 && q > 0) {
    uint64_t x = (uint64_t)sum + (uint64_t)v;
    return v < q ? (int64_t)(x >= (uint64_t)q ? x - (uint64_t)q : x) : (int64_t)(x % (uint64_t)q);
  }
  return crem128((i128)sum + (i128)v, q);
}

// ------------------------------------------------ lean post-permute form
// The same composition for the common case of a short reduced axis (the
// digits of a keyswitch): every offset fits 31 bits, the result view has at
// most 4 axes after merging, and the reduced axis has D <= 4 terms.  One
// thread per result element; axis roles enter as 0/1 multipliers instead of
// per-axis selects, and all 2D term loads are issued before the products.
struct TailArgs {
  const void *a, *b, *perms, *ptab;
  void *out;
  uint32_t n;                  // result elements
  int nd;                      // result view axes (1..4)
  FastDiv fd[4];               // result view dims
  int32_t as[4], bs[4], rs[4]; // strides in result coordinates (0 for a and b on the gathered axis)
  int32_t ew_m[4], pa_m[4], t_m[4];  // 1 on the elementwise / gathered / last axis
  int32_t a_ax, b_ax, a_pa, b_pa, ps0, ps1;
  Diag *diag;
};

// result element idx (< g.n)
template <typename T, typename PT, int D>
__device__ __forceinline__ void tail_one(const TailArgs &g, uint32_t idx) {
  typedef typename FusedMG<T>::type M;
  uint32_t rem = idx;
  int32_t ao = 0, bo = 0, ro = 0, cr = 0, cp = 0, t = 0;
#pragma unroll
  for (int k = 3; k >= 0; --k) {
    if (k >= g.nd) continue;
    const uint32_t qd = fastdiv(rem, g.fd[k]);
    const int32_t c = (int32_t)(rem - qd * g.fd[k].d);
    rem = qd;
    ao += c * g.as[k];
    bo += c * g.bs[k];
    ro += c * g.rs[k];
    cr += c * g.ew_m[k];
    cp += c * g.pa_m[k];
    t += c * g.t_m[k];
  }
  const int32_t v = (int32_t)((const PT *)g.perms)[cr * g.ps0 + cp * g.ps1];  // validated: 0 <= v < m
  const T *A = (const T *)g.a + (ao + v * g.a_pa);
  const T *B = (const T *)g.b + (bo + v * g.b_pa);
  int64_t av[D], bv[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    av[i] = (int64_t)A[i * g.a_ax];
    bv[i] = (int64_t)B[i * g.b_ax];
  }
  const M mc = ((const M *)g.ptab)[t];
  const int64_t q = sizeof(T) == 4 ? (int64_t)(int32_t)((const MG32 &)mc).q : (int64_t)((const MG64 &)mc).q;
  T *R = (T *)g.out;
  if (q == 0) {
    atomicAdd(&g.diag->zero_mod, 1ull);
    R[ro] = 0;
    return;
  }
  // canonical terms: (sum of products) mod q, accumulated exactly
  bool canon = q > 0;
#pragma unroll
  for (int i = 0; i < D; ++i) canon = canon && av[i] >= 0 && av[i] < q && bv[i] >= 0 && bv[i] < q;
  int64_t res;
  if (canon) {
    if (sizeof(T) == 4) {
      uint64_t lo = 0;  // D < 4 products below q^2 < 2^62: no overflow
#pragma unroll
      for (int i = 0; i < D; ++i) lo += (uint64_t)av[i] * (uint64_t)bv[i];
      res = (int64_t)mg32_mod(lo, (const MG32 &)mc);
    } else {
      const uint64_t uq = (uint64_t)q;
      uint64_t hi = 0, lo = 0;  // hi * 2^64 + lo, hi < q
#pragma unroll
      for (int i = 0; i < D; ++i) {
        const uint64_t x = (uint64_t)av[i], y = (uint64_t)bv[i];
        const uint64_t plo = x * y, phi = mulhi64(x, y);
        const uint64_t s = lo + plo;
        hi += phi + (s < lo ? 1 : 0);
        lo = s;
        hi = hi >= uq ? hi - uq : hi;
      }
      res = (int64_t)mg64_mod(hi, lo, (const MG64 &)mc);
    }
  } else {
    res = 0;
#pragma unroll
    for (int i = 0; i < D; ++i) res = exact_step<T>(res, av[i], bv[i], q, mc);
  }
  R[ro] = (T)res;
}

template <typename T, typename PT, int D>
__global__ void __launch_bounds__(256) tail_kernel(const __grid_constant__ TailArgs g) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < g.n) tail_one<T, PT, D>(g, idx);
}

// heal_modmul_axis_sum_permute's lean launch, recorded instead of launched
// (heal_keyswitch_batch runs it inside its persistent kernel): the
// arguments, the element and permutation types and the reduced length
struct TailRecorded {
  TailArgs args;
  int is32, perms32, len;
};
// Validates and prepares the call as heal_modmul_axis_sum_permute does and
// records its lean launch into *out; HEAL_ERR_INVALID_ARGUMENT when the call
// would not take the lean kernel or would need a temporary copy.
int tail_record(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, int64_t axis,
                const heal_tensor *perms, int64_t elementwise_axis, int64_t perm_axis, const heal_tensor *result,
                TailRecorded *out);

}  // namespace heal
