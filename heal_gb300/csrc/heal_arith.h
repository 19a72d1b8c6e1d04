// heal_arith.h — exact modular arithmetic shared by host and device code.
//
// HEAL computes every modular operation in the double-width type T_DP
// (example_impl/typing.h:4-20: int32 -> int64, int64 -> __int128) followed by
// C's truncating `%`.  For the operands the hot path sees (0 <= x and a
// positive modulus) that is the canonical residue, which these routines
// produce without a hardware divide:
//
//  * Moller & Granlund, "Improved division by invariant integers"
//    (IEEE Trans. Computers 60(2), 2011), Algorithm 4: remainder of a
//    two-word number by a normalised one-word divisor with a precomputed
//    reciprocal v = floor((B^2 - 1) / d) - B.  Used for a * b mod q when both
//    factors vary (modmul).  The 64-bit form reduces any 128-bit product, the
//    32-bit form any 64-bit product.
//  * Shoup's multiplication by a fixed operand: for w < q and
//    w' = floor(w * B / q), y * w - floor(y * w' / B) * q lies in [0, 2q) for
//    every y < B (B = 2^32 or 2^64).  Used for twiddle factors and m^-1.
//
// Everything else (negative operands, a non-positive modulus) goes through
// the compiler's own __int128 / int64 `%`, which has C's truncating
// semantics, so results stay bit-identical to HEAL's sample implementation.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define HEAL_HD __host__ __device__ __forceinline__
#else
#define HEAL_HD inline
#endif

namespace heal {

typedef unsigned __int128 u128;
typedef __int128 i128;

HEAL_HD uint32_t clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__clzll((long long)x);
#else
  return x ? (uint32_t)__builtin_clzll(x) : 64u;
#endif
}
HEAL_HD uint32_t clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__clz((int)x);
#else
  return x ? (uint32_t)__builtin_clz(x) : 32u;
#endif
}

HEAL_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((u128)a * b) >> 64);
#endif
}
HEAL_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// ---------------------------------------------------------------- 64-bit
// Reduction constants of one modulus q (int64 elements).  ok == 0 marks a
// non-positive q, which callers route to the exact `%` path.
struct MG64 {
  uint64_t q, d, v;
  uint32_t s, ok;
};

HEAL_HD MG64 mg64_make(int64_t q) {
  MG64 c;
  c.q = (uint64_t)q;
  c.ok = q > 0;
  c.s = 0;
  c.d = 0;
  c.v = 0;
  if (q > 0) {
    c.s = clz64((uint64_t)q);
    c.d = (uint64_t)q << c.s;
    u128 num = ((u128)(~c.d) << 64) | (u128)0xFFFFFFFFFFFFFFFFull;
    c.v = (uint64_t)(num / c.d);
  }
  return c;
}

// Remainder of (u1 * 2^64 + u0) / d for normalised d and u1 < d (MG Alg. 4).
HEAL_HD uint64_t mg64_rem2(uint64_t u1, uint64_t u0, uint64_t d, uint64_t v) {
  uint64_t plo = v * u1;
  uint64_t phi = mulhi64(v, u1);
  uint64_t q0 = plo + u0;
  uint64_t q1 = phi + u1 + (q0 < plo) + 1;
  uint64_t r = u0 - q1 * d;
  if (r > q0) r += d;
  if (r >= d) r -= d;
  return r;
}

// (x1 * 2^64 + x0) mod q for any 128-bit value.
HEAL_HD uint64_t mg64_mod(uint64_t x1, uint64_t x0, const MG64 &c) {
  if (c.s == 0) {
    uint64_t r1 = x1 >= c.d ? x1 - c.d : x1;
    return mg64_rem2(r1, x0, c.d, c.v);
  }
  const uint32_t s = c.s;
  uint64_t n1 = (x1 << s) | (x0 >> (64 - s));
  uint64_t n0 = x0 << s;
  uint64_t r1;
  if (x1 < c.q) {
    r1 = n1;  // (x1 << s) + (x0 >> (64 - s)) < d whenever x1 < q
  } else {
    uint64_t n2 = x1 >> (64 - s);
    r1 = mg64_rem2(n2, n1, c.d, c.v);
  }
  return mg64_rem2(r1, n0, c.d, c.v) >> s;
}

// a * b mod q for 0 <= a, b < 2^63 (c.ok).
HEAL_HD uint64_t mg64_mulmod(uint64_t a, uint64_t b, const MG64 &c) {
  return mg64_mod(mulhi64(a, b), a * b, c);
}

// ---------------------------------------------------------------- 32-bit
struct MG32 {
  uint32_t q, d, v, s;
  uint32_t ok, pad;
};

HEAL_HD MG32 mg32_make(int64_t q) {
  MG32 c;
  c.q = (uint32_t)q;
  c.ok = q > 0 && q <= 0x7FFFFFFF;
  c.s = 0;
  c.d = 0;
  c.v = 0;
  c.pad = 0;
  if (c.ok) {
    c.s = clz32((uint32_t)q);
    c.d = (uint32_t)q << c.s;
    uint64_t num = ((uint64_t)(~c.d) << 32) | 0xFFFFFFFFull;
    c.v = (uint32_t)(num / c.d);
  }
  return c;
}

HEAL_HD uint32_t mg32_rem2(uint32_t u1, uint32_t u0, uint32_t d, uint32_t v) {
  uint64_t qq = (uint64_t)v * u1 + (((uint64_t)u1 << 32) | u0);
  uint32_t q1 = (uint32_t)(qq >> 32) + 1;
  uint32_t q0 = (uint32_t)qq;
  uint32_t r = u0 - q1 * d;
  if (r > q0) r += d;
  if (r >= d) r -= d;
  return r;
}

// x mod q for any 64-bit x.
HEAL_HD uint32_t mg32_mod(uint64_t x, const MG32 &c) {
  uint32_t x1 = (uint32_t)(x >> 32), x0 = (uint32_t)x;
  if (c.s == 0) {
    uint32_t r1 = x1 >= c.d ? x1 - c.d : x1;
    return mg32_rem2(r1, x0, c.d, c.v);
  }
  const uint32_t s = c.s;
  uint32_t n1 = (x1 << s) | (x0 >> (32 - s));
  uint32_t n0 = x0 << s;
  uint32_t r1;
  if (x1 < c.q) {
    r1 = n1;
  } else {
    uint32_t n2 = x1 >> (32 - s);
    r1 = mg32_rem2(n2, n1, c.d, c.v);
  }
  return mg32_rem2(r1, n0, c.d, c.v) >> s;
}

// ---------------------------------------------------------------- Shoup
// Companion of a fixed factor w < q: floor(w * 2^64 / q) (64-bit words).
HEAL_HD uint64_t shoup64_companion(uint64_t w, uint64_t q) { return (uint64_t)(((u128)w << 64) / q); }
HEAL_HD uint32_t shoup32_companion(uint32_t w, uint32_t q) { return (uint32_t)(((uint64_t)w << 32) / q); }

// y * w mod q in [0, q) for any y < 2^64, q < 2^63.
HEAL_HD uint64_t shoup64(uint64_t y, uint64_t w, uint64_t wp, uint64_t q) {
  uint64_t r = y * w - mulhi64(y, wp) * q;
  return r >= q ? r - q : r;
}
// y * w mod q in [0, q) for any y < 2^32, q < 2^31.
HEAL_HD uint32_t shoup32(uint32_t y, uint32_t w, uint32_t wp, uint32_t q) {
  uint32_t r = y * w - mulhi32(y, wp) * q;
  return r >= q ? r - q : r;
}

// ------------------------------------------------------ invariant divisor
// Granlund & Montgomery, "Division by invariant integers using
// multiplication" (PLDI 1994), Figure 4.1: floor(n / d) for every 32-bit n
// with one high multiply, for a divisor d >= 1 fixed per launch.
struct FastDiv {
  uint32_t d, m, s1, s2;
};
HEAL_HD FastDiv fastdiv_make(uint32_t d) {
  FastDiv f;
  uint32_t l = d > 1 ? 32u - clz32(d - 1) : 0u;
  f.d = d;
  f.m = (uint32_t)(((((uint64_t)1) << 32) * ((((uint64_t)1) << l) - d)) / d) + 1u;
  f.s1 = l < 1 ? l : 1u;
  f.s2 = l > 0 ? l - 1u : 0u;
  return f;
}
HEAL_HD uint32_t fastdiv(uint32_t n, const FastDiv &f) {
  uint32_t t1 = mulhi32(f.m, n);
  return (t1 + ((n - t1) >> f.s1)) >> f.s2;
}

// -------------------------------------------------------- g_decomposition
// Digit d of `value` after d of the reference's steps (remainder and
// quotient of the value by the size_t base, quotient stored back in T;
// example_impl/g_decomposition_impl.cpp:17,52-58), in closed form.  int64: the
// first quotient is already non-negative, so the steps are logical shifts of
// the uint64 image.  int32: storing uv >> bits back into an int32 is an
// arithmetic shift of the int32 value (saturating at 31).
template <typename T>
HEAL_HD uint64_t gdec_digit(int64_t value, uint64_t d, uint64_t bits, uint64_t mask) {
  const uint64_t sh = d * bits;
  if (sizeof(T) == 4) {
    const int32_t v = (int32_t)value >> (sh > 31 ? 31 : sh);
    return (uint64_t)(int64_t)v & mask;
  }
  const uint64_t uv = (uint64_t)value;
  return (sh >= 64 ? 0 : (uv >> sh)) & mask;
}

// The residual after `power` steps as the reference's `value > 0` test sees it.
template <typename T>
HEAL_HD int64_t gdec_residual(int64_t value, uint64_t power, uint64_t bits) {
  const int64_t rest = (int64_t)gdec_digit<T>(value, power, bits, ~0ull);
  return sizeof(T) == 4 ? (int64_t)(int32_t)(uint32_t)rest : rest;
}

// -------------------------------------------------------------- exact C
// C's truncating remainder in the double-width type.
HEAL_HD int64_t crem128(i128 a, int64_t q) { return (int64_t)(a % (i128)q); }

}  // namespace heal
