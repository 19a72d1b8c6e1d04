// heal_ntt_kernels.cuh — NTT / INTT pass kernels (included by heal_ntt*.cu).
//
// A pass kernel owns a tile of P = 2^LOGP points x C adjacent limbs of one
// (i, j) slice and runs LOGP stages of HEAL's butterfly network on it (see
// heal_ntt.cu for how the stages split into passes and why the twiddle of
// every butterfly equals the reference's).
//
// Register-blocked form: each thread keeps 8 points (16 in the forward
// mode for q < 2^31) of one column in registers and runs up to 3 (4)
// stages per step on them (a radix-8 / radix-16 group: every twiddle is loaded
// once per group of butterflies that share it); between steps the points are
// exchanged through a shared-memory tile.
// The tile index of point s is XOR-swizzled, s ^ ((s >> 4) & 15), so that
// both the strided (s = r + 16j) and the blocked (s = 16r + j) access
// patterns of a step hit distinct banks.
//
// A tile holding a negative value (or a call with negative twiddles / m_inv)
// takes the exact path instead: the reference's per-step truncated `%` in
// __int128 on the shared tile, one stage per barrier.
#pragma once
#include <cuda_runtime.h>

#include "heal_internal.h"

namespace heal {

enum { KIND_STRIDED = 0, KIND_BLOCK = 1 };


struct NttArgs {
  const void *src;
  int64_t ss[4];
  const void *old;  // INTT: previous result contents for rows no index maps to
  int64_t os[4];
  void *dst;
  int64_t ds[4];
  int64_t l, m, r, k;
  int p, logC, C;
  int kind;
  int64_t nsets;      // sets (strided) or blocks per column
  int64_t ngroups_t;  // ceil(k / C)
  int fast_bid;       // ngroups_t, l * r and r below 2^32: 32-bit block-index split
  FastDiv fd_groups, fd_nij, fd_r;
  const int32_t *load_map;
  const int32_t *store_gather;
  const int32_t *store_scatter;
  const void *tw_pairs;
  const int32_t *tw_rowmap;  // limb -> row of tw_pairs (rows with equal content share one)
  const int *tw_neg;
  const void *tw_raw;
  int64_t tw_s0, tw_s1;
  const int64_t *q;
  const uint64_t *qone;  // floor(2^64 / q) per limb: Shoup companion of 1 (growing-range reduction)
  int lazy_out;          // growing ranges, forward first pass: store unreduced values (below 2^63)
  int unreduced_in;      // the input is such a first pass's output (non-negative, possibly >= q)
  int qone32;            // every modulus is above 2^32, so every qone fits in 32 bits
  int literal;           // reference compatibility: sums and the m^-1 product wrap in the element type
  const void *minv_pairs;
  const int *minv_neg;
  const void *minv_raw;
  int64_t minv_s0;
  int scale;
  int canon_load;
  int force_exact;
  int bitrev;  // log2(m) when the permutation is the index's bit reversal (computed, not loaded), else 0
  // g_decomposition on load (heal_g_decomposition_ntt, the pass that reads
  // the source): digit limb t is digit t % gdec_power of source limb
  // t / gdec_power (source limb stride ss[3]); 0 = off
  int gdec_power, gdec_bits;
  Diag *diag;
};

// row of a permutation table (load_map / store_scatter / store_gather), or
// the bit reversal of v when the call's permutation is bit reversal
__device__ __forceinline__ int64_t perm_row(const NttArgs &g, const int32_t *table, int64_t v) {
  return g.bitrev ? (int64_t)(__brev((uint32_t)v) >> (32 - g.bitrev)) : (int64_t)table[v];
}

template <bool WIDE>
struct Word;
template <>
struct Word<true> {
  typedef uint64_t W;
  typedef ulonglong2 Pair;
};
template <>
struct Word<false> {
  typedef uint32_t W;
  typedef uint2 Pair;
};

// Arithmetic modes of the register kernel:
//   0  32-bit words, values in [0, 2q)    (every q < 2^31)
//   1  32-bit words, Harvey's lazy ranges (every q < 2^30: 4q < 2^32)
//   2  64-bit words, Harvey's lazy ranges (every q < 2^62: 4q < 2^64)
//   3  64-bit words, growing ranges       (q < 2^56 forward, q < 2^(62 - P) inverse)
// Lazy butterflies keep forward values in [0, 4q) and inverse values in
// [0, 2q) with one conditional subtraction per butterfly instead of three;
// every pass still ends on canonical residues.
// Growing ranges drop that subtraction too, using the headroom of 64-bit
// words over the modulus.  Forward (Cooley-Tukey): the Shoup product t takes
// its quotient from a three-multiply high product (mulhi64_3), up to 2 below
// the exact one, so t lies in [0, 4q); with u < Bq, u + t and u - t + 4q both
// lie in [0, (B + 4)q), so a canonical input is below (1 + 4s)q after s
// stages and below 97q < 2^63 after the 24 stages of the longest transform
// (q < 2^56).  A first pass hands its unreduced
// values to the second (`lazy_out`); the last pass reduces once per point
// with a Shoup product by 1 (companion floor(2^64 / q)).  Inverse
// (Gentleman-Sande), with the same product in [0, 4q): values entering stage
// s are below 2^(s+1) q (below q at s = 0), so a - b + 2^(s+1) q is
// non-negative and stage s adds that constant; the sum stays below
// 2^(s+2) q and the product below 4q <= 2^(s+2) q; a pass of P stages ends
// below 2^(P+1) q and reduces once per point (the m^-1 product does it on the
// last pass).
enum { MODE_N32 = 0, MODE_N32_LAZY = 1, MODE_W64_LAZY = 2, MODE_W64_GROW = 3 };
__host__ __device__ constexpr bool mode_wide(int mode) { return mode >= MODE_W64_LAZY; }

// log2 of the points one thread of the register kernel holds (a radix-2^lpt
// step per shared-memory exchange): 16 points for the forward transform in
// mode 0 (32-bit words, q < 2^31), 8 otherwise (measured best for each: the 64-bit
// modes need two registers per point, and the inverse and lazy 32-bit
// kernels ran slower with 16)
#ifndef HEAL_NTT_LPT
#define HEAL_NTT_LPT 3
#endif
#ifndef HEAL_NTT_LPT_N32_FWD
#define HEAL_NTT_LPT_N32_FWD 4
#endif
__host__ __device__ constexpr int lpt_of(int mode, bool inv) {
  return (mode == MODE_N32 && !inv) ? HEAL_NTT_LPT_N32_FWD : HEAL_NTT_LPT;
}

// floor(a * b / 2^64) - e with e in {0, 1, 2}: of the four 32 x 32-bit
// partial products, the low-by-low one is dropped and the two cross products
// contribute only their high words.  The dropped parts sum to below 3 * 2^64,
// hence the error.  Three multiplies instead of four, one of them 64-bit wide.
__device__ __forceinline__ uint64_t mulhi64_3(uint64_t a, uint64_t b) {
  const uint32_t al = (uint32_t)a, ah = (uint32_t)(a >> 32), bl = (uint32_t)b, bh = (uint32_t)(b >> 32);
  return (uint64_t)ah * bh + __umulhi(ah, bl) + __umulhi(al, bh);
}

// The forward growing-range product: y * w mod q up to three extra q,
// [0, 4q) for any y < 2^64 (Shoup with the quotient of mulhi64_3: the exact
// quotient leaves [0, 2q), each missing unit of it one more q)
__device__ __forceinline__ uint64_t mulw_grow(uint64_t y, ulonglong2 pr, uint64_t q) {
  return y * pr.x - mulhi64_3(y, pr.y) * q;
}

// y * w mod q up to one extra q: [0, 2q) for any y (Shoup, no final step)
template <bool WIDE>
__device__ __forceinline__ typename Word<WIDE>::W mulw_lazy(typename Word<WIDE>::W y, typename Word<WIDE>::Pair pr,
                                                             typename Word<WIDE>::W q) {
  if (WIDE) return (typename Word<WIDE>::W)((uint64_t)y * pr.x - mulhi64((uint64_t)y, pr.y) * (uint64_t)q);
  return (typename Word<WIDE>::W)((uint32_t)y * pr.x - mulhi32((uint32_t)y, pr.y) * (uint32_t)q);
}

template <bool WIDE>
__device__ __forceinline__ typename Word<WIDE>::W mulw(typename Word<WIDE>::W y, typename Word<WIDE>::Pair pr,
                                                        typename Word<WIDE>::W q) {
  if (WIDE) return (typename Word<WIDE>::W)shoup64((uint64_t)y, (uint64_t)pr.x, (uint64_t)pr.y, (uint64_t)q);
  return (typename Word<WIDE>::W)shoup32((uint32_t)y, (uint32_t)pr.x, (uint32_t)pr.y, (uint32_t)q);
}

__device__ __forceinline__ int64_t raw_any(const void *base, int64_t off, bool is32) {
  return is32 ? (int64_t)((const int32_t *)base)[off] : ((const int64_t *)base)[off];
}

template <typename Pair>
__device__ __forceinline__ const Pair *tw_row(const NttArgs &g, int64_t t) {
  const int64_t row = g.tw_rowmap ? (int64_t)g.tw_rowmap[t] : t;
  return (const Pair *)g.tw_pairs + row * g.m;
}

// shared-tile word index of point s, column c
__host__ __device__ constexpr int swz_of(int s) { return s ^ ((s >> 4) & 15); }
__device__ __forceinline__ int tidx(int s, int c, int logC) { return (swz_of(s) << logC) + c; }

struct TileCtx {
  int64_t rset, i, j, t0, G;
  int P, C, logC;
  __device__ __forceinline__ int64_t row_of(const NttArgs &g, int s) const {
    return g.kind == KIND_BLOCK ? rset * P + s : rset + (int64_t)s * g.nsets;
  }
};

__device__ __forceinline__ TileCtx tile_ctx(const NttArgs &g, uint32_t block) {
  TileCtx x;
  x.P = 1 << g.p;
  x.C = g.C;
  x.logC = g.logC;
  // Limb groups vary fastest, then (i, j), then the set: neighbouring row
  // segments of one set are read back to back (one DRAM line serves them
  // all), and the CTAs that share twiddle rows (same set and limbs, other
  // i, j) run within a window of ngroups_t * l * r blocks.
  int64_t tg;
  if (g.fast_bid) {  // block < 2^31: divisions by invariant 32-bit divisors
    const uint32_t bid = block;
    const uint32_t rest = fastdiv(bid, g.fd_groups);
    tg = bid - rest * g.fd_groups.d;
    const uint32_t rs = fastdiv(rest, g.fd_nij);
    const uint32_t ij = rest - rs * g.fd_nij.d;
    x.rset = rs;
    const uint32_t ii = fastdiv(ij, g.fd_r);
    x.i = ii;
    x.j = ij - ii * g.fd_r.d;
  } else {
    const int64_t bid = block;
    const int64_t nij = g.l * g.r;
    tg = bid % g.ngroups_t;
    const int64_t rest = bid / g.ngroups_t;
    const int64_t ij = rest % nij;
    x.rset = rest / nij;
    x.j = ij % g.r;
    x.i = ij / g.r;
  }
  x.t0 = tg * g.C;
  x.G = g.kind == KIND_BLOCK ? g.nsets + x.rset : 1;
  return x;
}

// g_decomposition's capacity warning for source element (i, row, j, ts), as
// the separate call records it (first kDiagRecords with coordinates)
static __device__ __noinline__ void gdec_warn(const NttArgs &g, int64_t i, int64_t row, int64_t j, int64_t ts) {
  const unsigned long long slot = atomicAdd(&g.diag->count, 1ull);
  if (slot < (unsigned long long)kDiagRecords) {
    DiagRecord &rec = g.diag->rec[slot];
    rec.coord[0] = i;
    rec.coord[1] = row;
    rec.coord[2] = j;
    rec.coord[3] = ts;
    rec.ndim = 4;
    rec.kind = 1;
    rec.base_bits = (uint64_t)g.gdec_bits;
    rec.power = (uint64_t)g.gdec_power;
  }
}

// digit `d` of a loaded source value; the d == 0 load of each source element
// also makes g_decomposition's residual check
template <typename T>
__device__ __forceinline__ int64_t gdec_load(const NttArgs &g, int64_t value, int d, int64_t i, int64_t row, int64_t j,
                                             int64_t ts) {
  if (d == 0 && gdec_residual<T>(value, (uint64_t)g.gdec_power, (uint64_t)g.gdec_bits) > 0) gdec_warn(g, i, row, j, ts);
  return (int64_t)gdec_digit<T>(value, (uint64_t)d, (uint64_t)g.gdec_bits, (1ull << g.gdec_bits) - 1);
}

// Digits d of a thread's loaded source values, in place, with the per-thread
// shift, mask and residual shift formed once (the closed forms of gdec_digit
// and gdec_residual).  Returns whether a d == 0 load failed the residual
// check; the caller then records each such point (gdec_warn_points).
template <typename T, int kPT>
__device__ __forceinline__ bool gdec_digits(int64_t (&raw)[kPT], uint32_t d, const NttArgs &g) {
  const uint64_t bits = (uint64_t)g.gdec_bits;  // below 64
  const uint64_t mask = (1ull << bits) - 1;
  bool bad = false;
  if constexpr (sizeof(T) == 8) {
    const uint64_t sh = (uint64_t)d * bits, rsh = (uint64_t)g.gdec_power * bits;
    const uint32_t s = sh >= 64 ? 0u : (uint32_t)sh;
    const uint64_t m = sh >= 64 ? 0ull : mask;  // digits past the word are 0
    const bool check = d == 0 && rsh < 64;      // a residual shifted out entirely is 0
    const uint32_t rs = check ? (uint32_t)rsh : 0u;
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      const uint64_t uv = (uint64_t)raw[e];
      bad |= check && (int64_t)(uv >> rs) > 0;
      raw[e] = (int64_t)((uv >> s) & m);
    }
  } else {
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      bad |= d == 0 && gdec_residual<T>(raw[e], (uint64_t)g.gdec_power, bits) > 0;
      raw[e] = (int64_t)gdec_digit<T>(raw[e], (uint64_t)d, bits, mask);
    }
  }
  return bad;
}

template <typename T, bool GDEC = false>
__device__ __forceinline__ int64_t load_point(const NttArgs &g, const TileCtx &x, int s, int64_t t) {
  const int64_t v = x.row_of(g, s);
  if (GDEC) {
    const int64_t ts = t / g.gdec_power;
    const int64_t raw = (int64_t)((const T *)g.src)[x.i * g.ss[0] + v * g.ss[1] + x.j * g.ss[2] + ts * g.ss[3]];
    return gdec_load<T>(g, raw, (int)(t - ts * g.gdec_power), x.i, v, x.j, ts);
  }
  if (g.load_map) {
    const int64_t sr = perm_row(g, g.load_map, v);
    if (sr < 0) return (int64_t)((const T *)g.old)[x.i * g.os[0] + v * g.os[1] + x.j * g.os[2] + t * g.os[3]];
    return (int64_t)((const T *)g.src)[x.i * g.ss[0] + (int64_t)sr * g.ss[1] + x.j * g.ss[2] + t * g.ss[3]];
  }
  return (int64_t)((const T *)g.src)[x.i * g.ss[0] + v * g.ss[1] + x.j * g.ss[2] + t * g.ss[3]];
}

template <typename T>
__device__ __forceinline__ void store_point(const NttArgs &g, const TileCtx &x, int s, int64_t t, int64_t val) {
  const int64_t v = x.row_of(g, s);
  const int64_t dr = g.store_scatter ? perm_row(g, g.store_scatter, v) : v;
  ((T *)g.dst)[x.i * g.ds[0] + dr * g.ds[1] + x.j * g.ds[2] + t * g.ds[3]] = (T)val;
}

// Values that need the reference's own arithmetic: negative ones, and for the
// inverse loaded from user data also values >= q (its first butterfly forms
// u + q - v, negative when v > u + q).  The forward NTT reduces those instead.
template <bool INV>
__device__ __forceinline__ bool needs_exact(const NttArgs &g, int64_t x, int64_t q) {
  return x < 0 || (INV && g.canon_load && x >= q);
}

// ---------------------------------------------------------- exact path
// x in the element type T with two's-complement wraparound (what the sample
// implementation's int32 / int64 expressions compute), widened again
template <typename T>
__device__ __forceinline__ i128 wrap_elem(i128 x) {
  return sizeof(T) == 4 ? (i128)(int32_t)(uint32_t)(uint64_t)x : (i128)(int64_t)(uint64_t)x;
}

// The tile (raw values, tidx layout) through the reference's arithmetic,
// one stage per barrier; then stored (with m_inv scaling / gather).  TT is
// the tile's word: int64, or the element type itself for int32 tensors
// (each stage's results are truncated remainders by q < 2^31 and fit).
// The tile is named by its index, not by its TileCtx: a context passed by
// reference to this out-of-line function would be stored to local memory on
// every tile of the fast path.
template <typename T, bool INV, typename TT = int64_t>
__device__ __noinline__ void exact_tile(const NttArgs &g, uint32_t block, TT *tile) {
  const TileCtx x = tile_ctx(g, block);
  const int P = x.P, C = x.C, logC = x.logC, p = g.p;
  const bool is32 = sizeof(T) == 4;
  const int nbf = (P >> 1) * C;
  for (int st = 0; st < p; ++st) {
    for (int b = threadIdx.x; b < nbf; b += blockDim.x) {
      const int c = b & (C - 1);
      const int64_t t = x.t0 + c;
      if (t >= g.k) continue;
      const int jb = b >> logC;
      int su, sv;
      int64_t twidx;
      if (!INV) {
        const int hl = p - 1 - st;
        const int grp = jb >> hl;
        su = (grp << (hl + 1)) + (jb & ((1 << hl) - 1));
        sv = su + (1 << hl);
        twidx = (x.G << st) + grp;
      } else {
        const int grp = jb >> st;
        su = (grp << (st + 1)) + (jb & ((1 << st) - 1));
        sv = su + (1 << st);
        twidx = x.G * (int64_t)(P >> (st + 1)) + grp;
      }
      const int64_t q = g.q[t];
      const int64_t s = raw_any(g.tw_raw, t * g.tw_s0 + twidx * g.tw_s1, is32);
      const int64_t u = tile[tidx(su, c, logC)];
      const int64_t v = tile[tidx(sv, c, logC)];
      int64_t nu, nv;
      if (g.literal) {  // the sample implementation's sums in the element type (ntt_impl.cpp:106-107,155-157)
        if (!INV) {
          const int64_t vm = crem128((i128)v * s, q);
          nu = crem128(wrap_elem<T>((i128)u + vm), q);
          nv = crem128(wrap_elem<T>((i128)u + q - vm), q);
        } else {
          nu = crem128(wrap_elem<T>((i128)u + v), q);
          nv = crem128(wrap_elem<T>((i128)u + q - v) * s, q);
        }
      } else if (!INV) {
        const int64_t vm = crem128((i128)v * s, q);
        nu = crem128((i128)u + vm, q);
        nv = crem128((i128)u + q - vm, q);
      } else {
        nu = crem128((i128)u + v, q);
        nv = crem128(((i128)u + q - v) * s, q);
      }
      tile[tidx(su, c, logC)] = (TT)nu;
      tile[tidx(sv, c, logC)] = (TT)nv;
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < P * C; e += blockDim.x) {
    const int s = e >> logC, c = e & (C - 1);
    const int64_t t = x.t0 + c;
    if (t >= g.k) continue;
    int64_t val = g.store_gather ? (int64_t)tile[tidx((int)perm_row(g, g.store_gather, s), c, logC)]
                                 : (int64_t)tile[tidx(s, c, logC)];
    if (g.scale) {
      const i128 prod = (i128)val * raw_any(g.minv_raw, t * g.minv_s0, is32);
      // the sample implementation scales in the element type (ntt_impl.cpp:165)
      val = crem128(g.literal ? wrap_elem<T>(prod) : prod, g.q[t]);
    }
    store_point<T>(g, x, s, t, val);
  }
}

// ------------------------------------------------------ generic (P < 16)
template <typename T, bool WIDE, bool INV, bool GDEC = false>
__global__ void __launch_bounds__(256) ntt_small_kernel(const __grid_constant__ NttArgs g) {
  typedef typename Word<WIDE>::W W;
  typedef typename Word<WIDE>::Pair Pair;
  extern __shared__ __align__(16) int64_t tile[];
  const TileCtx x = tile_ctx(g, blockIdx.x);
  const int P = x.P, C = x.C, logC = x.logC;
  int neg = 0;
  for (int e = threadIdx.x; e < P * C; e += blockDim.x) {
    const int s = e >> logC, c = e & (C - 1);
    const int64_t t = x.t0 + c;
    if (t >= g.k) continue;
    const int64_t v = load_point<T, GDEC>(g, x, s, t);
    neg |= needs_exact<INV>(g, v, g.q[t]);
    tile[tidx(s, c, logC)] = v;
  }
  const bool exact = __syncthreads_or(neg) || g.force_exact || (g.tw_neg && *g.tw_neg) ||
                     (g.scale && g.minv_neg && *g.minv_neg);
  if (exact) {
    exact_tile<T, INV>(g, blockIdx.x, tile);
    return;
  }
  const int nbf = (P >> 1) * C;
  if (g.canon_load) {
    for (int e = threadIdx.x; e < P * C; e += blockDim.x) {
      const int s = e >> logC, c = e & (C - 1);
      const int64_t t = x.t0 + c;
      if (t >= g.k) continue;
      const uint64_t q = (uint64_t)g.q[t];
      const uint64_t v = (uint64_t)tile[tidx(s, c, logC)];
      if (v >= q) tile[tidx(s, c, logC)] = (int64_t)(v % q);
    }
    __syncthreads();
  }
  for (int st = 0; st < g.p; ++st) {
    for (int b = threadIdx.x; b < nbf; b += blockDim.x) {
      const int c = b & (C - 1);
      const int64_t t = x.t0 + c;
      if (t >= g.k) continue;
      const int jb = b >> logC;
      int su, sv;
      int64_t twidx;
      if (!INV) {
        const int hl = g.p - 1 - st;
        const int grp = jb >> hl;
        su = (grp << (hl + 1)) + (jb & ((1 << hl) - 1));
        sv = su + (1 << hl);
        twidx = (x.G << st) + grp;
      } else {
        const int grp = jb >> st;
        su = (grp << (st + 1)) + (jb & ((1 << st) - 1));
        sv = su + (1 << st);
        twidx = x.G * (int64_t)(P >> (st + 1)) + grp;
      }
      const W q = (W)g.q[t];
      const Pair pr = __ldg(tw_row<Pair>(g, t) + twidx);
      const W u = (W)tile[tidx(su, c, logC)];
      const W v = (W)tile[tidx(sv, c, logC)];
      W nu, nv;
      if (!INV) {
        const W tv = mulw<WIDE>(v, pr, q);
        nu = u + tv;
        nu = nu >= q ? nu - q : nu;
        nv = u >= tv ? u - tv : u + (q - tv);
      } else {
        nu = u + v;
        nu = nu >= q ? nu - q : nu;
        const W d = u >= v ? u - v : u + (q - v);
        nv = mulw<WIDE>(d, pr, q);
      }
      tile[tidx(su, c, logC)] = (int64_t)nu;
      tile[tidx(sv, c, logC)] = (int64_t)nv;
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < P * C; e += blockDim.x) {
    const int s = e >> logC, c = e & (C - 1);
    const int64_t t = x.t0 + c;
    if (t >= g.k) continue;
    int64_t val = g.store_gather ? tile[tidx((int)perm_row(g, g.store_gather, s), c, logC)] : tile[tidx(s, c, logC)];
    if (g.scale) {
      const Pair pr = __ldg((const Pair *)g.minv_pairs + t);
      val = (int64_t)mulw<WIDE>((W)val, pr, (W)g.q[t]);
    }
    store_point<T>(g, x, s, t, val);
  }
}

// --------------------------------------------------- register-blocked
// Point held in register e (0 .. kPT-1) by thread r during step `step`
// (steps of kLPT stages; the last one may be shorter).
template <bool INV, int LOGP, int kLPT>
__device__ __forceinline__ int point_of(int step, int r, int e) {
  const int st0 = kLPT * step;
  const int q = (LOGP - st0) < kLPT ? (LOGP - st0) : kLPT;
  const int jj = e & ((1 << q) - 1);
  const int id = (r << (kLPT - q)) + (e >> q);  // set index
  if (!INV) {
    const int lD = LOGP - st0 - q;  // log2 of the set spacing D
    const int hi = id >> lD, lo = id & ((1 << lD) - 1);
    return (hi << (lD + q)) + lo + (jj << lD);
  }
  const int hi = id >> st0, lo = id & ((1 << st0) - 1);
  return (hi << (st0 + q)) + lo + (jj << st0);
}

// The rare path of gdec_digits, run after the tile's stores: reloads this
// thread's source values and records every d == 0 load whose residual is
// non-zero, with its coordinates, as the separate g_decomposition call does.
// Out of line, with the tile recomputed from its index, so that the fast path
// keeps no state for it.
template <typename T, bool INV, int LOGP, int kLPT>
__device__ __noinline__ void gdec_warn_points(const NttArgs &g, uint32_t block) {
  const TileCtx x = tile_ctx(g, block);
  const int r = threadIdx.x >> x.logC;
  const int64_t t = x.t0 + (threadIdx.x & (x.C - 1));
  if (t >= g.k) return;
  const int64_t ts = t / g.gdec_power;
  for (int e = 0; e < (1 << kLPT); ++e) {
    const int64_t row = x.row_of(g, point_of<INV, LOGP, kLPT>(0, r, e));
    const int64_t v = (int64_t)((const T *)g.src)[x.i * g.ss[0] + row * g.ss[1] + x.j * g.ss[2] + ts * g.ss[3]];
    if (gdec_residual<T>(v, (uint64_t)g.gdec_power, (uint64_t)g.gdec_bits) > 0) gdec_warn(g, x.i, row, x.j, ts);
  }
}

// One register step: stages [kLPT*STEP, kLPT*STEP + qn) on the kPT >> qn
// sets of 2^qn points this thread holds.  TWS: the twiddle row is in shared
// memory (the staged kernel), else read through the read-only cache.  LPT:
// log2 of the points per thread (the register kernel's lpt_of by default).
template <int MODE, bool INV, int LOGP, int STEP, bool TWS = false, int LPT = lpt_of(MODE, INV)>
__device__ __forceinline__ void reg_step(typename Word<mode_wide(MODE)>::W (&v)[1 << LPT], int r, int64_t G,
                                         const typename Word<mode_wide(MODE)>::Pair *twp,
                                         typename Word<mode_wide(MODE)>::W q) {
  constexpr bool WIDE = mode_wide(MODE);
  constexpr bool GROW = MODE == MODE_W64_GROW;
  constexpr bool LAZY = MODE != MODE_N32;
  constexpr int kLPT = LPT, kPT = 1 << kLPT;
  typedef typename Word<WIDE>::W W;
  typedef typename Word<WIDE>::Pair Pair;
  constexpr int P = 1 << LOGP;
  constexpr int st0 = kLPT * STEP;
  constexpr int qn = (LOGP - st0) < kLPT ? (LOGP - st0) : kLPT;
  const W q2 = q + q, q4 = q2 + q2;
#pragma unroll
  for (int set = 0; set < (kPT >> qn); ++set) {
    const int id = (r << (kLPT - qn)) + set;
    const int base = set << qn;
#pragma unroll
    for (int kk = 0; kk < qn; ++kk) {
      const int st = st0 + kk;
      if (!INV) {
        constexpr int lD = LOGP - st0 - qn;
        const int hi = id >> lD;
        const int dist = 1 << (qn - 1 - kk);
#pragma unroll
        for (int gl = 0; gl < (1 << kk); ++gl) {
          // below 2m <= 2^25 (G < 2m / P, st < LOGP): 32-bit index arithmetic
          const uint32_t ti = ((uint32_t)G << st) + ((uint32_t)hi << kk) + (uint32_t)gl;
          const Pair pr = TWS ? twp[ti] : __ldg(twp + ti);
#pragma unroll
          for (int off = 0; off < dist; ++off) {
            const int a = base + gl * 2 * dist + off, b = a + dist;
            if constexpr (GROW) {
              const W u = v[a];
              const W tv = (W)mulw_grow((uint64_t)v[b], pr, (uint64_t)q);
              v[a] = u + tv;
              v[b] = u - tv + q4;
            } else if (LAZY) {
              W u = v[a];
              u = u >= q2 ? u - q2 : u;
              const W tv = mulw_lazy<WIDE>(v[b], pr, q);
              v[a] = u + tv;
              v[b] = u - tv + q2;
            } else {  // 32-bit words, values in [0, 2q) (q < 2^31: 2q < 2^32)
              const W u = min(v[a], v[a] - q);        // [0, q): u - q wraps above u when u < q
              W tv = mulw_lazy<WIDE>(v[b], pr, q);    // [0, 2q)
              tv = min(tv, tv - q);
              v[a] = u + tv;                          // [0, 2q)
              v[b] = u - tv + q;                      // (0, 2q)
            }
          }
        }
      } else {
        const int hi = id >> st0;
        const int dist = 1 << kk;
        // growing ranges: every value entering stage st >= 1 is below 2^(st+1) q
        const W qs = q << (st + 1);
        // one flat loop over the step's butterflies (group gl, offset off):
        // nested gl / off loops were left partly rolled at 16 points per
        // thread, which put v[] in local memory
        Pair pr;
#pragma unroll
        for (int j = 0; j < (1 << (qn - 1)); ++j) {
          const int gl = j >> kk, off = j & (dist - 1);
          if (off == 0) {
            const int64_t ti = G * (int64_t)(P >> (st + 1)) + ((int64_t)hi << (qn - 1 - kk)) + gl;
            pr = TWS ? twp[ti] : __ldg(twp + ti);
          }
          {
            const int a = base + gl * 2 * dist + off, b = a + dist;
            if constexpr (GROW) {
              const W d = v[a] - v[b] + qs;
              v[a] = v[a] + v[b];
              v[b] = (W)mulw_grow((uint64_t)d, pr, (uint64_t)q);
            } else if (LAZY) {
              W s = v[a] + v[b];
              s = s >= q2 ? s - q2 : s;
              const W d = v[a] - v[b] + q2;
              v[a] = s;
              v[b] = mulw_lazy<WIDE>(d, pr, q);
            } else {  // 32-bit words, values in [0, 2q)
              const W u = min(v[a], v[a] - q), w = min(v[b], v[b] - q);  // [0, q)
              v[a] = u + w;                                               // [0, 2q)
              v[b] = mulw_lazy<WIDE>(u - w + q, pr, q);                   // [0, 2q)
            }
          }
        }
      }
    }
  }
}

// Steps STEP .. NSTEP-1, exchanging through the shared tile between steps.
template <int MODE, bool INV, int LOGP, int STEP, bool TWS = false, int LPT = lpt_of(MODE, INV)>
__device__ __forceinline__ void reg_steps(typename Word<mode_wide(MODE)>::W (&v)[1 << LPT], int r, int c, int logC,
                                          int64_t *tile, int64_t G,
                                          const typename Word<mode_wide(MODE)>::Pair *twp,
                                          typename Word<mode_wide(MODE)>::W q) {
  typedef typename Word<mode_wide(MODE)>::W W;
  constexpr int kLPT = LPT, kPT = 1 << kLPT;
  constexpr int NSTEP = (LOGP + kLPT - 1) / kLPT;
  if constexpr (STEP < NSTEP) {
    if constexpr (STEP > 0) {
      // the fast path exchanges words of its own width (4 bytes in the
      // 32-bit modes); the exact path never shares a CTA with it.
      // Addresses: a thread's points in a step are point_of(step, r, 0) | B(e)
      // with disjoint bits, B linear in the bits of e, and the swizzle is
      // linear over XOR, so tidx(point, c) = tidx(point_of(step, r, 0), c) ^
      // (swz(B(e)) << logC): one per-thread base and a constant per point.
      W *wt = reinterpret_cast<W *>(tile);
      {
        const int ia = tidx(point_of<INV, LOGP, kLPT>(STEP - 1, r, 0), c, logC);
#pragma unroll
        for (int e = 0; e < kPT; ++e) wt[ia ^ (swz_of(point_of<INV, LOGP, kLPT>(STEP - 1, 0, e)) << logC)] = v[e];
      }
      __syncthreads();
      {
        const int ia = tidx(point_of<INV, LOGP, kLPT>(STEP, r, 0), c, logC);
#pragma unroll
        for (int e = 0; e < kPT; ++e) v[e] = wt[ia ^ (swz_of(point_of<INV, LOGP, kLPT>(STEP, 0, e)) << logC)];
      }
      __syncthreads();
    }
    reg_step<MODE, INV, LOGP, STEP, TWS, LPT>(v, r, G, twp, q);
    reg_steps<MODE, INV, LOGP, STEP + 1, TWS, LPT>(v, r, c, logC, tile, G, twp, q);
  }
}

// High 64 bits of a * b for b < 2^32: (a_hi b + floor(a_lo b / 2^32)) / 2^32,
// the sum below 2^64 (the dropped low word of a_lo b cannot carry into it)
__device__ __forceinline__ uint64_t mulhi64_u32(uint64_t a, uint32_t b) {
  return ((uint64_t)(uint32_t)(a >> 32) * b + __umulhi((uint32_t)a, b)) >> 32;
}

// The kPT addresses base + point_of(step, 0, e) * stride: point_of is a sum
// of per-bit weights of e (a thread's points differ in disjoint bits), so
// each address is an earlier one plus one weight * stride (kLPT products in
// all, the rest additions), not a product per point.
template <bool INV, int LOGP, int kLPT, int STEP, typename P>
__device__ __forceinline__ void step_addresses(P *base, int64_t stride, P *(&out)[1 << kLPT]) {
  int64_t w[kLPT];
#pragma unroll
  for (int i = 0; i < kLPT; ++i) w[i] = point_of<INV, LOGP, kLPT>(STEP, 0, 1 << i) * stride;
  out[0] = base;
#pragma unroll
  for (int e = 1; e < (1 << kLPT); ++e) {
    int low = 0;  // the lowest set bit of e (a constant after unrolling)
    while (!((e >> low) & 1)) ++low;
    out[e] = out[e & (e - 1)] + w[low];
  }
}

// minimum resident 512-thread CTAs per SM the register allocation must allow
// (2, at most 64 registers, measured fastest: 1 lets some kernels take more
// registers and fewer warps, 3 caps at 40 registers and spills)
#ifndef HEAL_NTT_MINB
#define HEAL_NTT_MINB 2
#endif
// GDEC: the forward first pass of heal_g_decomposition_ntt (digits extracted
// on load); a separate instantiation so that the plain kernels keep their
// register allocation.
template <typename T, int MODE, bool INV, int LOGP, bool GDEC, int LPT = lpt_of(MODE, INV)>
__device__ __forceinline__ void ntt_reg_tile(const NttArgs &g, uint32_t block, bool &gdec_bad) {
  constexpr bool WIDE = mode_wide(MODE);
  constexpr bool LAZY = MODE != MODE_N32;
  constexpr int kLPT = LPT, kPT = 1 << kLPT;
  typedef typename Word<WIDE>::W W;
  typedef typename Word<WIDE>::Pair Pair;
  constexpr int NSTEP = (LOGP + kLPT - 1) / kLPT;
  extern __shared__ __align__(16) int64_t tile[];
  const TileCtx x = tile_ctx(g, block);
  const int logC = x.logC;
  const int c = threadIdx.x & (x.C - 1);
  const int r = threadIdx.x >> logC;
  const int64_t t = x.t0 + c;
  const bool act = t < g.k;
  const int64_t tq = act ? t : g.k - 1;
  const int64_t q64 = g.q[tq];

  // ---- load (step-0 layout).  In the first and the last step a thread's
  // points sit at offsets point_of(step, 0, e) from its first point, the
  // same for every thread, so one base pointer and one row stride address
  // them all.
  const int64_t rowmul = g.kind == KIND_BLOCK ? 1 : g.nsets;
  int64_t raw[kPT];
  // forward: one unsigned compare per point flags negative values and, with
  // canon_load, values at or above q; inverse: the values that need the
  // exact path
  int big = 0;
  auto flag = [&](int64_t w) {
    if constexpr (INV) return needs_exact<INV>(g, w, q64);
    return g.canon_load ? (uint64_t)w >= (uint64_t)q64 : w < 0;
  };
  if (g.load_map && !g.bitrev) {
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      raw[e] = act ? load_point<T>(g, x, point_of<INV, LOGP, kLPT>(0, r, e), t) : 0;
      big |= flag(raw[e]);
    }
  } else if (g.load_map) {
    // gather through the bit reversal: a thread's rows are row0 | d_e with
    // disjoint bits, and bit reversal maps disjoint bits to disjoint bits, so
    // bitrev(row) = bitrev(row0) | bitrev(d_e): one base and a per-point offset
    const int sh = 32 - g.bitrev;
    const T *p0 = (const T *)g.src + (x.i * g.ss[0] + x.j * g.ss[2] + tq * g.ss[3]);
    const uint32_t rb = __brev((uint32_t)x.row_of(g, point_of<INV, LOGP, kLPT>(0, r, 0))) >> sh;
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      const uint32_t de = (uint32_t)(point_of<INV, LOGP, kLPT>(0, 0, e) * rowmul);
      raw[e] = act ? (int64_t)p0[(int64_t)(rb | (__brev(de) >> sh)) * g.ss[1]] : 0;
      big |= flag(raw[e]);
    }
  } else {
    // source limb (digit limbs below 2^31, checked on the host)
    const int64_t ts = GDEC ? (int64_t)((uint32_t)tq / (uint32_t)g.gdec_power) : tq;
    const T *p0 = (const T *)g.src + (x.i * g.ss[0] + x.j * g.ss[2] + ts * g.ss[3]) +
                  x.row_of(g, point_of<INV, LOGP, kLPT>(0, r, 0)) * g.ss[1];
    const int64_t rs = rowmul * g.ss[1];
    const T *pe[kPT];
    step_addresses<INV, LOGP, kLPT, 0>(p0, rs, pe);
#pragma unroll
    for (int e = 0; e < kPT; ++e) raw[e] = act ? (int64_t)*pe[e] : 0;
    if (GDEC && act) {
      const uint32_t d = (uint32_t)tq - (uint32_t)ts * (uint32_t)g.gdec_power;
      gdec_bad = gdec_digits<T>(raw, d, g);
    }
#pragma unroll
    for (int e = 0; e < kPT; ++e) big |= flag(raw[e]);
  }
  // The exact path takes a negative value, and for the inverse one at or
  // above q as well (its first butterfly forms u + q - v); the forward
  // reduces those on load instead.  The rare flagged threads tell them apart.
  int neg = big;
  if (!INV && g.canon_load && big) {
    neg = 0;
#pragma unroll
    for (int e = 0; e < kPT; ++e) neg |= raw[e] < 0;
  }
  const bool exact = __syncthreads_or(neg) || g.force_exact || (g.tw_neg && *g.tw_neg) ||
                     (g.scale && g.minv_neg && *g.minv_neg);
  if (exact) {
    // a growing-range first pass left its fast tiles' values unreduced; the
    // reference's arithmetic sees canonical residues there
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      int64_t w = raw[e];
      if (g.unreduced_in && w >= q64) w %= q64;
      tile[tidx(point_of<INV, LOGP, kLPT>(0, r, e), c, logC)] = w;
    }
    __syncthreads();
    exact_tile<T, INV>(g, block, tile);
    return;
  }

  const W q = (W)q64;
  const Pair *twp = tw_row<Pair>(g, tq);
  W v[kPT];
  if (INV) {
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      uint64_t u = (uint64_t)raw[e];
      if (g.canon_load && u >= (uint64_t)q64) u %= (uint64_t)q64;
      v[e] = (W)u;
    }
  } else if (big) {  // canonical load with values at or above q (none negative here)
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      uint64_t u = (uint64_t)raw[e];
      if (u >= (uint64_t)q64) u %= (uint64_t)q64;
      v[e] = (W)u;
    }
  } else {
#pragma unroll
    for (int e = 0; e < kPT; ++e) v[e] = (W)(uint64_t)raw[e];
  }
  reg_steps<MODE, INV, LOGP, 0, false, kLPT>(v, r, c, logC, tile, x.G, twp, q);

  // ---- back to canonical residues (forward values < 4q, inverse < 2q,
  // both < 2q in mode 0;
  // growing ranges: a Shoup product by 1, unless the m^-1 product follows or
  // the next pass takes the values as they are)
  if (MODE == MODE_W64_GROW) {
    if (INV ? !g.scale : !g.lazy_out) {
      const W one = (W)g.qone[tq];
      if (g.qone32) {  // floor(2^64 / q) below 2^32: a three-instruction high product
#pragma unroll
        for (int e = 0; e < kPT; ++e) {
          const W u = v[e] - (W)mulhi64_u32((uint64_t)v[e], (uint32_t)one) * q;
          v[e] = u >= q ? u - q : u;
        }
      } else {
#pragma unroll
        for (int e = 0; e < kPT; ++e) {
          const W u = v[e] - (W)mulhi64((uint64_t)v[e], (uint64_t)one) * q;
          v[e] = u >= q ? u - q : u;
        }
      }
    }
  } else {
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      W u = v[e];
      if (LAZY && !INV) u = u >= q + q ? u - (q + q) : u;
      v[e] = u >= q ? u - q : u;
    }
  }

  // ---- store
  if (g.store_gather) {  // single-pass forward: out[u] = res[perm[u]]
    W *wt = reinterpret_cast<W *>(tile);
    if (NSTEP == 1) __syncthreads();  // no exchange ran: the tile may still hold raw loads
#pragma unroll
    for (int e = 0; e < kPT; ++e) wt[tidx(point_of<INV, LOGP, kLPT>(NSTEP - 1, r, e), c, logC)] = v[e];
    __syncthreads();
    if (act) {
#pragma unroll
      for (int e = 0; e < kPT; ++e) {
        const int s = point_of<INV, LOGP, kLPT>(0, r, e);
        store_point<T>(g, x, s, t, (int64_t)wt[tidx((int)perm_row(g, g.store_gather, s), c, logC)]);
      }
    }
    return;
  }
  if (!act) return;
  Pair mp;
  if (g.scale) mp = __ldg((const Pair *)g.minv_pairs + t);
  if (g.store_scatter && g.bitrev) {  // scatter through the bit reversal (see the gather above)
    const int sh = 32 - g.bitrev;
    T *p1 = (T *)g.dst + (x.i * g.ds[0] + x.j * g.ds[2] + t * g.ds[3]);
    const uint32_t rb = __brev((uint32_t)x.row_of(g, point_of<INV, LOGP, kLPT>(NSTEP - 1, r, 0))) >> sh;
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      W val = v[e];
      if (g.scale) val = mulw<WIDE>(val, mp, q);
      const uint32_t de = (uint32_t)(point_of<INV, LOGP, kLPT>(NSTEP - 1, 0, e) * rowmul);
      p1[(int64_t)(rb | (__brev(de) >> sh)) * g.ds[1]] = (T)(int64_t)val;
    }
    return;
  }
  if (g.store_scatter) {
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      W val = v[e];
      if (g.scale) val = mulw<WIDE>(val, mp, q);
      store_point<T>(g, x, point_of<INV, LOGP, kLPT>(NSTEP - 1, r, e), t, (int64_t)val);
    }
    return;
  }
  T *p1 = (T *)g.dst + (x.i * g.ds[0] + x.j * g.ds[2] + t * g.ds[3]) +
          x.row_of(g, point_of<INV, LOGP, kLPT>(NSTEP - 1, r, 0)) * g.ds[1];
  const int64_t rsd = rowmul * g.ds[1];
  if constexpr (!INV && !GDEC) {
    T *pe[kPT];
    step_addresses<INV, LOGP, kLPT, NSTEP - 1>(p1, rsd, pe);
#pragma unroll
    for (int e = 0; e < kPT; ++e) *pe[e] = (T)(int64_t)v[e];  // the forward has no m^-1 product
  } else {
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      W val = v[e];
      if (g.scale) val = mulw<WIDE>(val, mp, q);
      p1[point_of<INV, LOGP, kLPT>(NSTEP - 1, 0, e) * rsd] = (T)(int64_t)val;
    }
  }
}

// One tile of a pass; with GDEC, the capacity warnings of its digit loads
// are recorded once its results are stored.
template <typename T, int MODE, bool INV, int LOGP, bool GDEC, int LPT = lpt_of(MODE, INV)>
__device__ __forceinline__ void ntt_reg_body(const NttArgs &g, uint32_t block) {
  bool gdec_bad = false;
  ntt_reg_tile<T, MODE, INV, LOGP, GDEC, LPT>(g, block, gdec_bad);
  if (GDEC && gdec_bad) gdec_warn_points<T, INV, LOGP, LPT>(g, block);
}

template <typename T, int MODE, bool INV, int LOGP, bool GDEC = false>
__global__ void __launch_bounds__(512, HEAL_NTT_MINB) ntt_reg_kernel(const __grid_constant__ NttArgs g) {
  ntt_reg_body<T, MODE, INV, LOGP, GDEC>(g, blockIdx.x);
}

// The plain forward passes in 64-bit words at up to 72 registers: they do
// not spill there, and at 7 resident CTAs of 128 threads per SM instead of 8
// the digit NTT of the keyswitch measured 1.7-2.5% faster than at 64
// registers.  The inverse passes and the first passes of
// heal_g_decomposition_ntt measured best at 64 (1% slower at 72), and 80 was
// slower for all.
#ifndef HEAL_NTT_FWD64_REGS
#define HEAL_NTT_FWD64_REGS 72
#endif
template <typename T, int MODE, bool INV, int LOGP, bool GDEC = false>
__global__ void __maxnreg__(HEAL_NTT_FWD64_REGS) ntt_reg_kernel_fwd64(const __grid_constant__ NttArgs g) {
  ntt_reg_body<T, MODE, INV, LOGP, GDEC>(g, blockIdx.x);
}

// The plain 64-bit forward passes of 256 points with 16 points per thread
// (two radix-16 register steps and one exchange instead of three radix-8
// steps and two) at up to 128 registers: the digit NTT of the keyswitch
// measured 4.5% faster than 8 points per thread at 72 registers (at 96
// registers, 16 points per thread were no faster).  The tile, its tiling of
// the tensor and the host's tile widths are those of the 8-point kernels;
// only the threads per CTA halve.
#ifndef HEAL_NTT_FWD64_R16_REGS
#define HEAL_NTT_FWD64_R16_REGS 128
#endif
constexpr int kFwd64R16Lpt = 4;
template <typename T, int MODE, int LOGP>
__global__ void __maxnreg__(HEAL_NTT_FWD64_R16_REGS) ntt_reg_kernel_fwd64_r16(const __grid_constant__ NttArgs g) {
  ntt_reg_body<T, MODE, false, LOGP, false, kFwd64R16Lpt>(g, blockIdx.x);
}

// ---------------------------------------------------------- ragged batch
// One launch over the passes of up to kNttBatch transforms of one kernel
// class (element type, arithmetic mode, direction, pass length, tile width):
// CTA b runs tile b - first[j] of pass j, j the last with first[j] <= b.
// The arguments travel in the launch parameters, so the launch is captured
// into a graph like any other.
constexpr int kNttBatch = 64;  // 64 x 400-byte arguments: within the 32 KB of launch parameters
struct NttBatchArgs {
  int n;
  uint32_t first[kNttBatch + 1];
  NttArgs pass[kNttBatch];
};
// a kernel's parameters may take at most 32,764 bytes (CUDA 12.1 and later)
static_assert(sizeof(NttBatchArgs) <= 32764, "heal_ntt_batch arguments exceed the kernel parameter limit");

template <typename T, int MODE, bool INV, int LOGP>
__global__ void __launch_bounds__(512, HEAL_NTT_MINB) ntt_reg_batch_kernel(const __grid_constant__ NttBatchArgs b) {
  int lo = 0, hi = b.n - 1;
  while (lo < hi) {  // largest j with first[j] <= blockIdx.x
    const int mid = (lo + hi + 1) >> 1;
    if (b.first[mid] <= blockIdx.x) lo = mid;
    else hi = mid - 1;
  }
  ntt_reg_body<T, MODE, INV, LOGP, false>(b.pass[lo], blockIdx.x - b.first[lo]);
}

}  // namespace heal
