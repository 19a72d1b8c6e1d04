// heal_ntt_staged.cuh — the staged NTT pass kernel (included by heal_ntt_*.cu).
//
// The same pass as ntt_reg_kernel (heal_ntt_kernels.cuh: a P-point piece of
// HEAL's butterfly network on C adjacent limbs, register radix-8 / radix-16
// steps exchanging through a swizzled shared tile, the same arithmetic
// modes), organised so that no global load sits on the compute path:
//
//  * Persistent CTAs, each walking tiles b, b + grid, b + 2 grid, ...
//  * Two shared-memory stages.  While tile i computes in one, the other
//    fills with tile i+1 through cp.async (16-byte LDGSTS, no register
//    round trip): the tile's row segments (C limbs of each of its P rows,
//    laid out in the exchange layout tidx(s, c) so the first step reads them
//    conflict-free), its limbs' constants (q, floor(2^64 / q), m^-1) and its
//    P - 1 twiddle pairs per limb, stored by heap slot h = 2^lv + g (stage lv
//    of the forward network, stage LOGP - 1 - lv of the inverse): the pass's
//    twiddle of slot h is tw[(G - 1) 2^lv + h], one contiguous run of 2^lv
//    pairs per stage.
//  * The results go back through the same stage in the exchange layout and
//    leave as 16-byte row-segment stores (bit-reversal scatter included).
//
// Measured against the register kernel on GB300: 12% faster for the 32-bit
// word modes ([64, 65536, 1, 32] int32, 31-bit primes: 1.13 against 1.28 ms
// per call), 16% slower for the 64-bit growing-range mode (the digit NTT of
// the keyswitch chain), which therefore stays on the register kernel.
// Ablations (copies with parts removed, never committed) showed the 64-bit
// passes bound by neither their butterfly arithmetic (removing it saved 15%)
// nor the exchanges (0%): their per-tile structure is the cost.
//
// Eligible passes (the host checks): register-kernel modes, limbs contiguous
// (stride 1) in source and destination, every row segment 16-byte aligned,
// k a multiple of 16 / sizeof(T), no permutation or the bit reversal on
// load and store, no gather after the pass, no g_decomposition on load.
// A tile with a value the fast arithmetic cannot take runs exact_tile as the
// register kernel does.
#pragma once
#include "heal_ntt_kernels.cuh"

namespace heal {

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// every group of this thread's copies has landed
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

constexpr int ilog2c(int x) { return x <= 1 ? 0 : 1 + ilog2c(x >> 1); }

template <typename T, int MODE, bool INV, int LOGP, int C, int MINB_>
struct StagedShape {
  static constexpr bool WIDE = mode_wide(MODE);
  typedef typename Word<WIDE>::W W;
  typedef typename Word<WIDE>::Pair Pair;
  static constexpr int P = 1 << LOGP;
  static constexpr int kLPT = lpt_of(MODE, INV), kPT = 1 << kLPT;
  static constexpr int NSTEP = (LOGP + kLPT - 1) / kLPT;
  static constexpr int LOGC = ilog2c(C);
  static constexpr int THREADS = P * C / kPT;
  static constexpr int EPC = 16 / (int)sizeof(T);      // elements per 16-byte chunk
  static constexpr int CPR = C / EPC;                  // chunks per row segment
  static constexpr int NCHUNK = P * CPR;
  static constexpr int RSTEP = THREADS / CPR;          // rows between a thread's chunks
  static constexpr int DATA_ITERS = NCHUNK / THREADS;
  static constexpr int PPC = 16 / (int)sizeof(Pair);   // twiddle pairs per 16-byte chunk
  static constexpr int TWROW = P + PPC;                // padded: the limbs' rows start in different banks
  static constexpr int TPL = THREADS / C;              // threads filling one limb's twiddles
  static constexpr int TW_ITERS = P / PPC / TPL;
  static constexpr int DATA_BYTES = P * C * (int)sizeof(T);
  static constexpr int TW_BYTES = C * TWROW * (int)sizeof(Pair);
  static constexpr int LIMB_BYTES = C * 32;            // per limb: q, floor(2^64 / q), the m^-1 pair
  static constexpr int STAGE_BYTES = DATA_BYTES + TW_BYTES + LIMB_BYTES;
  static constexpr int SMEM_BYTES = 2 * STAGE_BYTES;
  static constexpr int MINB = MINB_;                   // resident CTAs per SM the register budget allows
  // the exact path of a 32-bit tile runs on the twiddle region as int64
  static_assert(sizeof(T) == 8 || TW_BYTES >= P * C * 8, "exact tile does not fit the twiddle region");
  static_assert((P / PPC) % TPL == 0, "twiddle chunks split evenly");
  static_assert(C % EPC == 0 && THREADS % CPR == 0 && NCHUNK % THREADS == 0, "row chunks split evenly");
  static_assert((RSTEP & (RSTEP - 1)) == 0, "a thread's rows differ in disjoint bits");
  static_assert(THREADS % C == 0, "whole threads per limb");
};

// per-limb constants of a tile, staged with it
struct StagedLimb {
  int64_t q;
  uint64_t qone;
  uint64_t minv[2];  // the m^-1 pair (Word<WIDE>::Pair, 16 or 8 bytes)
};

// limb group of a tile (limb groups vary fastest, tile_ctx)
__device__ __forceinline__ int64_t tile_group(const NttArgs &g, uint32_t tile) {
  if (g.fast_bid) return (int64_t)(tile - fastdiv(tile, g.fd_groups) * g.fd_groups.d);
  return (int64_t)tile % g.ngroups_t;
}

// Offset (in pairs) of the twiddle row of limb t0 + c of `tile`, or 0 past
// the last tile.  Loaded one iteration before the fill that uses it.
template <int C>
__device__ __forceinline__ int64_t staged_tw_row(const NttArgs &g, uint32_t tile, uint32_t ntiles, int c) {
  if (tile >= ntiles) return 0;
  int64_t t = tile_group(g, tile) * C + c;
  if (t >= g.k) t = g.k - 1;
  return (g.tw_rowmap ? (int64_t)__ldg(g.tw_rowmap + t) : t) * g.m;
}

// Issues the cp.async copies of one tile into `stage`; tw_off is the twiddle
// row of the limb whose twiddles this thread copies (limb threadIdx.x / TPL).
template <typename T, int MODE, bool INV, int LOGP, int C, int MINB>
__device__ __forceinline__ void staged_fill(const NttArgs &g, const TileCtx &x, unsigned char *stage, int64_t tw_off) {
  typedef StagedShape<T, MODE, INV, LOGP, C, MINB> S;
  typedef typename S::Pair Pair;
  const int tid = threadIdx.x;
  // row segments: this thread's chunks are column c0 of rows s0 + RSTEP * i
  {
    T *data = reinterpret_cast<T *>(stage);
    const int c0 = (tid % S::CPR) * S::EPC, s0 = tid / S::CPR;
    const int ia = tidx(s0, c0, S::LOGC);
    if (x.t0 + c0 < g.k) {
      const T *base = (const T *)g.src + (x.i * g.ss[0] + x.j * g.ss[2] + x.t0 + c0);
#pragma unroll
      for (int i = 0; i < S::DATA_ITERS; ++i) {
        int64_t row = x.row_of(g, s0 + S::RSTEP * i);
        if (g.load_map) row = perm_row(g, g.load_map, row);
        cp_async16(data + (ia ^ (swz_of(S::RSTEP * i) << S::LOGC)), base + row * g.ss[1]);
      }
    } else {  // limbs past k: zeros (never stored; keep the exact-path test quiet)
#pragma unroll
      for (int i = 0; i < S::DATA_ITERS; ++i)
        *reinterpret_cast<uint4 *>(data + (ia ^ (swz_of(S::RSTEP * i) << S::LOGC))) = make_uint4(0, 0, 0, 0);
    }
  }
  // per-limb constants
  if (tid < C) {
    StagedLimb *lim = reinterpret_cast<StagedLimb *>(stage + S::DATA_BYTES + S::TW_BYTES) + tid;
    const int64_t t = x.t0 + tid < g.k ? x.t0 + tid : g.k - 1;
    cp_async8(&lim->q, g.q + t);
    if (MODE == MODE_W64_GROW) cp_async8(&lim->qone, g.qone + t);
    if (g.scale) {
      if (sizeof(Pair) == 16) cp_async16(lim->minv, (const Pair *)g.minv_pairs + t);
      else cp_async8(lim->minv, (const Pair *)g.minv_pairs + t);
    }
  }
  // twiddles: slot h of limb c = tw[(G - 1) 2^lv + h], lv = floor(log2 h)
  {
    const int ctw = tid / S::TPL, lane = tid % S::TPL;
    const Pair *row = (const Pair *)g.tw_pairs + tw_off;
    Pair *dst = reinterpret_cast<Pair *>(stage + S::DATA_BYTES) + ctw * S::TWROW;
    const int64_t G1 = x.G - 1;
#pragma unroll
    for (int i = 0; i < S::TW_ITERS; ++i) {
      const int h = (lane + S::TPL * i) * S::PPC;
      if (h == 0) {  // slot 0 is unused; with 8-byte pairs the chunk's second pair is slot 1 = tw[G]
        if (S::PPC == 2) cp_async8(dst + 1, row + G1 + 1);
        continue;
      }
      const int lv = 31 - __clz(h);
      cp_async16(dst + h, row + (G1 << lv) + h);
    }
  }
}

template <typename T, int MODE, bool INV, int LOGP, int C, int MINB>
__device__ __forceinline__ void staged_tile(const NttArgs &g, const TileCtx &x, unsigned char *stage, bool call_exact) {
  typedef StagedShape<T, MODE, INV, LOGP, C, MINB> S;
  typedef typename S::W W;
  typedef typename S::Pair Pair;
  constexpr bool WIDE = S::WIDE;
  constexpr bool LAZY = MODE != MODE_N32;
  constexpr int kLPT = S::kLPT, kPT = S::kPT, NSTEP = S::NSTEP, LOGC = S::LOGC;
  const int c = threadIdx.x & (C - 1);
  const int r = threadIdx.x >> LOGC;
  const StagedLimb &lim = reinterpret_cast<const StagedLimb *>(stage + S::DATA_BYTES + S::TW_BYTES)[c];
  const int64_t q64 = lim.q;
  T *data = reinterpret_cast<T *>(stage);

  // the thread's points of the first step (step-0 layout): one per-thread
  // base XOR a per-point constant, as in the exchanges
  T raw[kPT];
  int neg = 0;
  {
    const int ia = tidx(point_of<INV, LOGP, kLPT>(0, r, 0), c, LOGC);
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      raw[e] = data[ia ^ (swz_of(point_of<INV, LOGP, kLPT>(0, 0, e)) << LOGC)];
      neg |= needs_exact<INV>(g, (int64_t)raw[e], q64);
    }
  }
  if (__syncthreads_or(neg) || call_exact) {
    // the reference's arithmetic on an int64 tile: the data region itself for
    // 64-bit elements (each thread rewrites the words it read), the twiddle
    // region for 32-bit ones (nothing reads it on this path)
    int64_t *et = sizeof(T) == 8 ? reinterpret_cast<int64_t *>(data)
                                 : reinterpret_cast<int64_t *>(stage + S::DATA_BYTES);
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      int64_t w = (int64_t)raw[e];
      if (g.unreduced_in && w >= q64) w %= q64;
      et[tidx(point_of<INV, LOGP, kLPT>(0, r, e), c, LOGC)] = w;
    }
    __syncthreads();
    exact_tile<T, INV>(g, x, et);
    return;
  }

  const W q = (W)q64;
  W v[kPT];
  int big = 0;
#pragma unroll
  for (int e = 0; e < kPT; ++e) {
    v[e] = (W)(uint64_t)(int64_t)raw[e];
    big |= (uint64_t)(int64_t)raw[e] >= (uint64_t)q64;
  }
  if (g.canon_load && big) {  // non-canonical input (rare): reduce it first
#pragma unroll
    for (int e = 0; e < kPT; ++e) v[e] = (W)((uint64_t)(int64_t)raw[e] % (uint64_t)q64);
  }
  // 64-bit elements under a 32-bit mode exchange 4-byte words at other offsets
  if (sizeof(T) != sizeof(W)) __syncthreads();
  const Pair *tws = reinterpret_cast<const Pair *>(stage + S::DATA_BYTES) + c * S::TWROW;
  reg_steps<MODE, INV, LOGP, 0, true>(v, r, c, LOGC, reinterpret_cast<int64_t *>(data), 1, tws, q);

  // back to canonical residues, as ntt_reg_body does
  if (MODE == MODE_W64_GROW) {
    if (INV ? !g.scale : !g.lazy_out) {
      const W one = (W)lim.qone;
#pragma unroll
      for (int e = 0; e < kPT; ++e) {
        const W u = v[e] - (W)mulhi64((uint64_t)v[e], (uint64_t)one) * q;
        v[e] = u >= q ? u - q : u;
      }
    }
  } else {  // 32-bit words: forward lazy values < 4q, otherwise < 2q
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      W u = v[e];
      if (LAZY && !INV) u = u >= q + q ? u - (q + q) : u;
      v[e] = u >= q ? u - q : u;
    }
  }
  if (g.scale) {
    const Pair mp = *reinterpret_cast<const Pair *>(lim.minv);
#pragma unroll
    for (int e = 0; e < kPT; ++e) v[e] = mulw<WIDE>(v[e], mp, q);
  }
  // results into the stage in the last step's layout (the words this thread
  // read in that step, when elements and words have one size), then out as
  // 16-byte row segments
  if (sizeof(T) != sizeof(W)) __syncthreads();
  {
    const int ia = tidx(point_of<INV, LOGP, kLPT>(NSTEP - 1, r, 0), c, LOGC);
#pragma unroll
    for (int e = 0; e < kPT; ++e)
      data[ia ^ (swz_of(point_of<INV, LOGP, kLPT>(NSTEP - 1, 0, e)) << LOGC)] = (T)(int64_t)v[e];
  }
  __syncthreads();
  {
    const int tid = threadIdx.x;
    const int c0 = (tid % S::CPR) * S::EPC, s0 = tid / S::CPR;
    if (x.t0 + c0 < g.k) {
      const int ia = tidx(s0, c0, LOGC);
      T *base = (T *)g.dst + (x.i * g.ds[0] + x.j * g.ds[2] + x.t0 + c0);
#pragma unroll
      for (int i = 0; i < S::DATA_ITERS; ++i) {
        int64_t row = x.row_of(g, s0 + S::RSTEP * i);
        if (g.store_scatter) row = perm_row(g, g.store_scatter, row);
        *reinterpret_cast<uint4 *>(base + row * g.ds[1]) =
            *reinterpret_cast<const uint4 *>(data + (ia ^ (swz_of(S::RSTEP * i) << LOGC)));
      }
    }
  }
}

template <typename T, int MODE, bool INV, int LOGP, int C, int MINB>
__global__ void __launch_bounds__(StagedShape<T, MODE, INV, LOGP, C, MINB>::THREADS, MINB)
    ntt_staged_kernel(const __grid_constant__ NttArgs g, uint32_t ntiles) {
  typedef StagedShape<T, MODE, INV, LOGP, C, MINB> S;
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t tile = blockIdx.x;
  if (tile >= ntiles) return;
  // call-wide reasons for the exact path (negative twiddles or m^-1, m = 1, q >= 2^62)
  const bool call_exact = g.force_exact || (g.tw_neg && *g.tw_neg) || (g.scale && g.minv_neg && *g.minv_neg);
  const int ctw = threadIdx.x / S::TPL;  // the limb whose twiddles this thread copies
  TileCtx x = tile_ctx(g, tile);
  staged_fill<T, MODE, INV, LOGP, C, MINB>(g, x, smem, staged_tw_row<C>(g, tile, ntiles, ctw));
  cp_async_commit();
  int64_t tw_next = staged_tw_row<C>(g, tile + gridDim.x, ntiles, ctw);
  for (int it = 0; tile < ntiles; ++it, tile += gridDim.x) {
    unsigned char *cur = smem + (it & 1) * S::STAGE_BYTES;
    cp_async_wait_all();
    // every thread's copies of this tile have landed, and the other stage's
    // last tile has been stored: refill it with the next tile
    __syncthreads();
    const uint32_t next = tile + gridDim.x;
    const int64_t tw_after = staged_tw_row<C>(g, next + gridDim.x, ntiles, ctw);  // used one iteration on
    TileCtx xn;
    if (next < ntiles) {
      xn = tile_ctx(g, next);
      staged_fill<T, MODE, INV, LOGP, C, MINB>(g, xn, smem + ((it + 1) & 1) * S::STAGE_BYTES, tw_next);
      cp_async_commit();
    }
    staged_tile<T, MODE, INV, LOGP, C, MINB>(g, x, cur, call_exact);
    x = xn;
    tw_next = tw_after;
  }
}

}  // namespace heal
