// heal_ntt_staged.cuh — the staged NTT pass kernel (included by heal_ntt_*.cu).
//
// The same pass as ntt_reg_kernel (heal_ntt_kernels.cuh: a P-point piece of
// HEAL's butterfly network on C adjacent limbs, register radix steps
// exchanging through a swizzled shared tile, the same arithmetic modes),
// organised so that no global load sits on the compute path:
//
//  * Persistent CTAs.  A CTA keeps one limb group (C adjacent limbs) and
//    walks a contiguous run of the (set or block, slice) tiles of it, so its
//    limbs' constants (q, floor(2^64 / q), m^-1) and twiddle rows are fixed,
//    and the tiles that share twiddles (every tile of a strided pass, the
//    l * r slices of one block) follow one another.
//  * Row segments in two shared-memory stages.  While tile i computes in
//    one, the other fills with tile i+1 through cp.async (16-byte LDGSTS, no
//    register round trip), laid out in the exchange layout tidx(s, c) so the
//    first step reads them conflict-free.
//  * Twiddles in two shared-memory buffers, P - 1 pairs per limb by heap
//    slot h = 2^lv + g (stage lv of the forward network, stage LOGP - 1 - lv
//    of the inverse): the pass's twiddle of slot h is tw[(G - 1) 2^lv + h],
//    one contiguous run of 2^lv pairs per stage.  A buffer is refilled only
//    when the next tile's block G differs from the current tile's.
//  * 16 points per thread in the 32-bit word modes (two radix-16 steps and
//    one exchange per 256-point pass).
//  * The results go back through the data stage in the exchange layout and
//    leave as 16-byte row-segment stores (bit-reversal scatter included).
//
// The host sends it the 256-point passes of int32 tensors, where it measured
// faster than the register kernel; the 64-bit growing-range passes stay on
// the register kernel, which measured faster for them (ablations, in copies
// never committed, showed those passes bound by neither their butterfly
// arithmetic nor their exchanges: their per-tile structure is the cost).
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
  // 16 points per thread in the 32-bit word modes, else the register kernel's choice
  static constexpr int kLPT = WIDE ? lpt_of(MODE, INV) : 4, kPT = 1 << kLPT;
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
  static constexpr int SMEM_BYTES = 2 * DATA_BYTES + 2 * TW_BYTES + LIMB_BYTES;
  static constexpr int MINB = MINB_;                   // resident CTAs per SM the register budget allows
  static_assert((P / PPC) % TPL == 0, "twiddle chunks split evenly");
  static_assert(C % EPC == 0 && THREADS % CPR == 0 && NCHUNK % THREADS == 0, "row chunks split evenly");
  static_assert((RSTEP & (RSTEP - 1)) == 0, "a thread's rows differ in disjoint bits");
  static_assert(THREADS % C == 0, "whole threads per limb");
};

// per-limb constants of the CTA's limb group
struct StagedLimb {
  int64_t q;
  uint64_t qone;
  uint64_t minv[2];  // the m^-1 pair (Word<WIDE>::Pair, 16 or 8 bytes)
};

// Issues the cp.async copies of one tile's row segments into `data`.
template <typename T, int MODE, bool INV, int LOGP, int C, int MINB>
__device__ __forceinline__ void staged_fill_rows(const NttArgs &g, const TileCtx &x, T *data) {
  typedef StagedShape<T, MODE, INV, LOGP, C, MINB> S;
  const int tid = threadIdx.x;
  const int c0 = (tid % S::CPR) * S::EPC, s0 = tid / S::CPR;  // column c0 of rows s0 + RSTEP * i
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

// Issues the cp.async copies of the twiddles of block G (1 for strided
// sets): slot h of limb c = tw[(G - 1) 2^lv + h], lv = floor(log2 h).  `row`
// is the twiddle row of the limb this thread copies (threadIdx.x / TPL).
template <typename T, int MODE, bool INV, int LOGP, int C, int MINB>
__device__ __forceinline__ void staged_fill_twiddles(const typename StagedShape<T, MODE, INV, LOGP, C, MINB>::Pair *row,
                                                     int64_t G,
                                                     typename StagedShape<T, MODE, INV, LOGP, C, MINB>::Pair *tw) {
  typedef StagedShape<T, MODE, INV, LOGP, C, MINB> S;
  typedef typename S::Pair Pair;
  const int ctw = threadIdx.x / S::TPL, lane = threadIdx.x % S::TPL;
  Pair *dst = tw + ctw * S::TWROW;
  const int64_t G1 = G - 1;
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

template <typename T, int MODE, bool INV, int LOGP, int C, int MINB>
__device__ __forceinline__ void staged_tile(const NttArgs &g, uint32_t tile, const TileCtx &x, T *data,
                                            const typename StagedShape<T, MODE, INV, LOGP, C, MINB>::Pair *tw,
                                            const StagedLimb *limbs, bool call_exact) {
  typedef StagedShape<T, MODE, INV, LOGP, C, MINB> S;
  typedef typename S::W W;
  typedef typename S::Pair Pair;
  constexpr bool WIDE = S::WIDE;
  constexpr bool LAZY = MODE != MODE_N32;
  constexpr int kLPT = S::kLPT, kPT = S::kPT, NSTEP = S::NSTEP, LOGC = S::LOGC;
  const int c = threadIdx.x & (C - 1);
  const int r = threadIdx.x >> LOGC;
  const StagedLimb &lim = limbs[c];
  const int64_t q64 = lim.q;

  // the thread's points of the first step (step-0 layout): one per-thread
  // base XOR a per-point constant, as in the exchanges.  The rare paths below
  // re-read the stage instead of keeping the raw words in registers.
  const W q = (W)q64;
  const int ia0 = tidx(point_of<INV, LOGP, kLPT>(0, r, 0), c, LOGC);
  W v[kPT];
  int neg = 0, big = 0;
#pragma unroll
  for (int e = 0; e < kPT; ++e) {
    const T w = data[ia0 ^ (swz_of(point_of<INV, LOGP, kLPT>(0, 0, e)) << LOGC)];
    v[e] = (W)(uint64_t)(int64_t)w;
    neg |= needs_exact<INV>(g, (int64_t)w, q64);
    big |= (uint64_t)(int64_t)w >= (uint64_t)q64;
  }
  if (__syncthreads_or(neg) || call_exact) {
    // the reference's arithmetic on the data stage itself, which still holds
    // the raw words; a growing-range first pass's unreduced values are reduced
    // first (each thread its own words), as the register kernel does
    if (g.unreduced_in) {
#pragma unroll
      for (int e = 0; e < kPT; ++e) {
        const int ix = ia0 ^ (swz_of(point_of<INV, LOGP, kLPT>(0, 0, e)) << LOGC);
        const int64_t w = (int64_t)data[ix];
        if (w >= q64) data[ix] = (T)(w % q64);
      }
    }
    __syncthreads();
    exact_tile<T, INV, T>(g, tile, data);
    return;
  }
  // forward: reduce a non-canonical input first (rare); the inverse sent
  // values >= q to the exact path above
  if (!INV && g.canon_load && big) {
#pragma unroll
    for (int e = 0; e < kPT; ++e) {
      const uint64_t w = (uint64_t)(int64_t)data[ia0 ^ (swz_of(point_of<INV, LOGP, kLPT>(0, 0, e)) << LOGC)];
      v[e] = sizeof(T) == 4 ? (W)((uint32_t)w % (uint32_t)q64) : (W)(w % (uint64_t)q64);
    }
  }
  // 64-bit elements under a 32-bit mode exchange 4-byte words at other offsets
  if (sizeof(T) != sizeof(W)) __syncthreads();
  reg_steps<MODE, INV, LOGP, 0, true, kLPT>(v, r, c, LOGC, reinterpret_cast<int64_t *>(data), 1, tw + c * S::TWROW, q);

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
  } else {  // forward lazy values < 4q, otherwise < 2q
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

// Grid: ngroups * shares CTAs; CTA b keeps limb group b % ngroups and runs
// the units u of [u_begin, u_end) of its share, u = set * (l * r) + slice
// (the tile index is u * ngroups + group, tile_ctx's order).
template <typename T, int MODE, bool INV, int LOGP, int C, int MINB>
__global__ void __launch_bounds__(StagedShape<T, MODE, INV, LOGP, C, MINB>::THREADS, MINB)
    ntt_staged_kernel(const __grid_constant__ NttArgs g, uint32_t nunits) {
  typedef StagedShape<T, MODE, INV, LOGP, C, MINB> S;
  typedef typename S::Pair Pair;
  extern __shared__ __align__(16) unsigned char smem[];
  // stage i at smem + i * DATA_BYTES, twiddle buffer b at smem + 2 * DATA_BYTES + b * TW_BYTES
  auto stage = [&](uint32_t i) { return reinterpret_cast<T *>(smem + (i & 1) * S::DATA_BYTES); };
  auto twb = [&](int b) { return reinterpret_cast<Pair *>(smem + 2 * S::DATA_BYTES + b * S::TW_BYTES); };
  StagedLimb *limbs = reinterpret_cast<StagedLimb *>(smem + 2 * S::DATA_BYTES + 2 * S::TW_BYTES);
  const uint32_t ngroups = (uint32_t)g.ngroups_t;
  const uint32_t tg = blockIdx.x % ngroups, share = blockIdx.x / ngroups, shares = gridDim.x / ngroups;
  const uint32_t u_begin = (uint32_t)((uint64_t)share * nunits / shares);
  const uint32_t u_end = (uint32_t)((uint64_t)(share + 1) * nunits / shares);
  if (u_begin >= u_end) return;
  // call-wide reasons for the exact path (negative twiddles or m^-1, m = 1, q >= 2^62)
  const bool call_exact = g.force_exact || (g.tw_neg && *g.tw_neg) || (g.scale && g.minv_neg && *g.minv_neg);
  // the limb group's constants and this thread's twiddle row, once
  const int64_t t0 = (int64_t)tg * C;
  if (threadIdx.x < C) {
    const int64_t t = t0 + threadIdx.x < g.k ? t0 + threadIdx.x : g.k - 1;
    StagedLimb &l = limbs[threadIdx.x];
    l.q = g.q[t];
    l.qone = MODE == MODE_W64_GROW ? g.qone[t] : 0;
    if (g.scale) *reinterpret_cast<Pair *>(l.minv) = ((const Pair *)g.minv_pairs)[t];
  }
  const Pair *twrow;
  {
    int64_t t = t0 + threadIdx.x / S::TPL;
    if (t >= g.k) t = g.k - 1;
    twrow = (const Pair *)g.tw_pairs + (g.tw_rowmap ? (int64_t)g.tw_rowmap[t] : t) * g.m;
  }
  TileCtx x = tile_ctx(g, u_begin * ngroups + tg);
  staged_fill_rows<T, MODE, INV, LOGP, C, MINB>(g, x, stage(0));
  staged_fill_twiddles<T, MODE, INV, LOGP, C, MINB>(twrow, x.G, twb(0));
  cp_async_commit();
  int64_t key0 = x.G, key1 = -1;  // the block whose twiddles each buffer holds (uniform over the CTA)
  int cb = 0;                     // buffer of the current tile
  for (uint32_t u = u_begin, it = 0; u < u_end; ++u, ++it) {
    cp_async_wait_all();
    // every thread's copies of this tile have landed, and the last tile that
    // used the other stage (and the other twiddle buffer) is done
    __syncthreads();
    TileCtx xn;
    int nb = cb;
    if (u + 1 < u_end) {
      xn = tile_ctx(g, (u + 1) * ngroups + tg);
      staged_fill_rows<T, MODE, INV, LOGP, C, MINB>(g, xn, stage(it + 1));
      if (xn.G != (cb ? key1 : key0)) {
        nb = cb ^ 1;
        staged_fill_twiddles<T, MODE, INV, LOGP, C, MINB>(twrow, xn.G, twb(nb));
        if (nb) key1 = xn.G;
        else key0 = xn.G;
      }
      cp_async_commit();
    }
    staged_tile<T, MODE, INV, LOGP, C, MINB>(g, u * ngroups + tg, x, stage(it), twb(cb), limbs, call_exact);
    x = xn;
    cb = nb;
  }
}

}  // namespace heal
