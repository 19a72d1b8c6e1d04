// heal_ntt.cu — batched negacyclic NTT / INTT over HEAL's [l, m, r, k]
// layout (moduli innermost), HEAL include/ntt.h:31-52.
//
// The transform is the butterfly network of example_impl/ntt_impl.cpp:
//   forward  Cooley-Tukey, stage with 2^st groups uses twiddles[t, 2^st + g]
//            (ntt_impl.cpp:92-110), then out[u] = res[perm[u]] (:46-65);
//   inverse  res[perm[u]] = a[u] (:138-141), Gentleman-Sande with
//            inv_twiddles[t, m/2^(g+1) + group] (:143-161), times m_inv (:163-166).
// The same twiddle meets the same butterfly here, so the output equals the
// reference's for any twiddle table, not only for powers of one root.
//
// Work decomposition.  A column is one (i, j, t) polynomial of m points
// spaced r*k elements apart.  A CTA owns a tile of P points x C adjacent
// limbs (t0 .. t0+C-1), so each of its global loads reads C*sizeof(T)
// contiguous bytes of a row.  For m <= 4096 one pass holds whole columns
// (P = m).  Larger m splits the network in two passes: the first log2(P1)
// forward stages only combine points congruent mod m/P1 (strided sets), the
// remaining stages only points inside contiguous blocks of m/P1.  The inverse
// is the mirror image.  Inside a pass the tile is a local P-point network
// whose twiddle index is G * 2^st + group (forward) or G * (P >> (g+1)) +
// group (inverse), with G = 1 for strided sets and G = m/P + block for
// contiguous blocks.
//
// Arithmetic: canonical inputs (0 <= x) use Shoup multiplication with the
// twiddle's precomputed companion, 32-bit words when every q < 2^31 and
// 64-bit words otherwise, with every value kept in [0, q).  A tile that
// holds a negative value (or any call whose twiddles / m_inv are negative)
// runs the reference's own arithmetic instead: C's truncating `%` in
// __int128, step by step, which is bit-identical to example_impl.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "heal_internal.h"

namespace heal {

enum { KIND_STRIDED = 0, KIND_BLOCK = 1 };
constexpr int kNttThreads = 256;
constexpr int kSinglePassLogMax = 12;  // m <= 4096 in one pass

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
  int64_t nsets;     // sets (strided) or blocks per column
  int64_t ngroups_t; // ceil(k / C)
  const int32_t *load_map;
  const int32_t *store_gather;
  const int32_t *store_scatter;
  const void *tw_pairs;
  const int *tw_neg;
  const void *tw_raw;
  int64_t tw_s0, tw_s1;
  const int64_t *q;
  const void *minv_pairs;
  const int *minv_neg;
  const void *minv_raw;
  int64_t minv_s0;
  int scale;
  int canon_load;
  int force_exact;
};

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

template <bool WIDE>
__device__ __forceinline__ typename Word<WIDE>::W mulw(typename Word<WIDE>::W y, typename Word<WIDE>::Pair pr,
                                                        typename Word<WIDE>::W q) {
  if (WIDE)
    return (typename Word<WIDE>::W)shoup64((uint64_t)y, (uint64_t)pr.x, (uint64_t)pr.y, (uint64_t)q);
  return (typename Word<WIDE>::W)shoup32((uint32_t)y, (uint32_t)pr.x, (uint32_t)pr.y, (uint32_t)q);
}

template <typename T>
__device__ __forceinline__ int64_t ld_raw(const void *base, int64_t off) {
  return (int64_t)((const T *)base)[off];
}

__device__ __forceinline__ int64_t raw_any(const void *base, int64_t off, bool is32) {
  return is32 ? (int64_t)((const int32_t *)base)[off] : ((const int64_t *)base)[off];
}

template <typename T, bool WIDE, bool INV>
__global__ void __launch_bounds__(kNttThreads) ntt_pass_kernel(const __grid_constant__ NttArgs g) {
  typedef typename Word<WIDE>::W W;
  typedef typename Word<WIDE>::Pair Pair;
  extern __shared__ __align__(16) int64_t tile[];

  const int P = 1 << g.p;
  const int C = g.C, logC = g.logC;
  const int64_t bid = blockIdx.x;
  const int64_t rset = bid % g.nsets;
  const int64_t cg = bid / g.nsets;
  const int64_t tg = cg % g.ngroups_t;
  const int64_t ij = cg / g.ngroups_t;
  const int64_t j = ij % g.r, i = ij / g.r;
  const int64_t t0 = tg * C;
  const bool is32 = sizeof(T) == 4;

  auto row_of = [&](int64_t s) -> int64_t {
    return g.kind == KIND_BLOCK ? rset * P + s : rset + s * g.nsets;
  };

  // ---- load the tile (raw values)
  int neg = 0;
  const int64_t sb = i * g.ss[0] + j * g.ss[2];
  for (int e = threadIdx.x; e < P * C; e += blockDim.x) {
    const int s = e >> logC, c = e & (C - 1);
    const int64_t t = t0 + c;
    if (t >= g.k) continue;
    const int64_t v = row_of(s);
    int64_t x;
    if (g.load_map) {
      const int32_t sr = g.load_map[v];
      if (sr < 0)
        x = ld_raw<T>(g.old, i * g.os[0] + v * g.os[1] + j * g.os[2] + t * g.os[3]);
      else
        x = ld_raw<T>(g.src, sb + (int64_t)sr * g.ss[1] + t * g.ss[3]);
    } else {
      x = ld_raw<T>(g.src, sb + v * g.ss[1] + t * g.ss[3]);
    }
    // Negative values always need the reference's arithmetic.  For the
    // inverse so do values >= q: its first butterfly forms u + q - v, which
    // goes negative when v > u + q.  The forward NTT reduces them instead
    // (its stage-1 outputs are canonical whenever the inputs are >= 0).
    neg |= x < 0 || (INV && g.canon_load && x >= g.q[t]);
    tile[e] = x;
  }
  bool exact = __syncthreads_or(neg) || g.force_exact || (g.tw_neg && *g.tw_neg) ||
               (g.scale && g.minv_neg && *g.minv_neg);

  const int64_t G = g.kind == KIND_BLOCK ? g.nsets + rset : 1;
  const int nbf = (P >> 1) * C;

  if (!exact) {
    // ---- fast path: canonical residues, Shoup butterflies
    if (g.canon_load) {
      for (int e = threadIdx.x; e < P * C; e += blockDim.x) {
        const int64_t t = t0 + (e & (C - 1));
        if (t >= g.k) continue;
        const uint64_t q = (uint64_t)g.q[t];
        const uint64_t x = (uint64_t)tile[e];
        if (x >= q) tile[e] = (int64_t)(x % q);
      }
      __syncthreads();
    }
    for (int st = 0; st < g.p; ++st) {
      for (int b = threadIdx.x; b < nbf; b += blockDim.x) {
        const int c = b & (C - 1);
        const int64_t t = t0 + c;
        if (t >= g.k) continue;
        const int jb = b >> logC;
        int su, sv;
        int64_t twidx;
        if (!INV) {
          const int hl = g.p - 1 - st;  // log2 of the pair distance
          const int grp = jb >> hl;
          su = (grp << (hl + 1)) + (jb & ((1 << hl) - 1));
          sv = su + (1 << hl);
          twidx = (G << st) + grp;
        } else {
          const int grp = jb >> st;
          su = (grp << (st + 1)) + (jb & ((1 << st) - 1));
          sv = su + (1 << st);
          twidx = G * (int64_t)(P >> (st + 1)) + grp;
        }
        const W q = (W)g.q[t];
        const Pair pr = __ldg((const Pair *)g.tw_pairs + t * g.m + twidx);
        const W u = (W)tile[(su << logC) + c];
        const W v = (W)tile[(sv << logC) + c];
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
        tile[(su << logC) + c] = (int64_t)nu;
        tile[(sv << logC) + c] = (int64_t)nv;
      }
      __syncthreads();
    }
  } else {
    // ---- exact path: the reference's arithmetic, C's `%` in __int128
    for (int st = 0; st < g.p; ++st) {
      for (int b = threadIdx.x; b < nbf; b += blockDim.x) {
        const int c = b & (C - 1);
        const int64_t t = t0 + c;
        if (t >= g.k) continue;
        const int jb = b >> logC;
        int su, sv;
        int64_t twidx;
        if (!INV) {
          const int hl = g.p - 1 - st;
          const int grp = jb >> hl;
          su = (grp << (hl + 1)) + (jb & ((1 << hl) - 1));
          sv = su + (1 << hl);
          twidx = (G << st) + grp;
        } else {
          const int grp = jb >> st;
          su = (grp << (st + 1)) + (jb & ((1 << st) - 1));
          sv = su + (1 << st);
          twidx = G * (int64_t)(P >> (st + 1)) + grp;
        }
        const int64_t q = g.q[t];
        const int64_t s = raw_any(g.tw_raw, t * g.tw_s0 + twidx * g.tw_s1, is32);
        const int64_t u = tile[(su << logC) + c];
        const int64_t v = tile[(sv << logC) + c];
        int64_t nu, nv;
        if (!INV) {
          const int64_t vm = crem128((i128)v * s, q);
          nu = crem128((i128)u + vm, q);
          nv = crem128((i128)u + q - vm, q);
        } else {
          nu = crem128((i128)u + v, q);
          nv = crem128(((i128)u + q - v) * s, q);
        }
        tile[(su << logC) + c] = nu;
        tile[(sv << logC) + c] = nv;
      }
      __syncthreads();
    }
  }

  // ---- store
  const int64_t db = i * g.ds[0] + j * g.ds[2];
  for (int e = threadIdx.x; e < P * C; e += blockDim.x) {
    const int s = e >> logC, c = e & (C - 1);
    const int64_t t = t0 + c;
    if (t >= g.k) continue;
    int64_t x = g.store_gather ? tile[((int)g.store_gather[s] << logC) + c] : tile[e];
    if (g.scale) {
      const int64_t q = g.q[t];
      if (!exact) {
        const Pair pr = __ldg((const Pair *)g.minv_pairs + t);
        x = (int64_t)mulw<WIDE>((W)x, pr, (W)q);
      } else {
        x = crem128((i128)x * raw_any(g.minv_raw, t * g.minv_s0, is32), q);
      }
    }
    const int64_t v = row_of(s);
    const int64_t dr = g.store_scatter ? (int64_t)g.store_scatter[v] : v;
    ((T *)g.dst)[db + dr * g.ds[1] + t * g.ds[3]] = (T)x;
  }
}

// out[i, u, j, t] = src[i, perm[u], j, t] (forward NTT with a non-bijective
// permutation after the two-pass transform)
template <typename T>
__global__ void __launch_bounds__(256) ntt_gather_kernel(const T *src, int64_t s0, int64_t s1, int64_t s2, int64_t s3,
                                                         T *dst, int64_t d0, int64_t d1, int64_t d2, int64_t d3,
                                                         const int32_t *perm, int64_t l, int64_t m, int64_t r,
                                                         int64_t k) {
  const int64_t n = l * m * r * k;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t t = idx % k, rest = idx / k;
    int64_t j = rest % r;
    rest /= r;
    int64_t u = rest % m, i = rest / m;
    dst[i * d0 + u * d1 + j * d2 + t * d3] = src[i * s0 + (int64_t)perm[u] * s1 + j * s2 + t * s3];
  }
}

// ----------------------------------------------------------- host side
template <typename T, bool WIDE, bool INV>
static int launch_pass(const NttArgs &a, int64_t nblocks) {
  const size_t smem = (size_t)(1 << a.p) * a.C * sizeof(int64_t);
  static bool attr_set = false;
  if (!attr_set) {
    HEAL_TRY_CUDA(
        cudaFuncSetAttribute(ntt_pass_kernel<T, WIDE, INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    attr_set = true;
  }
  ntt_pass_kernel<T, WIDE, INV><<<(unsigned)nblocks, kNttThreads, smem, stream()>>>(a);
  return check_launch("ntt_pass");
}

static int launch_any(const NttArgs &a, int64_t nblocks, bool is32, bool wide, bool inv) {
  if (is32) {
    if (wide) return inv ? launch_pass<int32_t, true, true>(a, nblocks) : launch_pass<int32_t, true, false>(a, nblocks);
    return inv ? launch_pass<int32_t, false, true>(a, nblocks) : launch_pass<int32_t, false, false>(a, nblocks);
  }
  if (wide) return inv ? launch_pass<int64_t, true, true>(a, nblocks) : launch_pass<int64_t, true, false>(a, nblocks);
  return inv ? launch_pass<int64_t, false, true>(a, nblocks) : launch_pass<int64_t, false, false>(a, nblocks);
}

static void set_strides(int64_t *dst, const heal_tensor &t) {
  for (int i = 0; i < 4; ++i) dst[i] = t.strides[i];
}

static int ilog2(int64_t x) {
  int r = 0;
  while ((int64_t(1) << r) < x) ++r;
  return r;
}

static int ntt_run(bool inv, const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm,
                   const heal_tensor *tw, const heal_tensor *minv, const heal_tensor *res) {
  clear_error();
  HEAL_CHECK(check_desc(a, "a", true));
  HEAL_CHECK(check_desc(p, "p", true));
  HEAL_CHECK(check_desc(perm, "perm", true));
  HEAL_CHECK(check_desc(tw, inv ? "inv_twiddles" : "twiddles", true));
  HEAL_CHECK(check_desc(res, "result", true));
  HEAL_CHECK(ensure_init());
  // validate_ntt_inputs (ntt_impl.cpp:15-43)
  if (a->ndim != 4) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Input tensor 'a' must have shape [l, m, r, k].");
  const int64_t l = a->dims[0], m = a->dims[1], r = a->dims[2], k = a->dims[3];
  if (!same_dims(*a, *res))
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "Output tensor must have the same shape as input tensor.");
  if (p->ndim != 1 || p->dims[0] != k) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Tensor 'p' must have shape [k].");
  if (perm->ndim != 1 || perm->dims[0] != m)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "Tensor 'perm' must have shape [m].");
  if (tw->ndim != 2 || tw->dims[0] != k || tw->dims[1] != m)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "Tensor 'twiddles' must have shape [k, m].");
  const int dt = a->dtype;
  if (res->dtype != dt || p->dtype != dt || perm->dtype != dt || tw->dtype != dt)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "all tensors must have the element type of a");
  if (m == 0 || l * r * k == 0) return HEAL_OK;
  if (inv) {
    // m_inv->at({t}) (ntt_impl.cpp:136): one index, t < dims[0]
    if (!minv) return set_error(HEAL_ERR_INVALID_ARGUMENT, "m_inv pointer must not be null.");
    HEAL_CHECK(check_desc(minv, "m_inv", true));
    if (minv->dtype != dt) return set_error(HEAL_ERR_INVALID_ARGUMENT, "all tensors must have the element type of a");
    if (minv->ndim != 1)
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "Number of indices does not match tensor dimensions.");
    if (minv->dims[0] < k) return set_error(HEAL_ERR_OUT_OF_RANGE, "Index out of bounds.");
  }
  // a non-power-of-two length makes the reference index past the twiddle
  // row (ntt_impl.cpp:99) or past the column (:151-152)
  if (m > 2 && (m & (m - 1))) return set_error(HEAL_ERR_OUT_OF_RANGE, "Index out of bounds.");
  const int logm = ilog2(m);
  if (logm > 2 * kSinglePassLogMax) return set_error(HEAL_ERR_INVALID_ARGUMENT, "transform length above 2^24");

  ModInfo mi;
  HEAL_CHECK(mod_info(*p, &mi));
  if (mi.min_q <= 0) return set_error(HEAL_ERR_RUNTIME, "moduli must be positive");
  const bool wide = mi.max_q > 0x7FFFFFFF;
  PermInfo pi;
  HEAL_CHECK(perm_info(*perm, &pi));
  if (pi.bad) return set_error(HEAL_ERR_OUT_OF_RANGE, "Index out of bounds.");
  TwiddleTable tt, mt;
  HEAL_CHECK(twiddle_table(*tw, *p, wide, &tt));
  if (inv) HEAL_CHECK(minv_table(*minv, *p, k, wide, &mt));

  heal_tensor A = *a;
  void *owned_a = nullptr;
  if (overlaps(A, *res) && !identical_view(A, *res)) HEAL_CHECK(materialize(A, &A, &owned_a));

  NttArgs base;
  memset(&base, 0, sizeof base);
  base.l = l;
  base.m = m;
  base.r = r;
  base.k = k;
  base.tw_pairs = tt.pairs;
  base.tw_neg = tt.neg_flag;
  base.tw_raw = tw->data;
  base.tw_s0 = tw->strides[0];
  base.tw_s1 = tw->strides[1];
  base.q = mi.q;
  if (inv) {
    base.minv_pairs = mt.pairs;
    base.minv_neg = mt.neg_flag;
    base.minv_raw = minv->data;
    base.minv_s0 = minv->strides[0];
  }
  base.force_exact = m == 1;
  const bool is32 = dt == HEAL_INT32;
  int C = 8;
  while (C > 1 && C / 2 >= k) C /= 2;
  int rc = HEAL_OK;
  void *tmp = nullptr, *tmp2 = nullptr;

  auto cfg = [&](NttArgs &x, int pbits, int kind) -> int64_t {
    int c = C;
    while (c > 1 && ((int64_t)1 << pbits) * c > 8192) c /= 2;
    x.p = pbits;
    x.C = c;
    x.logC = ilog2(c);
    x.kind = kind;
    x.nsets = m >> pbits;
    x.ngroups_t = (k + c - 1) / c;
    return x.nsets * l * r * x.ngroups_t;
  };

  if (logm <= kSinglePassLogMax) {
    NttArgs x = base;
    int64_t nb = cfg(x, logm, KIND_BLOCK);
    x.src = A.data;
    set_strides(x.ss, A);
    x.dst = res->data;
    set_strides(x.ds, *res);
    x.canon_load = 1;
    if (inv) {
      x.load_map = pi.inv32;
      x.old = res->data;
      set_strides(x.os, *res);
      x.scale = 1;
    } else {
      x.store_gather = pi.perm32;
    }
    rc = launch_any(x, nb, is32, wide, inv);
  } else {
    // two passes through a dense [l, m, r, k] scratch tensor
    const int p1 = logm / 2, p2 = logm - p1;
    heal_tensor T1 = *res;
    int64_t s = 1;
    for (int d = 3; d >= 0; --d) {
      T1.strides[d] = s;
      s *= T1.dims[d];
    }
    rc = scratch_alloc((size_t)s * elem_size(dt), &tmp);
    T1.data = tmp;
    if (!rc && !inv) {
      NttArgs x = base;  // pass 1: first p1 stages on strided sets
      int64_t nb = cfg(x, p1, KIND_STRIDED);
      x.src = A.data;
      set_strides(x.ss, A);
      x.dst = T1.data;
      set_strides(x.ds, T1);
      x.canon_load = 1;
      rc = launch_any(x, nb, is32, wide, false);
      if (!rc) {
        NttArgs y = base;  // pass 2: remaining stages on contiguous blocks
        nb = cfg(y, p2, KIND_BLOCK);
        y.src = T1.data;
        set_strides(y.ss, T1);
        if (pi.bijective) {
          y.dst = res->data;
          set_strides(y.ds, *res);
          y.store_scatter = pi.inv32;
          rc = launch_any(y, nb, is32, wide, false);
        } else {
          heal_tensor T2 = T1;
          rc = scratch_alloc((size_t)s * elem_size(dt), &tmp2);
          T2.data = tmp2;
          y.dst = T2.data;
          set_strides(y.ds, T2);
          if (!rc) rc = launch_any(y, nb, is32, wide, false);
          if (!rc) {
            int64_t n = l * m * r * k;
            int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)device_sm_count() * 16);
            if (is32)
              ntt_gather_kernel<int32_t><<<grid, 256, 0, stream()>>>(
                  (const int32_t *)T2.data, T2.strides[0], T2.strides[1], T2.strides[2], T2.strides[3],
                  (int32_t *)res->data, res->strides[0], res->strides[1], res->strides[2], res->strides[3],
                  pi.perm32, l, m, r, k);
            else
              ntt_gather_kernel<int64_t><<<grid, 256, 0, stream()>>>(
                  (const int64_t *)T2.data, T2.strides[0], T2.strides[1], T2.strides[2], T2.strides[3],
                  (int64_t *)res->data, res->strides[0], res->strides[1], res->strides[2], res->strides[3],
                  pi.perm32, l, m, r, k);
            rc = check_launch("ntt_gather");
          }
        }
      }
    } else if (!rc) {
      NttArgs x = base;  // pass 1: first p1 inverse stages on contiguous blocks
      int64_t nb = cfg(x, p1, KIND_BLOCK);
      x.src = A.data;
      set_strides(x.ss, A);
      x.load_map = pi.inv32;
      x.old = res->data;
      set_strides(x.os, *res);
      x.dst = T1.data;
      set_strides(x.ds, T1);
      x.canon_load = 1;
      rc = launch_any(x, nb, is32, wide, true);
      if (!rc) {
        NttArgs y = base;  // pass 2: remaining stages on strided sets, then m_inv
        nb = cfg(y, p2, KIND_STRIDED);
        y.src = T1.data;
        set_strides(y.ss, T1);
        y.dst = res->data;
        set_strides(y.ds, *res);
        y.scale = 1;
        rc = launch_any(y, nb, is32, wide, true);
      }
    }
  }
  scratch_free(tmp);
  scratch_free(tmp2);
  scratch_free(owned_a);
  if (!rc) mark_written(res->data);
  return rc;
}

}  // namespace heal

using namespace heal;

extern "C" {

int heal_ntt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm, const heal_tensor *twiddles,
             const heal_tensor *log2p, const heal_tensor *mu, const heal_tensor *result) {
  (void)log2p;
  (void)mu;  // optional Barrett inputs (include/ntt.h:24-26); Shoup needs neither
  return ntt_run(false, a, p, perm, twiddles, nullptr, result);
}

int heal_intt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm, const heal_tensor *inv_twiddles,
              const heal_tensor *m_inv, const heal_tensor *log2p, const heal_tensor *mu, const heal_tensor *result) {
  (void)log2p;
  (void)mu;
  return ntt_run(true, a, p, perm, inv_twiddles, m_inv, result);
}

}  // extern "C"
