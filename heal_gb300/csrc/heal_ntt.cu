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
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "heal_internal.h"
#include "heal_ntt_kernels.cuh"
#include "heal_ntt_record.h"

namespace heal {

constexpr int kSinglePassLogMax = 12;  // m <= 4096 in one pass

int launch_ntt_pass_fwd32(const NttArgs &a, int64_t nblocks, int mode);
int launch_ntt_pass_fwd64(const NttArgs &a, int64_t nblocks, int mode);
int launch_ntt_pass_inv32(const NttArgs &a, int64_t nblocks, int mode);
int launch_ntt_pass_inv64(const NttArgs &a, int64_t nblocks, int mode);
int launch_ntt_pass_fwd32_gdec(const NttArgs &a, int64_t nblocks, int mode);
int launch_ntt_pass_fwd64_gdec(const NttArgs &a, int64_t nblocks, int mode);
int launch_ntt_staged_fwd32(const NttArgs &a, int mode);
int launch_ntt_staged_inv32(const NttArgs &a, int mode);

// Passes the staged kernel (heal_ntt_staged.cuh) takes: 256-point passes of
// int32 tensors (the 32-bit word modes, where it measured faster than the
// register kernel), limbs contiguous in source and destination with every
// 16-byte row chunk aligned, no permutation or the bit reversal, no gather
// after the pass, no g_decomposition on load.  HEAL_NTT_STAGED=0 in the
// environment keeps every pass on the register kernel (for comparisons).
static bool staged_eligible(const NttArgs &a, bool is32, int mode) {
  static const bool on = [] {
    const char *e = getenv("HEAL_NTT_STAGED");
    return !e || atoi(e) != 0;
  }();
  if (!on || a.p != 8 || a.gdec_power || a.store_gather) return false;
  if ((a.load_map || a.store_scatter) && !a.bitrev) return false;
  if (!is32 || !(mode == MODE_N32 || mode == MODE_N32_LAZY)) return false;
  const int64_t esz = 4;
  if (a.ss[3] != 1 || a.ds[3] != 1 || a.k % (16 / esz)) return false;
  auto aligned = [&](const void *ptr, const int64_t *st) {
    return (uintptr_t)ptr % 16 == 0 && (st[0] * esz) % 16 == 0 && (st[1] * esz) % 16 == 0 && (st[2] * esz) % 16 == 0;
  };
  return aligned(a.src, a.ss) && aligned(a.dst, a.ds);
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

int launch_ntt_batch_fwd32(const NttBatchArgs &b, int64_t nblocks, int mode, int p, int threads, size_t smem);
int launch_ntt_batch_fwd64(const NttBatchArgs &b, int64_t nblocks, int mode, int p, int threads, size_t smem);
int launch_ntt_batch_inv32(const NttBatchArgs &b, int64_t nblocks, int mode, int p, int threads, size_t smem);
int launch_ntt_batch_inv64(const NttBatchArgs &b, int64_t nblocks, int mode, int p, int threads, size_t smem);

// ----------------------------------------------------------- host side
// heal_ntt_batch runs the per-transform host path (validation, tables, plans)
// with a collector installed on the calling thread: every pass that the
// register kernel runs is recorded instead of launched, scratch is released
// only after the batch is enqueued, and the recorded passes are then launched
// per kernel class, first passes before second passes.
struct NttDeferred {
  int phase;  // 0: first (or only) pass of its transform, 1: second pass
  NttArgs args;
  int64_t nblocks;
  int mode;
  bool is32, inv;
};
struct NttCollector {
  bool validate_only = false;
  bool record_all = false;  // ntt_record: every pass is recorded, none launched
  int force_first_log = 0;  // ntt_record: the two-pass split to use (0: the plan's)
  std::vector<NttDeferred> passes;
  size_t job_begin = 0;  // first recorded pass of the transform being prepared
  int job_phase = 0;
  std::vector<void *> release;
};
static thread_local NttCollector *t_collect = nullptr;

static int launch_now(const NttArgs &a, int64_t nblocks, bool is32, int mode, bool inv);

// the current transform's recorded passes, launched now (before a pass or a
// kernel of it that cannot be recorded)
static int flush_job(NttCollector *col) {
  for (size_t i = col->job_begin; i < col->passes.size(); ++i) {
    const NttDeferred &d = col->passes[i];
    HEAL_CHECK(launch_now(d.args, d.nblocks, d.is32, d.mode, d.inv));
  }
  col->passes.resize(col->job_begin);
  return HEAL_OK;
}

static void ntt_release(void *ptr) {
  if (!ptr) return;
  if (t_collect) t_collect->release.push_back(ptr);
  else scratch_free(ptr);
}

static bool batchable(const NttArgs &a, int mode, bool inv) {
  return a.gdec_power == 0 && a.p >= 3 && a.p <= kSinglePassLogMax && (a.p > 3 || lpt_of(mode, inv) <= 3);
}

static int launch_any(const NttArgs &a, int64_t nblocks, bool is32, int mode, bool inv) {
  if (NttCollector *col = t_collect) {
    const int phase = col->job_phase++;
    if (col->record_all) {
      col->passes.push_back(NttDeferred{phase, a, nblocks, mode, is32, inv});
      return HEAL_OK;
    }
    if (batchable(a, mode, inv)) {
      col->passes.push_back(NttDeferred{phase, a, nblocks, mode, is32, inv});
      return HEAL_OK;
    }
    HEAL_CHECK(flush_job(col));
  }
  return launch_now(a, nblocks, is32, mode, inv);
}

static int launch_now(const NttArgs &a, int64_t nblocks, bool is32, int mode, bool inv) {
  if (staged_eligible(a, is32, mode)) return inv ? launch_ntt_staged_inv32(a, mode) : launch_ntt_staged_fwd32(a, mode);
  if (inv) return is32 ? launch_ntt_pass_inv32(a, nblocks, mode) : launch_ntt_pass_inv64(a, nblocks, mode);
  if (a.gdec_power) return is32 ? launch_ntt_pass_fwd32_gdec(a, nblocks, mode) : launch_ntt_pass_fwd64_gdec(a, nblocks, mode);
  return is32 ? launch_ntt_pass_fwd32(a, nblocks, mode) : launch_ntt_pass_fwd64(a, nblocks, mode);
}

static void set_strides(int64_t *dst, const heal_tensor &t) {
  for (int i = 0; i < 4; ++i) dst[i] = t.strides[i];
}

static int ilog2(int64_t x) {
  int r = 0;
  while ((int64_t(1) << r) < x) ++r;
  return r;
}

// --------------------------------------------------------------- plans
// A plan fixes the limbs per tile and where the network splits into two
// passes (first_log = log2 of the first pass's length; 0 = one pass).
struct NttPlan {
  int tile_limbs;
  int first_log;
};
using PlanKey = std::tuple<int, int, int, int64_t>;  // dtype, inverse, log2 m, k
static std::mutex g_plan_mu;
static std::map<PlanKey, NttPlan> g_plans;

static int default_tile_limbs() {
  // 4 limbs per tile measured best for int32 and int64 alike (more, smaller
  // CTAs; fewer threads per barrier).  Neighbouring CTAs take neighbouring
  // limb groups, so a DRAM sector shared by two tiles is read once into L2.
  static const int v = [] {
    const char *e = getenv("HEAL_NTT_TILE_LIMBS");
    int x = e ? atoi(e) : 4;
    return (x == 1 || x == 2 || x == 4 || x == 8 || x == 16) ? x : 4;
  }();
  return v;
}

static NttPlan default_plan(int logm) {
  return NttPlan{default_tile_limbs(), logm <= kSinglePassLogMax ? 0 : logm / 2};
}

static NttPlan plan_for(int dt, bool inv, int logm, int64_t k) {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  auto it = g_plans.find(PlanKey{dt, inv ? 1 : 0, logm, k});
  return it != g_plans.end() ? it->second : default_plan(logm);
}

static bool plan_valid(const NttPlan &pl, int logm) {
  const int c = pl.tile_limbs;
  if (c < 1 || c > 16 || (c & (c - 1))) return false;
  if (pl.first_log == 0) return logm <= kSinglePassLogMax;
  const int second = logm - pl.first_log;
  return pl.first_log >= 1 && pl.first_log <= kSinglePassLogMax && second >= 1 && second <= kSinglePassLogMax;
}

// g_decomposition fused into the forward transform's first load
// (heal_g_decomposition_ntt): the transform runs on the digit tensor
// [l, m, r, k * power] that g_decomposition(a, power, bits) reshaped would be.
struct GdecSpec {
  int64_t power, bits;
};

static int ntt_run(bool inv, const heal_tensor *a_in, const heal_tensor *p, const heal_tensor *perm,
                   const heal_tensor *tw, const heal_tensor *minv, const heal_tensor *res,
                   const GdecSpec *gd = nullptr) {
  clear_error();
  HEAL_CHECK(check_desc(a_in, "a", true));
  heal_tensor Av;  // the transform's input shape (the digit tensor's, with g_decomposition)
  const heal_tensor *a = a_in;
  if (gd) {
    HEAL_CHECK(check_desc(res, "result", true));
    if (gd->bits < 0 || gd->bits >= 64) return set_error(HEAL_ERR_INVALID_ARGUMENT, "base_bits must be below 64");
    if (gd->power < 1 || gd->power > (1 << 20))
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "power must be in 1 .. 2^20");
    if (a_in->ndim != 4) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Input tensor 'a' must have shape [l, m, r, k].");
    bool ok = res->ndim == 4 && res->dims[3] == a_in->dims[3] * gd->power;
    for (int i = 0; ok && i < 3; ++i) ok = res->dims[i] == a_in->dims[i];
    if (!ok) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Output must have shape [l, m, r, k * power].");
    // the kernels split a digit limb into source limb and digit in 32 bits
    if (res->dims[3] >= ((int64_t)1 << 31)) return set_error(HEAL_ERR_INVALID_ARGUMENT, "k * power must be below 2^31");
    Av = *a_in;
    Av.dims[3] = a_in->dims[3] * gd->power;
    a = &Av;
  }
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
  // arithmetic mode from the largest modulus (heal_ntt_kernels.cuh)
  const int mode = mi.max_q < (int64_t(1) << 30)   ? MODE_N32_LAZY
                   : mi.max_q < (int64_t(1) << 31) ? MODE_N32
                                                   : MODE_W64_LAZY;
  const bool wide = mode == MODE_W64_LAZY;
  // 64-bit growing ranges where the headroom allows (heal_ntt_kernels.cuh):
  // forward values stay below (1 + 4 log2 m) q <= 97q < 2^63; an inverse pass
  // of P stages ends below 2^(P+1) q < 2^63
  auto mode_of = [&](int pbits) {
    if (!wide) return mode;
    const int lim = inv ? 62 - pbits : 56;
    return mi.max_q < (int64_t(1) << lim) ? (int)MODE_W64_GROW : mode;
  };
  PermInfo pi;
  HEAL_CHECK(perm_info(*perm, &pi));
  if (pi.bad) return set_error(HEAL_ERR_OUT_OF_RANGE, "Index out of bounds.");
  TwiddleTable tt, mt;
  HEAL_CHECK(twiddle_table(*tw, *p, wide, &tt));
  if (inv) HEAL_CHECK(minv_table(*minv, *p, k, wide, &mt));
  if (t_collect && t_collect->validate_only) return HEAL_OK;

  heal_tensor A = *a_in;  // the source as stored (with g_decomposition: the undecomposed tensor)
  void *owned_a = nullptr;
  if (overlaps(A, *res) && (gd || !identical_view(A, *res))) HEAL_CHECK(materialize(A, &A, &owned_a));

  NttArgs base;
  memset(&base, 0, sizeof base);
  base.l = l;
  base.m = m;
  base.r = r;
  base.k = k;
  base.tw_pairs = tt.pairs;
  base.tw_rowmap = tt.rowmap;
  base.tw_neg = tt.neg_flag;
  base.tw_raw = tw->data;
  base.tw_s0 = tw->strides[0];
  base.tw_s1 = tw->strides[1];
  base.q = mi.q;
  base.qone = mi.qone;
  base.qone32 = mi.min_q > ((int64_t)1 << 32);  // then floor(2^64 / q) < 2^32 for every modulus
  base.bitrev = pi.bitrev_log;  // every table this call indexes is the bit reversal (its own inverse)
  base.diag = diag_device();
  if (inv) {
    base.minv_pairs = mt.pairs;
    base.minv_neg = mt.neg_flag;
    base.minv_raw = minv->data;
    base.minv_s0 = minv->strides[0];
  }
  // m = 1 has no butterflies (the forward NTT is a plain copy, unreduced);
  // moduli >= 2^62 do not fit the 64-bit lazy ranges
  base.literal = reference_compat();
  base.force_exact = m == 1 || mi.max_q >= (int64_t(1) << 62) || base.literal;
  const bool is32 = dt == HEAL_INT32;
  NttPlan plan = plan_for(dt, inv, logm, k);
  if (t_collect && t_collect->force_first_log) {
    const int f = t_collect->force_first_log;
    if (f < 1 || f > kSinglePassLogMax || logm - f < 1 || logm - f > kSinglePassLogMax)
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT: no two-pass split of this length at the requested point");
    plan.first_log = f;
  }
  int C = plan.tile_limbs;
  while (C > 1 && C / 2 >= k) C /= 2;
  int rc = HEAL_OK;
  void *tmp = nullptr, *tmp2 = nullptr;

  auto cfg = [&](NttArgs &x, int pbits, int kind) -> int64_t {
    // at most 512 threads per CTA: P * C / (points per thread) <= 512
    int c = C;
    while (c > 1 && ((int64_t)1 << pbits) * c > ((int64_t)512 << lpt_of(mode, inv))) c /= 2;
    x.p = pbits;
    x.C = c;
    x.logC = ilog2(c);
    x.kind = kind;
    x.nsets = m >> pbits;
    x.ngroups_t = (k + c - 1) / c;
    x.fast_bid = x.ngroups_t < (int64_t)UINT32_MAX && l * r < (int64_t)UINT32_MAX && r < (int64_t)UINT32_MAX;
    if (x.fast_bid) {
      x.fd_groups = fastdiv_make((uint32_t)x.ngroups_t);
      x.fd_nij = fastdiv_make((uint32_t)(l * r));
      x.fd_r = fastdiv_make((uint32_t)r);
    }
    return x.nsets * l * r * x.ngroups_t;
  };

  if (plan.first_log == 0) {
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
    if (gd) {
      x.gdec_power = (int)gd->power;
      x.gdec_bits = (int)gd->bits;
    }
    rc = launch_any(x, nb, is32, mode_of(logm), inv);
  } else {
    // two passes through a dense [l, m, r, k] scratch tensor
    const int p1 = plan.first_log, p2 = logm - p1;
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
      // growing ranges carry across the two passes when both run them and the
      // second runs the register kernel (at least 3 stages)
      const int m1 = mode_of(p1), m2 = mode_of(p2);
      x.lazy_out = m1 == MODE_W64_GROW && m2 == MODE_W64_GROW && p2 >= 3;
      if (gd) {
        x.gdec_power = (int)gd->power;
        x.gdec_bits = (int)gd->bits;
      }
      rc = launch_any(x, nb, is32, m1, false);
      if (!rc) {
        NttArgs y = base;  // pass 2: remaining stages on contiguous blocks
        nb = cfg(y, p2, KIND_BLOCK);
        y.src = T1.data;
        set_strides(y.ss, T1);
        y.unreduced_in = x.lazy_out;
        if (pi.bijective) {
          y.dst = res->data;
          set_strides(y.ds, *res);
          y.store_scatter = pi.inv32;
          rc = launch_any(y, nb, is32, m2, false);
        } else if (t_collect && t_collect->record_all) {
          rc = set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT: a permutation that is not a bijection cannot be recorded");
        } else {
          heal_tensor T2 = T1;
          rc = scratch_alloc((size_t)s * elem_size(dt), &tmp2);
          T2.data = tmp2;
          y.dst = T2.data;
          set_strides(y.ds, T2);
          if (!rc) rc = launch_any(y, nb, is32, m2, false);
          if (!rc && t_collect) rc = flush_job(t_collect);  // the gather reads the second pass's output
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
      rc = launch_any(x, nb, is32, mode_of(p1), true);
      if (!rc) {
        NttArgs y = base;  // pass 2: remaining stages on strided sets, then m_inv
        nb = cfg(y, p2, KIND_STRIDED);
        y.src = T1.data;
        set_strides(y.ss, T1);
        y.dst = res->data;
        set_strides(y.ds, *res);
        y.scale = 1;
        rc = launch_any(y, nb, is32, mode_of(p2), true);
      }
    }
  }
  ntt_release(tmp);
  ntt_release(tmp2);
  ntt_release(owned_a);
  if (!rc) mark_written(res->data);
  return rc;
}


int ntt_record(bool inv, const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm, const heal_tensor *tw,
               const heal_tensor *minv, const heal_tensor *res, int64_t gdec_power, int64_t gdec_bits, int first_log,
               std::vector<NttRecorded> *out, std::vector<void *> *release) {
  if (t_collect) return set_error(HEAL_ERR_RUNTIME, "NTT: already recording on this thread");
  NttCollector col;
  col.record_all = true;
  col.force_first_log = first_log;
  t_collect = &col;
  const GdecSpec gd{gdec_power, gdec_bits};
  const int rc = ntt_run(inv, a, p, perm, tw, minv, res, gdec_power ? &gd : nullptr);
  t_collect = nullptr;
  for (const NttDeferred &d : col.passes) out->push_back(NttRecorded{d.args, d.nblocks, d.mode, d.inv, d.is32});
  release->insert(release->end(), col.release.begin(), col.release.end());
  return rc;
}

// the recorded passes of a batch, launched per class (element type, mode,
// direction, pass length, tile width), kNttBatch passes per launch
static int run_collected(NttCollector &col) {
  std::unique_ptr<NttBatchArgs> b(new NttBatchArgs);
  for (int phase = 0; phase < 2; ++phase) {
    std::map<std::tuple<int, int, int, int, int>, std::vector<size_t>> classes;
    for (size_t i = 0; i < col.passes.size(); ++i) {
      const NttDeferred &d = col.passes[i];
      if (d.phase == phase) classes[{d.is32 ? 1 : 0, d.mode, d.inv ? 1 : 0, d.args.p, d.args.C}].push_back(i);
    }
    for (auto &kv : classes) {
      const std::vector<size_t> &idx = kv.second;
      const NttDeferred &d0 = col.passes[idx[0]];
      const int p = d0.args.p, C = d0.args.C;
      const int threads = ((1 << p) >> lpt_of(d0.mode, d0.inv)) * C;
      const size_t smem = (size_t)(1 << p) * C * sizeof(int64_t);
      for (size_t at = 0; at < idx.size();) {
        b->n = 0;
        b->first[0] = 0;
        int64_t total = 0;
        while (at < idx.size() && b->n < kNttBatch && total + col.passes[idx[at]].nblocks < 0x7FFFFFFF) {
          const NttDeferred &d = col.passes[idx[at++]];
          b->pass[b->n] = d.args;
          total += d.nblocks;
          b->first[++b->n] = (uint32_t)total;
        }
        if (b->n == 0) return set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT batch: a transform has more than 2^31 - 1 tiles");
        int rc;
        if (d0.inv) rc = d0.is32 ? launch_ntt_batch_inv32(*b, total, d0.mode, p, threads, smem)
                                 : launch_ntt_batch_inv64(*b, total, d0.mode, p, threads, smem);
        else rc = d0.is32 ? launch_ntt_batch_fwd32(*b, total, d0.mode, p, threads, smem)
                          : launch_ntt_batch_fwd64(*b, total, d0.mode, p, threads, smem);
        HEAL_CHECK(rc);
      }
    }
  }
  return HEAL_OK;
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

int heal_g_decomposition_ntt(const heal_tensor *a, int64_t power, int64_t base_bits, const heal_tensor *p,
                             const heal_tensor *perm, const heal_tensor *twiddles, const heal_tensor *result) {
  const GdecSpec gd{power, base_bits};
  return ntt_run(false, a, p, perm, twiddles, nullptr, result, &gd);
}

int heal_intt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm, const heal_tensor *inv_twiddles,
              const heal_tensor *m_inv, const heal_tensor *log2p, const heal_tensor *mu, const heal_tensor *result) {
  (void)log2p;
  (void)mu;
  return ntt_run(true, a, p, perm, inv_twiddles, m_inv, result);
}


int heal_ntt_batch(int inverse, const heal_ntt_job *jobs, int64_t count) {
  clear_error();
  if (count < 0 || (count > 0 && !jobs)) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_ntt_batch: no jobs");
  if (t_collect) return set_error(HEAL_ERR_RUNTIME, "heal_ntt_batch: already running on this thread");
  HEAL_CHECK(ensure_init());
  const bool inv = inverse != 0;
  // no transform may write what another reads or writes
  for (int64_t i = 0; i < count; ++i) {
    HEAL_CHECK(check_desc(&jobs[i].a, "a", true));
    HEAL_CHECK(check_desc(&jobs[i].result, "result", true));
  }
  for (int64_t i = 0; i < count; ++i)
    for (int64_t j = 0; j < count; ++j)
      if (i != j && (overlaps(jobs[i].result, jobs[j].a) || overlaps(jobs[i].result, jobs[j].result)))
        return set_error(HEAL_ERR_INVALID_ARGUMENT,
                         "heal_ntt_batch: job " + std::to_string(i) + " writes memory job " + std::to_string(j) +
                             " uses");
  NttCollector col;
  t_collect = &col;
  struct Reset {
    ~Reset() { t_collect = nullptr; }
  } reset;
  auto one = [&](int64_t i) {
    const heal_ntt_job &j = jobs[i];
    return ntt_run(inv, &j.a, &j.p, &j.perm, &j.twiddles, inv ? &j.m_inv : nullptr, &j.result);
  };
  col.validate_only = true;  // every argument error before anything is enqueued
  for (int64_t i = 0; i < count; ++i) {
    const int rc = one(i);
    if (rc) return set_error(rc, "heal_ntt_batch: job " + std::to_string(i) + ": " + heal_last_error());
  }
  col.validate_only = false;
  // The recorded passes are launched every kBatchFlush jobs: a job touches at
  // most 5 cached tables, so the tables of the recorded passes stay among the
  // cache's most recent entries and none is evicted (its buffer freed) before
  // the passes that read it are enqueued.
  constexpr int64_t kBatchFlush = 512;
  int rc = HEAL_OK;
  for (int64_t i = 0; i < count && !rc; ++i) {
    col.job_begin = col.passes.size();
    col.job_phase = 0;
    rc = one(i);
    if (!rc && (i + 1) % kBatchFlush == 0) {
      rc = run_collected(col);
      col.passes.clear();
    }
  }
  if (!rc) rc = run_collected(col);
  t_collect = nullptr;
  for (void *ptr : col.release) scratch_free(ptr);  // stream-ordered: after the launches above
  return rc;
}

static int plan_shape(int dtype, int inverse, int64_t m, int64_t k, int *logm) {
  if (dtype != HEAL_INT32 && dtype != HEAL_INT64)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT plan: dtype must be HEAL_INT32 or HEAL_INT64");
  if (inverse != 0 && inverse != 1) return set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT plan: inverse must be 0 or 1");
  if (m < 1 || (m & (m - 1)) || m > (int64_t(1) << (2 * kSinglePassLogMax)))
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT plan: m must be a power of two up to 2^24");
  if (k < 1) return set_error(HEAL_ERR_INVALID_ARGUMENT, "NTT plan: k must be positive");
  *logm = ilog2(m);
  return HEAL_OK;
}

int heal_ntt_set_plan(int dtype, int inverse, int64_t m, int64_t k, int tile_limbs, int first_pass_log2) {
  clear_error();
  int logm;
  HEAL_CHECK(plan_shape(dtype, inverse, m, k, &logm));
  const NttPlan pl{tile_limbs, first_pass_log2};
  if (!plan_valid(pl, logm))
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_ntt_set_plan: tile_limbs must be 1, 2, 4, 8 or 16 and "
                                                "both passes 1..12 stages long (0 = one pass, m <= 4096)");
  std::lock_guard<std::mutex> lk(g_plan_mu);
  g_plans[PlanKey{dtype, inverse, logm, k}] = pl;
  return HEAL_OK;
}

int heal_ntt_get_plan(int dtype, int inverse, int64_t m, int64_t k, int *tile_limbs, int *first_pass_log2) {
  clear_error();
  int logm;
  HEAL_CHECK(plan_shape(dtype, inverse, m, k, &logm));
  const NttPlan pl = plan_for(dtype, inverse != 0, logm, k);
  if (tile_limbs) *tile_limbs = pl.tile_limbs;
  if (first_pass_log2) *first_pass_log2 = pl.first_log;
  return HEAL_OK;
}

int heal_ntt_clear_plans(void) {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  g_plans.clear();
  return HEAL_OK;
}

int heal_ntt_autotune(int inverse, const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm,
                      const heal_tensor *twiddles, const heal_tensor *m_inv, const heal_tensor *result, int reps,
                      int *tile_limbs, int *first_pass_log2) {
  clear_error();
  HEAL_CHECK(ensure_init());
  if (capturing()) return set_error(HEAL_ERR_RUNTIME, "heal_ntt_autotune: not allowed while a graph is being captured");
  if (reps < 1) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_ntt_autotune: reps must be positive");
  const bool inv = inverse != 0;
  auto run = [&]() { return ntt_run(inv, a, p, perm, twiddles, inv ? m_inv : nullptr, result); };
  HEAL_CHECK(run());  // validates the operands and caches their tables
  const int dt = a->dtype;
  const int64_t m = a->dims[1], k = a->dims[3];
  if (m == 0 || a->dims[0] * a->dims[2] * k == 0) return HEAL_OK;
  const int logm = ilog2(m);
  const PlanKey key{dt, inv ? 1 : 0, logm, k};
  NttPlan before;
  bool had;
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plans.find(key);
    had = it != g_plans.end();
    if (had) before = it->second;
  }
  // candidates: every distinct tile width, and the splits near the middle
  std::vector<NttPlan> cands;
  std::vector<int> splits;
  if (logm <= kSinglePassLogMax) splits.push_back(0);
  if (logm >= 8)
    for (int s = logm / 2 - 1; s <= logm / 2 + 1; ++s)
      if (s >= 4 && logm - s >= 4 && s <= kSinglePassLogMax && logm - s <= kSinglePassLogMax) splits.push_back(s);
  if (splits.empty()) splits.push_back(default_plan(logm).first_log);
  for (int c = 1; c <= 16; c *= 2) {
    if (c / 2 >= k) break;  // wider tiles shrink to this one
    for (int s : splits) cands.push_back(NttPlan{c, s});
  }
  cudaEvent_t e0, e1;
  HEAL_TRY_CUDA(cudaEventCreate(&e0));
  HEAL_TRY_CUDA(cudaEventCreate(&e1));
  int rc = HEAL_OK;
  float best_ms = 0.f, default_ms = 0.f;
  const NttPlan dflt = default_plan(logm);
  NttPlan best = dflt;
  for (const NttPlan &pl : cands) {
    {
      std::lock_guard<std::mutex> lk(g_plan_mu);
      g_plans[key] = pl;
    }
    rc = run();  // warm-up of this plan
    if (rc) break;
    cudaEventRecord(e0, stream());
    for (int i = 0; i < reps && !rc; ++i) rc = run();
    cudaEventRecord(e1, stream());
    if (rc) break;
    cudaError_t ce = cudaEventSynchronize(e1);
    if (ce != cudaSuccess) {
      rc = cuda_fail(ce, "heal_ntt_autotune");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (pl.tile_limbs == dflt.tile_limbs && pl.first_log == dflt.first_log) default_ms = ms;
    if (best_ms == 0.f || ms < best_ms) {
      best_ms = ms;
      best = pl;
    }
  }
  // plans within a few percent of each other swap places between runs: the
  // default plan stays unless another is at least kTuneMargin faster
  constexpr float kTuneMargin = 0.03f;
  if (default_ms > 0.f && best_ms > default_ms * (1.f - kTuneMargin)) best = dflt;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    if (rc) {
      if (had) g_plans[key] = before;
      else g_plans.erase(key);
    } else {
      g_plans[key] = best;
    }
  }
  if (rc) return rc;
  if (tile_limbs) *tile_limbs = best.tile_limbs;
  if (first_pass_log2) *first_pass_log2 = best.first_log;
  return HEAL_OK;
}

}  // extern "C"
