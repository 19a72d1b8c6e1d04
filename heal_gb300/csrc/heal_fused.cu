// heal_fused.cu — modmul_axis_sum, the fused compute op that HEAL's Python
// runtime routes to its backend (python_execution/lattica_heal_runtime/
// device_interface.py:67-68; HEAL names the op and leaves its definition to
// the backend).  Defined here as the composition of HEAL's own ops
//
//   result = axis_modsum(modmul(a', b, p), axis)
//
// with a and b broadcast like modmul (example_impl/modop_impl.cpp:44-101) to
// a common shape S, and a' = a or, with `perms`, a gathered like permute
// with elementwise_axis = axis (example_impl/permute_impl.cpp:8-65):
// a'[c] = a[c with c[perm_axis] <- perms[c[axis], c[perm_axis]]].  A perms
// tensor with one more axis, [S[axis], S[pa], S[pa+1]], gathers over the two
// axes pa, pa+1 taken as one flattened axis (a linear across them): the same
// as permute on a with those two axes reshaped into one.
// The product is never written: one thread per result element runs the
// reduction, so a rotate-multiply-accumulate over d rotations reads the
// rotated operand (resident in L2) and b once and writes only the result.
//
// Arithmetic.  With every term canonical (0 <= a', b < q) the running sum of
// residues equals (sum of products) mod q, so the products are accumulated
// exactly in 128 bits (64-bit words; high word kept below q by subtracting
// q * 2^64) or 64 bits (32-bit words; kept below q * 2^32) and reduced once
// (Moller-Granlund).  An element with any other term is recomputed term by
// term with the reference's semantics: modmul's C '%' in the double-width
// type, then axis_modsum's running (sum + v) % q.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "heal_internal.h"
#include "heal_tail.cuh"

namespace heal {

struct FusedArgs {
  View r;                 // result view
  View ao, bo;            // a and b strides in result coordinates
  int64_t a_ax, b_ax;     // strides along the reduced axis
  int64_t len;            // reduced length
  int pa, pa2;            // gathered axes in result coordinates (-1: none)
  int last;               // last axis in result coordinates
  int64_t a_pa;           // a's stride along the (innermost) gathered axis
  int64_t ps0, ps1;       // perms strides: reduced axis, flattened gathered index
  int gather32;           // every gathered offset index * a_pa (and * b_pa) fits in 31 bits
  int prow;               // POST: result axis whose coordinate selects the perms row
  int64_t b_pa;           // POST: b's stride along the gathered axis
  const void *a, *b, *perms;
  int perms_dtype;
  const void *ptab;       // MG64 / MG32 per modulus
  void *out;
  int64_t n;
  FastDims fd;
  Diag *diag;
};

template <typename PT>
__device__ __forceinline__ int64_t fused_perm(const FusedArgs &g, int64_t i, int64_t c) {
  return (int64_t)((const PT *)g.perms)[i * g.ps0 + c * g.ps1];
}

// terms per batch of the reduction loop
#ifndef HEAL_FUSED_U
#define HEAL_FUSED_U 4
#endif
constexpr int kFusedU = HEAL_FUSED_U;

// POST = false: a' gathered with perms row = the reduced index (modmul_axis_sum);
// POST = true: a and b both gathered with one perms row per result element,
// selected by its coordinate along g.prow (permute after the reduction).
template <typename T, typename PT, typename Off, bool POST>
__global__ void __launch_bounds__(256) modmul_axis_sum_kernel(const __grid_constant__ FusedArgs g) {
  typedef typename FusedMG<T>::type M;
  const T *A = (const T *)g.a;
  const T *B = (const T *)g.b;
  const PT *PP = (const PT *)g.perms;
  T *R = (T *)g.out;
  const Off a_ax = (Off)g.a_ax, b_ax = (Off)g.b_ax, ps0 = (Off)g.ps0;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < g.n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t a0 = 0, b0 = 0, r0 = 0, t = 0, cp = 0, cp2 = 0, cr = 0;
    if (g.fd.fast) {
      uint32_t rem = (uint32_t)idx;
#pragma unroll
      for (int k = 0; k < HEAL_MAX_DIMS; ++k) {  // unrolled: per-axis parameters at fixed offsets
        const int i = HEAL_MAX_DIMS - 1 - k;
        if (i >= g.r.ndim) continue;
        const uint32_t qd = fastdiv(rem, g.fd.fd[i]);
        const int64_t c = rem - qd * (uint32_t)g.r.dims[i];
        rem = qd;
        if (i == g.last) t = c;
        if (i == g.pa) cp = c;
        if (i == g.pa2) cp2 = c;
        if (POST && i == g.prow) cr = c;
        a0 += c * g.ao.strides[i];
        b0 += c * g.bo.strides[i];
        r0 += c * g.r.strides[i];
      }
    } else {
      int64_t rem = idx;
      for (int i = g.r.ndim - 1; i >= 0; --i) {
        const int64_t c = rem % g.r.dims[i];
        rem /= g.r.dims[i];
        if (i == g.last) t = c;
        if (i == g.pa) cp = c;
        if (i == g.pa2) cp2 = c;
        if (POST && i == g.prow) cr = c;
        a0 += c * g.ao.strides[i];
        b0 += c * g.bo.strides[i];
        r0 += c * g.r.strides[i];
      }
    }
    if (g.pa2 >= 0) cp = cp * g.r.dims[g.pa2] + cp2;  // flattened index over the gathered pair
    const M mc = ((const M *)g.ptab)[t];
    const int64_t q = sizeof(T) == 4 ? (int64_t)(int32_t)((const MG32 &)mc).q : (int64_t)((const MG64 &)mc).q;
    if (q == 0) {  // modmul and axis_modsum both give 0 for a zero modulus
      atomicAdd(&g.diag->zero_mod, 1ull);
      R[r0] = 0;
      continue;
    }
    const bool perm = g.pa >= 0;
    const uint64_t uq = (uint64_t)q, q32 = uq << 32;
    // Admission of the fast path.  For non-negative terms the composition is
    // (sum of products) mod q whatever their size; with 64-bit words and
    // q < 2^62, terms below 2^bitlen(q) keep the accumulator's high word below
    // q, so OR-ing every term and testing the high bits once suffices.
    // Otherwise (32-bit words, larger q) every term is compared with q.
    const bool orcheck = sizeof(T) == 8 && q > 0 && q < ((int64_t)1 << 62);
    const uint64_t himask = orcheck ? ~((uint64_t(1) << (64 - __clzll(q))) - 1) : 0;
    uint64_t ormask = 0;
    bool canon = q > 0;
    uint64_t hi = 0, lo = 0;  // 64-bit words: hi * 2^64 + lo, hi < q; 32-bit words: lo < q * 2^32
    auto mac = [&](uint64_t x, uint64_t y) {
      if (orcheck) ormask |= x | y;
      else canon = canon && x < uq && y < uq;  // also rejects negative values
      if (sizeof(T) == 4) {
        lo += x * y;                            // < 2 q 2^32 < 2^64
        lo = lo >= q32 ? lo - q32 : lo;
      } else {
        const uint64_t plo = x * y, phi = mulhi64(x, y);
        const uint64_t s = lo + plo;
        hi += phi + (s < lo ? 1 : 0);           // < 2q
        lo = s;
        hi = hi >= uq ? hi - uq : hi;
      }
    };
    // kFusedU terms per batch through running offsets; the permutation
    // indices of the next batch are fetched while this batch's operands load
    Off ai = (Off)a0, bi = (Off)b0, pi = perm ? (Off)(cp * g.ps1) : (Off)0;
    auto gather = [&](Off v) -> Off { return g.gather32 ? (Off)((int32_t)v * (int32_t)g.a_pa) : v * (Off)g.a_pa; };
    if (POST) {  // one source row for every term: fold it into both bases
      const Off v = (Off)PP[(Off)(cr * g.ps0) + pi];
      ai += gather(v);
      bi += g.gather32 ? (Off)((int32_t)v * (int32_t)g.b_pa) : v * (Off)g.b_pa;
    }
    Off pidx[kFusedU];
#pragma unroll
    for (int u = 0; u < kFusedU; ++u) pidx[u] = (!POST && perm && u < g.len) ? (Off)PP[pi + u * ps0] : (Off)0;
    int64_t i0 = 0;
    for (; i0 + kFusedU <= g.len && (orcheck || canon); i0 += kFusedU) {
      uint64_t av[kFusedU], bv[kFusedU];
#pragma unroll
      for (int u = 0; u < kFusedU; ++u) {
        av[u] = (uint64_t)(int64_t)A[ai + u * a_ax + (POST ? (Off)0 : gather(pidx[u]))];
        bv[u] = (uint64_t)(int64_t)B[bi + u * b_ax];
      }
      ai += kFusedU * a_ax;
      bi += kFusedU * b_ax;
      if (!POST && perm) {
        pi += kFusedU * ps0;
#pragma unroll
        for (int u = 0; u < kFusedU; ++u) pidx[u] = i0 + kFusedU + u < g.len ? (Off)PP[pi + u * ps0] : (Off)0;
      }
#pragma unroll
      for (int u = 0; u < kFusedU; ++u) mac(av[u], bv[u]);
    }
#pragma unroll
    for (int u = 0; u < kFusedU; ++u) {  // the last len % kFusedU terms
      if (i0 + u >= g.len) break;
      mac((uint64_t)(int64_t)A[ai + u * a_ax + (POST ? (Off)0 : gather(pidx[u]))], (uint64_t)(int64_t)B[bi + u * b_ax]);
    }
    if (orcheck) canon = (ormask & himask) == 0;
    int64_t res;
    if (canon) {
      res = sizeof(T) == 4 ? (int64_t)mg32_mod(lo, (const MG32 &)mc) : (int64_t)mg64_mod(hi, lo, (const MG64 &)mc);
    } else {
      res = 0;
      const int64_t prow_v = POST ? fused_perm<PT>(g, cr, cp) : 0;
      for (int64_t i = 0; i < g.len; ++i) {
        const int64_t aoffs = a0 + i * g.a_ax + (POST ? prow_v * g.a_pa : perm ? fused_perm<PT>(g, i, cp) * g.a_pa : 0);
        const int64_t boffs = b0 + i * g.b_ax + (POST ? prow_v * g.b_pa : 0);
        res = exact_step<T>(res, (int64_t)A[aoffs], (int64_t)B[boffs], q, mc);
      }
    }
    R[r0] = (T)res;
  }
}

// set while tail_record prepares a call: the lean launch is recorded here
static thread_local TailRecorded *t_tail_rec = nullptr;

// post = false: modmul_axis_sum (perm_axis in the operands' axes).
// post = true:  modmul_axis_sum_permute (perm_axis and ew in result axes).
static int fused(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, const heal_tensor *perms,
                 int64_t perm_axis, const heal_tensor *r, int64_t axis, bool post = false, int64_t ew = 0) {
  clear_error();
  if (post && !perms) return set_error(HEAL_ERR_INVALID_ARGUMENT, "perms pointer must not be null.");
  HEAL_CHECK(check_desc(a, "a", true));
  HEAL_CHECK(check_desc(b, "b", true));
  HEAL_CHECK(check_desc(p, "p", true));
  if (perms) HEAL_CHECK(check_desc(perms, "perms", true));
  HEAL_CHECK(check_desc(r, "result", true));
  HEAL_CHECK(ensure_init());
  const int dt = r->dtype;
  if (a->dtype != dt || b->dtype != dt || p->dtype != dt)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "all tensors must have the element type of result");
  // common shape of a and b, right-aligned as modmul broadcasts
  const int nd = std::max(a->ndim, b->ndim);
  if (nd < 2) return set_error(HEAL_ERR_INVALID_ARGUMENT, "a and b must have at least 2 dimensions");
  int64_t S[HEAL_MAX_DIMS];
  for (int i = 0; i < nd; ++i) {
    const int ia = i - (nd - a->ndim), ib = i - (nd - b->ndim);
    const int64_t da = ia >= 0 ? a->dims[ia] : 1, db = ib >= 0 ? b->dims[ib] : 1;
    if (da != db && da != 1 && db != 1)
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "a and b are not broadcast-compatible.");
    S[i] = da == 1 ? db : da;
  }
  if (axis < 0 || axis >= nd - 1)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "axis must be in range [0, ndim - 2] (can't reduce across last axis)");
  if (p->ndim != 1 || p->dims[0] != S[nd - 1])
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "p must be a 1D tensor of shape [k], k the last dimension");
  if (r->ndim != nd - 1)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "Result must have the shape of a and b with the reduced axis removed.");
  for (int i = 0, j = 0; i < nd; ++i) {
    if (i == axis) continue;
    if (r->dims[j++] != S[i])
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "Result must have the shape of a and b with the reduced axis removed.");
  }
  // gathered axes: one (perms [l, m], as permute) or a pair taken as one
  // flattened axis (perms [l, m1, m2], linear across its last two axes)
  const int gp = perms ? (post ? 1 : perms->ndim - 1) : 0;
  int64_t mflat = 0;
  int64_t paS = perm_axis;  // the gathered axis in the operands' (S) coordinates
  if (post) {
    // permute on the reduced result (permute_impl.cpp:19-35)
    const int rd = nd - 1;
    if (ew < 0 || ew >= rd || perm_axis < 0 || perm_axis >= rd)
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "Axis out of bounds.");
    if (ew == perm_axis) return set_error(HEAL_ERR_INVALID_ARGUMENT, "elementwise_axis and perm_axis must be different.");
    if (perms->ndim != 2 || perms->dims[0] != r->dims[ew] || perms->dims[1] != r->dims[perm_axis])
      return set_error(HEAL_ERR_INVALID_ARGUMENT,
                       "Perms must have shape [l, m] where l and m match a.shape at elementwise and perm axes.");
    paS = perm_axis < axis ? perm_axis : perm_axis + 1;
    mflat = S[paS];
  } else if (perms) {
    if (gp < 1 || gp > 2)
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "Perms must have shape [l, m] (or [l, m1, m2] for two axes).");
    if (perm_axis < 0 || perm_axis + gp > nd) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Axis out of bounds.");
    if (axis >= perm_axis && axis < perm_axis + gp)
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "axis and perm_axis must be different.");
    bool shape_ok = perms->dims[0] == S[axis];
    mflat = 1;
    for (int k = 0; k < gp; ++k) {
      shape_ok = shape_ok && perms->dims[1 + k] == S[perm_axis + k];
      mflat *= S[perm_axis + k];
    }
    if (!shape_ok)
      return set_error(HEAL_ERR_INVALID_ARGUMENT,
                       "Perms must have shape [l, m] where l and m match the shape at axis and perm_axis.");
    if (gp == 2 && perms->dims[2] > 1 && perms->strides[1] != perms->strides[2] * perms->dims[2])
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "Perms must be linear across its last two axes.");
  }
  const int64_t n = numel(*r);
  if (n == 0) return HEAL_OK;
  heal_tensor PV;  // perms as [l, m1 * m2]
  if (post) {
    PV = *perms;
  } else if (perms) {
    PV = *perms;
    PV.ndim = 2;
    PV.dims[1] = mflat;
    PV.strides[1] = (gp == 2 && perms->dims[2] == 1) ? perms->strides[1] : perms->strides[gp];
  }
  if (perms && (post || S[axis] > 0)) {
    bool valid = false;
    HEAL_CHECK(perms_valid(PV, mflat, &valid));
    if (!valid) return set_error(HEAL_ERR_OUT_OF_RANGE, "Permutation index out of bounds.");
  }
  heal_tensor A = *a, B = *b, P = *p, PR = perms ? PV : heal_tensor();
  void *owned[4] = {nullptr, nullptr, nullptr, nullptr};
  auto detach = [&](heal_tensor &t, int slot) -> int {
    return overlaps(t, *r) ? materialize(t, &t, &owned[slot]) : HEAL_OK;
  };
  int rc = detach(A, 0);
  if (!rc) rc = detach(B, 1);
  if (!rc) rc = detach(P, 2);
  if (!rc && perms) rc = detach(PR, 3);
  ModTable mt;
  if (!rc) rc = mod_table(P, &mt);
  FusedArgs g;
  memset(&g, 0, sizeof g);
  if (!rc) {
    // strides of a and b in S coordinates (0 on broadcast axes)
    int64_t as[HEAL_MAX_DIMS], bs[HEAL_MAX_DIMS];
    for (int i = 0; i < nd; ++i) {
      const int ia = i - (nd - A.ndim), ib = i - (nd - B.ndim);
      as[i] = (ia >= 0 && A.dims[ia] != 1) ? A.strides[ia] : 0;
      bs[i] = (ib >= 0 && B.dims[ib] != 1) ? B.strides[ib] : 0;
    }
    if (!post && gp == 2 && S[perm_axis + 1] > 1 && as[perm_axis] != as[perm_axis + 1] * S[perm_axis + 1]) {
      rc = set_error(HEAL_ERR_INVALID_ARGUMENT, "a must be linear across the two gathered axes.");
    } else {
      g.r = make_view(*r);
      g.ao = g.r;
      g.bo = g.r;
      for (int i = 0, j = 0; i < nd; ++i) {
        if (i == axis) continue;
        const bool gathered = perms && i >= paS && i < paS + gp;
        g.ao.strides[j] = gathered ? 0 : as[i];
        g.bo.strides[j] = (post && gathered) ? 0 : bs[i];
        ++j;
      }
      g.a_ax = as[axis];
      g.b_ax = bs[axis];
      g.len = S[axis];
      // stride of the flattened gathered index: the inner axis's (the outer's if the inner has length 1)
      g.a_pa = !perms ? 0 : post ? as[paS] : (gp == 2 && S[perm_axis + 1] == 1) ? as[perm_axis] : as[perm_axis + gp - 1];
      g.b_pa = post ? bs[paS] : 0;
      const int pa = post ? (int)perm_axis : perms ? (int)(perm_axis < axis ? perm_axis : perm_axis - 1) : -1;
      const int last = nd - 2;
      // merge axes other than the ones whose coordinates the kernel reads
      unsigned keep = 1u << last;
      if (pa >= 0) keep |= 1u << pa;
      if (gp == 2) keep |= 1u << (pa + 1);
      if (post) keep |= 1u << ew;
      View *vs[3] = {&g.r, &g.ao, &g.bo};
      int map[HEAL_MAX_DIMS];
      coalesce_views(vs, 3, keep, map);
      g.pa = pa >= 0 ? map[pa] : -1;
      g.pa2 = gp == 2 ? map[pa + 1] : -1;
      g.prow = post ? map[ew] : -1;
      g.last = map[last];
      make_fast_dims(g.r, n, &g.fd);
      g.ps0 = perms ? PR.strides[0] : 0;
      g.ps1 = perms ? PR.strides[1] : 0;
      // indices are validated to lie in [0, mflat)
      g.gather32 = perms && g.a_pa >= 0 && g.b_pa >= 0 && mflat > 0 &&
                   (__int128)std::max(g.a_pa, g.b_pa) * (__int128)(mflat - 1) < ((__int128)1 << 31);
      g.a = A.data;
      g.b = B.data;
      g.perms = perms ? PR.data : nullptr;
      g.perms_dtype = perms ? PR.dtype : HEAL_INT64;
      g.ptab = mt.consts;
      g.out = r->data;
      g.n = n;
      g.diag = diag_device();
    }
  }
  // 32-bit running offsets when every operand spans fewer than 2^31 elements
  auto span_ok = [](const heal_tensor &t) {
    __int128 s = 0;
    for (int i = 0; i < t.ndim; ++i) s += (__int128)(t.dims[i] > 0 ? t.dims[i] - 1 : 0) * (t.strides[i] < 0 ? -t.strides[i] : t.strides[i]);
    return s < ((__int128)1 << 31) - 1;
  };
  const bool off32 = span_ok(A) && span_ok(B) && (!perms || span_ok(PR)) && g.a_ax >= 0 && g.b_ax >= 0 &&
                     g.ps0 >= 0 && g.ps1 >= 0 && g.a_pa >= 0 && g.b_pa >= 0;
  // the lean post-permute kernel where its limits hold
  bool lean = !rc && post && off32 && g.fd.fast && g.r.ndim <= 4 && g.len >= 1 && g.len <= 4 &&
              n < ((int64_t)1 << 32) && g.a_pa >= 0 && g.b_pa >= 0;
  TailArgs ta;
  memset(&ta, 0, sizeof ta);
  if (lean) {
    ta.nd = g.r.ndim;
    for (int k = 0; k < g.r.ndim; ++k) {
      lean = lean && g.r.strides[k] >= 0 && g.ao.strides[k] >= 0 && g.bo.strides[k] >= 0;
      ta.fd[k] = g.fd.fd[k];
      ta.as[k] = (int32_t)g.ao.strides[k];
      ta.bs[k] = (int32_t)g.bo.strides[k];
      ta.rs[k] = (int32_t)g.r.strides[k];
      ta.ew_m[k] = k == g.prow;
      ta.pa_m[k] = k == g.pa;
      ta.t_m[k] = k == g.last;
    }
    ta.a = g.a;
    ta.b = g.b;
    ta.perms = g.perms;
    ta.ptab = g.ptab;
    ta.out = g.out;
    ta.n = (uint32_t)n;
    ta.a_ax = (int32_t)g.a_ax;
    ta.b_ax = (int32_t)g.b_ax;
    ta.a_pa = (int32_t)g.a_pa;
    ta.b_pa = (int32_t)g.b_pa;
    ta.ps0 = (int32_t)g.ps0;
    ta.ps1 = (int32_t)g.ps1;
    ta.diag = g.diag;
  }
  if (t_tail_rec && !rc) {  // recording for heal_keyswitch_batch: the lean launch only, no temporaries
    for (void *o : owned)
      if (o) lean = false;
    if (!lean) {
      for (void *o : owned) scratch_free(o);
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "the keyswitch tail does not take the lean kernel here (a reduced "
                                                  "axis above 4 terms, a result view above 4 axes, offsets past "
                                                  "2^31, or operands overlapping the result)");
    }
    t_tail_rec->args = ta;
    t_tail_rec->is32 = dt == HEAL_INT32;
    t_tail_rec->perms32 = g.perms_dtype == HEAL_INT32;
    t_tail_rec->len = (int)g.len;
    mark_written(r->data);
    return HEAL_OK;
  }
  if (lean) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    const bool p32 = g.perms_dtype == HEAL_INT32;
    auto go = [&](auto t_tag, auto p_tag) {
      typedef decltype(t_tag) TT;
      typedef decltype(p_tag) PTT;
      switch (g.len) {
        case 1: tail_kernel<TT, PTT, 1><<<blocks, 256, 0, stream()>>>(ta); break;
        case 2: tail_kernel<TT, PTT, 2><<<blocks, 256, 0, stream()>>>(ta); break;
        case 3: tail_kernel<TT, PTT, 3><<<blocks, 256, 0, stream()>>>(ta); break;
        default: tail_kernel<TT, PTT, 4><<<blocks, 256, 0, stream()>>>(ta); break;
      }
    };
    if (dt == HEAL_INT32) {
      if (p32) go(int32_t(), int32_t());
      else go(int32_t(), int64_t());
    } else {
      if (p32) go(int64_t(), int32_t());
      else go(int64_t(), int64_t());
    }
    rc = check_launch("modmul_axis_sum_permute");
  } else if (!rc) {
    const int threads = 256;
    const int64_t want = (n + threads - 1) / threads;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)device_sm_count() * 16));
    const bool p32 = g.perms_dtype == HEAL_INT32;
    auto go = [&](auto t_tag, auto p_tag) {
      typedef decltype(t_tag) TT;
      typedef decltype(p_tag) PTT;
      if (post) {
        if (off32) modmul_axis_sum_kernel<TT, PTT, int32_t, true><<<grid, threads, 0, stream()>>>(g);
        else modmul_axis_sum_kernel<TT, PTT, int64_t, true><<<grid, threads, 0, stream()>>>(g);
      } else {
        if (off32) modmul_axis_sum_kernel<TT, PTT, int32_t, false><<<grid, threads, 0, stream()>>>(g);
        else modmul_axis_sum_kernel<TT, PTT, int64_t, false><<<grid, threads, 0, stream()>>>(g);
      }
    };
    if (dt == HEAL_INT32) {
      if (p32) go(int32_t(), int32_t());
      else go(int32_t(), int64_t());
    } else {
      if (p32) go(int64_t(), int32_t());
      else go(int64_t(), int64_t());
    }
    rc = check_launch(post ? "modmul_axis_sum_permute" : "modmul_axis_sum");
  }
  for (void *o : owned) scratch_free(o);
  if (!rc) mark_written(r->data);
  return rc;
}

int tail_record(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, int64_t axis,
                const heal_tensor *perms, int64_t elementwise_axis, int64_t perm_axis, const heal_tensor *result,
                TailRecorded *out) {
  memset(out, 0, sizeof *out);
  t_tail_rec = out;
  const int rc = fused(a, b, p, perms, perm_axis, result, axis, true, elementwise_axis);
  t_tail_rec = nullptr;
  return rc;
}

}  // namespace heal

using namespace heal;

extern "C" {

int heal_modmul_axis_sum(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, const heal_tensor *perms,
                         int64_t perm_axis, const heal_tensor *result, int64_t axis) {
  return fused(a, b, p, perms, perm_axis, result, axis);
}

int heal_modmul_axis_sum_permute(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, int64_t axis,
                                 const heal_tensor *perms, int64_t elementwise_axis, int64_t perm_axis,
                                 const heal_tensor *result) {
  return fused(a, b, p, perms, perm_axis, result, axis, true, elementwise_axis);
}

}  // extern "C"
