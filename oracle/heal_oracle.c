/*
 * heal_oracle.c — CPU restatement of HEAL's sample implementation
 * (Lattica-ai/heal, example_impl/), used ONLY as the checker of the GPU
 * backend: by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline.  It is test infrastructure and never part of the product path.
 *
 * Each function follows the cited reference lines step by step (same loop
 * order, same per-step `%` in the double-width type T_DP of
 * example_impl/typing.h:4-20), reading elements through (dims, strides)
 * exactly as DeviceTensor::at / at_with_broadcast do
 * (example_impl/device_memory_impl.cpp:87-124).
 *
 * Two arithmetic modes:
 *   exact = 0  "literal": sums and the INTT scaling are done in the element
 *              type T with two's-complement wraparound, which is what the
 *              reference's int32/int64 expressions compute on x86/Arm
 *              (ntt_impl.cpp:106-107,155-157,165; axis_modsum_impl.cpp:70).
 *   exact = 1  every intermediate in T_DP, so nothing wraps.  This is the
 *              mathematically correct result and the GPU backend's contract.
 * The two agree whenever the reference does not overflow (e.g. q < 2^30 for
 * int32 NTTs, val*m_inv < 2^63 for int64 INTT scaling).
 *
 * Parity pinning: tests/golden/ holds outputs of the reference itself
 * (built from its own sources by oracle/build_ref.sh) and the literal tables
 * of its GoogleTest suite; tests/test_oracle.py checks this file against them.
 *
 * Errors are returned as HEAL status codes (1 invalid_argument,
 * 2 out_of_range, 3 runtime_error) with a message from ora_last_error().
 * Where the reference has undefined behaviour (division by zero, indices
 * that at() does not check) this file returns an error instead.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/heal_gb300.h"

typedef __int128 i128;
typedef unsigned __int128 u128;

static __thread char g_err[512];

static int fail(int code, const char *msg) {
  snprintf(g_err, sizeof g_err, "%s", msg);
  return code;
}

const char *ora_last_error(void) { return g_err; }

int ora_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

static int64_t numel(const heal_tensor *t) {
  int64_t n = 1;
  for (int i = 0; i < t->ndim; ++i) n *= t->dims[i];
  return n;
}

static int same_dims(const heal_tensor *a, const heal_tensor *b) {
  if (a->ndim != b->ndim) return 0;
  for (int i = 0; i < a->ndim; ++i)
    if (a->dims[i] != b->dims[i]) return 0;
  return 1;
}

/* element load / store as int64 (int32 sign-extended) */
static inline int64_t ld(const heal_tensor *t, int64_t off) {
  if (t->dtype == HEAL_INT32) return ((const int32_t *)t->data)[off];
  return ((const int64_t *)t->data)[off];
}
static inline void st(const heal_tensor *t, int64_t off, int64_t v) {
  if (t->dtype == HEAL_INT32)
    ((int32_t *)t->data)[off] = (int32_t)v;
  else
    ((int64_t *)t->data)[off] = v;
}

/* wrap an integer to the element type's width (two's complement) */
static inline int64_t wrapT(int is32, i128 v) {
  if (is32) return (int64_t)(int32_t)(uint32_t)(uint64_t)v;
  return (int64_t)(uint64_t)v;
}

/* C's truncating remainder in the double-width type */
static inline i128 crem(i128 a, i128 b) { return a % b; }

/* row-major coordinates of linear index `idx` over dims */
static inline void unravel(int64_t idx, int nd, const int64_t *dims, int64_t *c) {
  for (int i = nd - 1; i >= 0; --i) {
    int64_t d = dims[i];
    c[i] = d ? idx % d : 0;
    idx = d ? idx / d : 0;
  }
}

static inline int64_t offset_of(const heal_tensor *t, const int64_t *c) {
  int64_t off = 0;
  for (int i = 0; i < t->ndim; ++i) off += c[i] * t->strides[i];
  return off;
}

/* at_with_broadcast (device_memory_impl.cpp:116-124): right-aligned, index 0
 * on size-1 axes, then at()'s bounds check (device_memory_impl.cpp:100-103). */
static inline int64_t bcast_offset(const heal_tensor *t, int full_nd, const int64_t *c) {
  int off_ax = full_nd - t->ndim;
  int64_t off = 0;
  for (int i = 0; i < t->ndim; ++i) {
    int64_t ci = t->dims[i] == 1 ? 0 : c[i + off_ax];
    off += ci * t->strides[i];
  }
  return off;
}

/* the bounds at() would enforce for every coordinate of `r` */
static int bcast_in_range(const heal_tensor *t, const heal_tensor *r) {
  if (t->ndim > r->ndim) return fail(1, "operand has more dims than result.");
  if (numel(r) == 0) return 0;
  int off_ax = r->ndim - t->ndim;
  for (int i = 0; i < t->ndim; ++i)
    if (t->dims[i] != 1 && t->dims[i] < r->dims[i + off_ax]) return fail(2, "Index out of bounds.");
  return 0;
}

/* ===================================================================== NTT
 * ntt<T> (ntt_impl.cpp:69-116): validation (:15-43), per column copy
 * (:88-90), iterative Cooley-Tukey stages with twiddle tw[t, stage+u]
 * (:92-110), then the gather out[u] = res[perm[u]] (:46-65). */
static int validate_ntt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm,
                        const heal_tensor *tw, const heal_tensor *res) {
  if (a->ndim != 4) return fail(1, "Input tensor 'a' must have shape [l, m, r, k].");
  if (!same_dims(a, res)) return fail(1, "Output tensor must have the same shape as input tensor.");
  if (p->ndim != 1 || p->dims[0] != a->dims[3]) return fail(1, "Tensor 'p' must have shape [k].");
  if (perm->ndim != 1 || perm->dims[0] != a->dims[1]) return fail(1, "Tensor 'perm' must have shape [m].");
  if (tw->ndim != 2 || tw->dims[0] != a->dims[3] || tw->dims[1] != a->dims[1])
    return fail(1, "Tensor 'twiddles' must have shape [k, m].");
  int64_t m = a->dims[1];
  if (m > 2 && (m & (m - 1))) return fail(2, "Index out of bounds.");
  for (int64_t t = 0; t < a->dims[3]; ++t)
    if (ld(p, t * p->strides[0]) <= 0) return fail(3, "moduli must be positive");
  return 0;
}

int ora_ntt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm, const heal_tensor *tw,
            const heal_tensor *res, int exact) {
  int rc = validate_ntt(a, p, perm, tw, res);
  if (rc) return rc;
  const int64_t l = a->dims[0], m = a->dims[1], r = a->dims[2], k = a->dims[3];
  const int is32 = a->dtype == HEAL_INT32;
  for (int64_t u = 0; u < m; ++u) {
    int64_t pu = ld(perm, u * perm->strides[0]);
    if (pu < 0 || pu >= m) return fail(2, "Index out of bounds.");
  }
  const int64_t ncol = l * r * k;
  int err = 0;
#pragma omp parallel
  {
    i128 *col = (i128 *)malloc(sizeof(i128) * (size_t)(m ? m : 1));
    int64_t *tmp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m ? m : 1));
    if (!col || !tmp) {
#pragma omp atomic write
      err = 1;
    }
#pragma omp for schedule(dynamic, 1)
    for (int64_t c = 0; c < ncol; ++c) {
      if (!col || !tmp) continue;
      int64_t t = c % k, j = (c / k) % r, i = c / (k * r);
      int64_t base_a = i * a->strides[0] + j * a->strides[2] + t * a->strides[3];
      int64_t base_r = i * res->strides[0] + j * res->strides[2] + t * res->strides[3];
      i128 mod = ld(p, t * p->strides[0]);
      for (int64_t u = 0; u < m; ++u) col[u] = ld(a, base_a + u * a->strides[1]);
      int64_t step = m;
      for (int64_t stage = 1; stage < m; stage *= 2) {
        step /= 2;
        for (int64_t u = 0; u < stage; ++u) {
          int64_t j1 = 2 * u * step, j2 = j1 + step;
          i128 s = ld(tw, t * tw->strides[0] + (stage + u) * tw->strides[1]);
          for (int64_t jx = j1; jx < j2; ++jx) {
            i128 uv = col[jx], vv = col[jx + step];
            i128 vmod = crem(vv * s, mod); /* T_DP product, % in T_DP (:104-105) */
            if (exact) {
              col[jx] = crem(uv + vmod, mod);
              col[jx + step] = crem(uv + mod - vmod, mod);
            } else { /* (u_val + v_mod) % mod and (u_val + mod - v_mod) % mod in T (:106-107) */
              col[jx] = crem(wrapT(is32, uv + vmod), mod);
              col[jx + step] = crem(wrapT(is32, uv + mod - vmod), mod);
            }
          }
        }
      }
      for (int64_t u = 0; u < m; ++u) tmp[u] = (int64_t)col[ld(perm, u * perm->strides[0])];
      for (int64_t u = 0; u < m; ++u) st(res, base_r + u * res->strides[1], tmp[u]);
    }
    free(col);
    free(tmp);
  }
  return err ? fail(3, "allocation failed") : 0;
}

/* ==================================================================== INTT
 * intt<T> (ntt_impl.cpp:118-170): scatter res[perm[u]] = a[u] into the
 * result's previous contents (:138-141), Gentleman-Sande stages with
 * inv_twiddles[t, half+group] (:143-161), scaling by m_inv[t] (:163-166).
 * `a` is read in full before the result column is written (the reference
 * scatters in place; the two differ only when result aliases a). */
int ora_intt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm, const heal_tensor *itw,
             const heal_tensor *minv, const heal_tensor *res, int exact) {
  int rc = validate_ntt(a, p, perm, itw, res);
  if (rc) return rc;
  const int64_t l = a->dims[0], m = a->dims[1], r = a->dims[2], k = a->dims[3];
  const int is32 = a->dtype == HEAL_INT32;
  if (k > 0 && l * r > 0 && m > 0) {
    if (!minv || minv->ndim != 1) return fail(1, "Number of indices does not match tensor dimensions.");
    if (minv->dims[0] < k) return fail(2, "Index out of bounds.");
  }
  for (int64_t u = 0; u < m; ++u) {
    int64_t pu = ld(perm, u * perm->strides[0]);
    if (pu < 0 || pu >= m) return fail(2, "Index out of bounds.");
  }
  const int64_t ncol = l * r * k;
  int err = 0;
#pragma omp parallel
  {
    i128 *col = (i128 *)malloc(sizeof(i128) * (size_t)(m ? m : 1));
    if (!col) {
#pragma omp atomic write
      err = 1;
    }
#pragma omp for schedule(dynamic, 1)
    for (int64_t c = 0; c < ncol; ++c) {
      if (!col) continue;
      int64_t t = c % k, j = (c / k) % r, i = c / (k * r);
      int64_t base_a = i * a->strides[0] + j * a->strides[2] + t * a->strides[3];
      int64_t base_r = i * res->strides[0] + j * res->strides[2] + t * res->strides[3];
      i128 mod = ld(p, t * p->strides[0]);
      i128 mi = ld(minv, t * minv->strides[0]);
      for (int64_t u = 0; u < m; ++u) col[u] = ld(res, base_r + u * res->strides[1]);
      for (int64_t u = 0; u < m; ++u) col[ld(perm, u * perm->strides[0])] = ld(a, base_a + u * a->strides[1]);
      int64_t ts = 1, half = m / 2;
      while (half >= 1) {
        for (int64_t tid = 0; tid < m / 2; ++tid) {
          int64_t group = tid / ts;
          int64_t iu = group * ts * 2 + (tid % ts), iv = iu + ts;
          i128 s = ld(itw, t * itw->strides[0] + (half + group) * itw->strides[1]);
          i128 uv = col[iu], vv = col[iv];
          if (exact) {
            col[iu] = crem(uv + vv, mod);
            col[iv] = crem((uv + mod - vv) * s, mod);
          } else {
            col[iu] = crem(wrapT(is32, uv + vv), mod);
            col[iv] = crem((i128)wrapT(is32, uv + mod - vv) * s, mod);
          }
        }
        ts *= 2;
        half /= 2;
      }
      for (int64_t u = 0; u < m; ++u) {
        i128 v = col[u];
        i128 o = exact ? crem(v * mi, mod) : crem(wrapT(is32, v * mi), mod);
        st(res, base_r + u * res->strides[1], (int64_t)o);
      }
    }
    free(col);
  }
  return err ? fail(3, "allocation failed") : 0;
}

/* ================================================================== modop
 * elementwise_modop (modop_impl.cpp:44-80) through the wrappers of
 * DEFINE_MODULAR_ARITHMETIC_WRAPPER (:108-180): checks (:84-101), then for
 * every result coordinate (T)((T_DP)a op (T_DP)b % (T_DP)p).
 * op: 0 = modmul, 1 = modsum, 2 = modneg (extension: (p - a % p) % p).
 * A NULL tensor selects the scalar argument beside it. */
static int check_broadcastable(const heal_tensor *t, const heal_tensor *r, const char *label) {
  static __thread char buf[128];
  if (t->ndim > r->ndim) {
    snprintf(buf, sizeof buf, "%s has more dims than result.", label);
    return fail(1, buf);
  }
  for (int i = 1; i <= t->ndim; ++i) {
    int64_t td = t->dims[t->ndim - i], rd = r->dims[r->ndim - i];
    if (td != 1 && td != rd) {
      snprintf(buf, sizeof buf, "%s not broadcast-compatible with result.", label);
      return fail(1, buf);
    }
  }
  return 0;
}

int ora_modop(int op, const heal_tensor *a, const heal_tensor *b, int64_t b_scalar, const heal_tensor *p,
              int64_t p_scalar, const heal_tensor *res) {
  int rc;
  if (!a) return fail(1, "a pointer must not be null.");
  if ((rc = check_broadcastable(a, res, "a"))) return rc;
  if (b && (rc = check_broadcastable(b, res, "b"))) return rc;
  if (p && p->ndim != 1 && p->dims[p->ndim - 1] != res->dims[res->ndim - 1])
    return fail(1, "Last dimension of p must match last dimension of result.");
  if (p && (rc = bcast_in_range(p, res))) return rc;
  const int is32 = res->dtype == HEAL_INT32;
  const int64_t total = numel(res);
  const int nd = res->ndim;
  int zero_mod = 0;
#pragma omp parallel for schedule(static)
  for (int64_t idx = 0; idx < total; ++idx) {
    int64_t c[HEAL_MAX_DIMS];
    unravel(idx, nd, res->dims, c);
    i128 av = ld(a, bcast_offset(a, nd, c));
    i128 bv = b ? ld(b, bcast_offset(b, nd, c)) : (i128)(is32 ? (int32_t)b_scalar : b_scalar);
    i128 pv = p ? ld(p, bcast_offset(p, nd, c)) : (i128)(is32 ? (int32_t)p_scalar : p_scalar);
    if (pv == 0) {
      zero_mod = 1;
      continue;
    }
    i128 o;
    if (op == 0)
      o = crem(av * bv, pv);
    else if (op == 1)
      o = crem(av + bv, pv);
    else
      o = crem(pv - crem(av, pv), pv);
    st(res, offset_of(res, c), (int64_t)o);
  }
  return zero_mod ? fail(3, "modulus is zero") : 0;
}

/* elementwise_modred (modop_impl.cpp:13-42) via DEFINE_SIMPLE_MOD_WRAPPER
 * (:188-235): identical shapes, (T)(a % b) in T.  A NULL tensor selects the
 * scalar beside it (cast to T as static_cast<T>(scalar), :216,:230). */
int ora_mod(const heal_tensor *a, int64_t a_scalar, const heal_tensor *b, int64_t b_scalar, const heal_tensor *res) {
  if (a && !same_dims(a, res)) return fail(1, "a must have exactly the same shape as result.");
  if (b && !same_dims(b, res)) return fail(1, "b must have exactly the same shape as result.");
  const int is32 = res->dtype == HEAL_INT32;
  const int64_t total = numel(res);
  const int nd = res->ndim;
  int zero_div = 0;
#pragma omp parallel for schedule(static)
  for (int64_t idx = 0; idx < total; ++idx) {
    int64_t c[HEAL_MAX_DIMS];
    unravel(idx, nd, res->dims, c);
    int64_t av = a ? ld(a, offset_of(a, c)) : (is32 ? (int32_t)a_scalar : a_scalar);
    int64_t bv = b ? ld(b, offset_of(b, c)) : (is32 ? (int32_t)b_scalar : b_scalar);
    if (bv == 0) {
      zero_div = 1;
      continue;
    }
    int64_t o = (bv == -1) ? 0 : av % bv; /* INT_MIN % -1 is 0 mathematically */
    st(res, offset_of(res, c), o);
  }
  return zero_div ? fail(3, "division by zero") : 0;
}

/* ============================================================ axis_modsum
 * axis_modsum<T> (axis_modsum_impl.cpp:12-76): checks (:19-33); for every
 * result coordinate, in_coord = result coordinate with `axis` inserted
 * (:55-64), mod = p[in_coord.back()] (:66), sum = (sum + a) % mod
 * sequentially over the axis (:67-71). */
int ora_axis_modsum(const heal_tensor *a, const heal_tensor *p, const heal_tensor *res, int64_t axis, int exact) {
  if (p->ndim != 1) return fail(1, "p must be a 1D tensor of shape [k]");
  const int nd = a->ndim;
  if (axis < 0 || axis >= nd - 1)
    return fail(1, "axis must be in range [0, ndim - 2] (can't reduce across last axis)");
  if (a->dims[nd - 1] != p->dims[0]) return fail(1, "Last dimension of a must match shape of p");
  if (res->ndim != nd - 1) return fail(1, "Result must have the shape of a with the reduced axis removed.");
  for (int i = 0, j = 0; i < nd; ++i) {
    if (i == axis) continue;
    if (res->dims[j] > a->dims[i] && numel(res) > 0) return fail(2, "Index out of bounds.");
    ++j;
  }
  const int is32 = a->dtype == HEAL_INT32;
  const int64_t total = numel(res);
  const int64_t L = a->dims[axis];
  int zero_mod = 0;
#pragma omp parallel for schedule(static)
  for (int64_t idx = 0; idx < total; ++idx) {
    int64_t rc[HEAL_MAX_DIMS], ic[HEAL_MAX_DIMS];
    unravel(idx, res->ndim, res->dims, rc);
    for (int i = 0, j = 0; i < nd; ++i) ic[i] = (i == axis) ? 0 : rc[j++];
    i128 mod = ld(p, ic[nd - 1] * p->strides[0]);
    if (mod == 0) {
      zero_mod = 1;
      continue;
    }
    i128 sum = 0;
    for (int64_t rr = 0; rr < L; ++rr) {
      ic[axis] = rr;
      i128 v = ld(a, offset_of(a, ic));
      sum = exact ? crem(sum + v, mod) : crem(wrapT(is32, sum + v), mod);
    }
    st(res, offset_of(res, rc), (int64_t)sum);
  }
  return zero_mod ? fail(3, "modulus is zero") : 0;
}

/* ======================================================== g_decomposition
 * g_decomposition<T> (g_decomposition_impl.cpp:10-67).  base is size_t, so
 * `value % base` and `value /= base` convert value to uint64 first (usual
 * arithmetic conversions), and the quotient is stored back into T (:54-55).
 * A residual > 0 is counted (the reference prints a warning, :58-65). */
int ora_g_decomposition(const heal_tensor *a, const heal_tensor *res, uint64_t power, uint64_t base_bits,
                        int64_t *warn_count) {
  if (res->ndim != a->ndim + 1 || res->dims[res->ndim - 1] != (int64_t)power)
    return fail(1, "Output must have shape a.shape + [power]");
  for (int i = 0; i < a->ndim; ++i)
    if (a->dims[i] != res->dims[i]) return fail(1, "Output must have shape a.shape + [power]");
  if (base_bits >= 64) return fail(1, "base_bits must be below 64");
  const uint64_t base = 1ULL << base_bits;
  const int is32 = a->dtype == HEAL_INT32;
  const int64_t total = numel(a);
  int64_t warns = 0;
#pragma omp parallel for schedule(static) reduction(+ : warns)
  for (int64_t idx = 0; idx < total; ++idx) {
    int64_t c[HEAL_MAX_DIMS + 1];
    unravel(idx, a->ndim, a->dims, c);
    c[a->ndim] = 0; /* digit coordinate */
    int64_t value = ld(a, offset_of(a, c));
    int64_t obase = offset_of(res, c);
    for (uint64_t d = 0; d < power; ++d) {
      uint64_t uv = (uint64_t)value;
      st(res, obase + (int64_t)d * res->strides[res->ndim - 1], (int64_t)(uv % base));
      uint64_t q = uv / base;
      value = is32 ? (int64_t)(int32_t)(uint32_t)q : (int64_t)q;
    }
    if (value > 0) warns++;
  }
  if (warn_count) *warn_count = warns;
  return 0;
}

/* ================================================================ permute
 * permute<T> (permute_impl.cpp:8-65): checks (:19-35); for every coordinate
 * res[c] = a[c with c[perm_axis] <- perms[c[ew], c[perm_axis]]] (:40-64);
 * an index >= m raises out_of_range (:45-47; negative ones too here). */
int ora_permute(const heal_tensor *a, const heal_tensor *perms, const heal_tensor *res, int64_t ew, int64_t pa) {
  const int nd = a->ndim;
  if (!same_dims(a, res)) return fail(1, "Result shape must match input shape.");
  if (ew < 0 || ew >= nd || pa < 0 || pa >= nd) return fail(1, "Axis out of bounds.");
  if (ew == pa) return fail(1, "elementwise_axis and perm_axis must be different.");
  const int64_t l = a->dims[ew], m = a->dims[pa];
  if (perms->ndim != 2 || perms->dims[0] != l || perms->dims[1] != m)
    return fail(1, "Perms must have shape [l, m] where l and m match a.shape at elementwise and perm axes.");
  if (numel(a) > 0)
    for (int64_t i = 0; i < l; ++i)
      for (int64_t j = 0; j < m; ++j) {
        int64_t v = ld(perms, i * perms->strides[0] + j * perms->strides[1]);
        if (v < 0 || v >= m) return fail(2, "Permutation index out of bounds.");
      }
  const int64_t total = numel(a);
  int64_t *tmp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(total ? total : 1));
  if (!tmp) return fail(3, "allocation failed");
#pragma omp parallel for schedule(static)
  for (int64_t idx = 0; idx < total; ++idx) {
    int64_t c[HEAL_MAX_DIMS];
    unravel(idx, nd, a->dims, c);
    int64_t pidx = ld(perms, c[ew] * perms->strides[0] + c[pa] * perms->strides[1]);
    c[pa] = pidx;
    tmp[idx] = ld(a, offset_of(a, c));
  }
#pragma omp parallel for schedule(static)
  for (int64_t idx = 0; idx < total; ++idx) {
    int64_t c[HEAL_MAX_DIMS];
    unravel(idx, nd, a->dims, c);
    st(res, offset_of(res, c), tmp[idx]);
  }
  free(tmp);
  return 0;
}

/* ========================================================= make_contiguous
 * The gather of contiguous_impl.cpp:31-40: dst[idx] = src.at(coord(idx)). */
int ora_copy_strided(const heal_tensor *src, const heal_tensor *dst) {
  if (!same_dims(src, dst)) return fail(1, "shape mismatch");
  const int64_t total = numel(src);
  const size_t es = src->dtype == HEAL_INT32 ? 4 : 8;
#pragma omp parallel for schedule(static)
  for (int64_t idx = 0; idx < total; ++idx) {
    int64_t c[HEAL_MAX_DIMS];
    unravel(idx, src->ndim, src->dims, c);
    memcpy((char *)dst->data + es * offset_of(dst, c), (const char *)src->data + es * offset_of(src, c), es);
  }
  return 0;
}
