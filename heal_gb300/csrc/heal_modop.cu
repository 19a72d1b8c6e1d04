// heal_modop.cu — elementwise modular arithmetic with broadcasting:
// modmul / modsum (HEAL include/modop.h:47-111), mod (modop.h:115-134) and
// the modneg extension, over int32 and int64 tensors of any strides.
//
// Semantics follow example_impl/modop_impl.cpp: for every coordinate of
// `result`, res = (T)((T_DP)a op (T_DP)b % (T_DP)p) with C's truncating `%`,
// operands read with at_with_broadcast (right-aligned, index 0 on size-1
// axes).  Non-negative operands with a positive modulus take the fast paths
// of heal_arith.h; anything else takes the exact double-width `%`.
//
// Three kernels: a dense kernel (result, a and b row-major with the same
// shape, p a scalar or a [k] vector on the last axis — every call of the
// keyswitch chain) that streams 16-byte vectors; a vector kernel for a
// result contiguous on its innermost axis with operands contiguous or
// broadcast there (16-byte units, one coordinate decomposition each); and a
// general strided kernel.  All are HBM-bound: per element they move
// sizeof(T) x (reads of a and b + one write), less for broadcast operands.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <type_traits>
#include <cstring>
#include <mutex>

#include "heal_internal.h"

namespace heal {

enum Op { OP_MUL = 0, OP_SUM = 1, OP_NEG = 2, OP_MOD = 3 };

struct ModopArgs {
  View a, b, p, r;  // views in result coordinates (stride 0 on broadcast axes)
  View pd;          // result coordinate -> dense index into the modulus table
  const void *ap, *bp, *pp;
  void *rp;
  int64_t bs, ps;      // scalars when bp / pp are null
  const void *ptab;    // MG32 / MG64 per modulus element, or null
  MG64 pc64;           // scalar-modulus constants
  MG32 pc32;
  int64_t n;
  int64_t last;        // result's last dimension (dense kernel)
  FastDiv last_div;    // division by `last` (dense kernel, n < 2^32)
  int p_per_last;      // dense kernel: modulus index = coordinate on the last axis
  int b_stream;        // dense kernel, in-place update r = a op b: b is loaded evict-first so that the
                       // updated tensor (read next) keeps its place in L2
  FastDims fd;         // general kernel: 32-bit decomposition of r's coordinates
  int vs_a, vs_b, vs_pd;  // vector kernel: innermost stride (0 or 1) of a, b and the modulus index
  int off32;              // vector kernel: every offset fits 32 bits
  Diag *diag;
};

// ------------------------------------------------------------ element op
template <typename T> struct MGOf;
template <> struct MGOf<int32_t> { typedef MG32 type; };
template <> struct MGOf<int64_t> { typedef MG64 type; };

template <typename T, int OP>
__device__ __forceinline__ T elem_op(int64_t a, int64_t b, int64_t p, const typename MGOf<T>::type &c, Diag *diag) {
  if (OP == OP_MOD) {  // (T)(a % b) in T; p unused
    if (b == 0) {
      atomicAdd(&diag->zero_mod, 1ull);
      return 0;
    }
    if (b == -1) return 0;
    return (T)(a % b);
  }
  if (p == 0) {
    atomicAdd(&diag->zero_mod, 1ull);
    return 0;
  }
  if (OP == OP_MUL) {
    if (a >= 0 && b >= 0 && p > 0) {
      if (sizeof(T) == 4) return (T)mg32_mod((uint64_t)a * (uint64_t)b, (const MG32 &)c);
      return (T)mg64_mulmod((uint64_t)a, (uint64_t)b, (const MG64 &)c);
    }
    return (T)((i128)a * (i128)b % (i128)p);
  }
  if (OP == OP_SUM) {
    if (a >= 0 && b >= 0 && p > 0) {
      uint64_t x = (uint64_t)a + (uint64_t)b;
      if (a < p && b < p) return (T)(x >= (uint64_t)p ? x - (uint64_t)p : x);
      return (T)(x % (uint64_t)p);
    }
    return (T)(((i128)a + (i128)b) % (i128)p);
  }
  // OP_NEG: (p - a % p) % p
  if (a >= 0 && p > 0) {
    int64_t t = a < p ? a : a % p;
    return (T)(t ? p - t : 0);
  }
  i128 t = (i128)a % (i128)p;
  return (T)(((i128)p - t) % (i128)p);
}

// modulus constants and value of modulus element `idx` (table) or the scalar
template <typename T>
__device__ __forceinline__ typename MGOf<T>::type mg_of(const ModopArgs &g, int64_t idx) {
  typedef typename MGOf<T>::type M;
  if (g.ptab) return ((const M *)g.ptab)[idx];
  if (sizeof(T) == 4) {
    MG32 c = g.pc32;
    return *(const M *)&c;
  }
  MG64 c = g.pc64;
  return *(const M *)&c;
}
template <typename T>
__device__ __forceinline__ int64_t q_of(const ModopArgs &g, const typename MGOf<T>::type &c) {
  if (!g.ptab) return g.ps;
  return sizeof(T) == 4 ? (int64_t)(int32_t)c.q : (int64_t)c.q;
}

template <typename T>
struct VecOf {
  typedef typename std::conditional<sizeof(T) == 8, longlong2, int4>::type type;
};

// ------------------------------------------------------ dense kernel
// result, a (and b) row-major with result's shape; VEC elements per vector,
// two vectors per iteration.  With HOIST the grid stride is a multiple of
// the modulus period (`last`), so every thread keeps the same moduli for its
// whole run and loads their constants once.
// Grid: 8 CTAs of 256 threads per SM, except for the 64-bit multiplication.
// Its reduction took 66 registers (3 resident CTAs per SM against a grid of
// 8, so the last of 2.7 waves ran a third empty); its own entry kernel
// (modop_dense_mul64_kernel) is held to 64 registers by its launch bound, 4
// resident CTAs, and its grid is exactly 4 per SM.
template <typename T, int OP>
constexpr bool dense_wide_mul() { return OP == OP_MUL && sizeof(T) == 8; }
template <typename T, int OP>
constexpr int dense_blocks_per_sm() { return dense_wide_mul<T, OP>() ? 4 : 8; }
template <typename T, int OP, int VEC, bool HOIST>
__device__ __forceinline__ void modop_dense_body(const ModopArgs &g) {
  typedef typename VecOf<T>::type V;
  typedef typename MGOf<T>::type M;
  const T *A = (const T *)g.ap;
  const T *B = (const T *)g.bp;
  T *R = (T *)g.rp;
  const int64_t nvec = g.n / VEC;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  auto col_of = [&](int64_t e) -> uint32_t {
    return g.p_per_last ? (uint32_t)e - fastdiv((uint32_t)e, g.last_div) * (uint32_t)g.last : 0u;
  };
  M cst[VEC];
  int64_t qv[VEC];
  if (HOIST) {
    uint32_t col = col_of(v * VEC);
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
      cst[j] = mg_of<T>(g, col);
      qv[j] = q_of<T>(g, cst[j]);
      if (g.p_per_last && ++col == (uint32_t)g.last) col = 0;
    }
  }
  auto compute = [&](int64_t base, const T *av, const T *bv, T *rv) {
    uint32_t col = HOIST ? 0u : col_of(base);
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
      const int64_t b = B ? (int64_t)bv[j] : g.bs;
      if (HOIST) {
        rv[j] = elem_op<T, OP>((int64_t)av[j], b, qv[j], cst[j], g.diag);
      } else {
        const M c = mg_of<T>(g, col);
        rv[j] = elem_op<T, OP>((int64_t)av[j], b, q_of<T>(g, c), c, g.diag);
        if (g.p_per_last && ++col == (uint32_t)g.last) col = 0;
      }
    }
  };
  for (; v + stride < nvec; v += 2 * stride) {
    T a0[VEC], a1[VEC], b0[VEC], b1[VEC], r0[VEC], r1[VEC];
    if (VEC == 1) {
      a0[0] = A[v];
      a1[0] = A[v + stride];
      if (B) {
        b0[0] = B[v];
        b1[0] = B[v + stride];
      }
    } else {
      *(V *)a0 = *(const V *)(A + v * VEC);
      *(V *)a1 = *(const V *)(A + (v + stride) * VEC);
      if (B) {
        if (g.b_stream) {
          *(V *)b0 = __ldcs((const V *)(B + v * VEC));
          *(V *)b1 = __ldcs((const V *)(B + (v + stride) * VEC));
        } else {
          *(V *)b0 = *(const V *)(B + v * VEC);
          *(V *)b1 = *(const V *)(B + (v + stride) * VEC);
        }
      }
    }
    compute(v * VEC, a0, b0, r0);
    compute((v + stride) * VEC, a1, b1, r1);
    if (VEC == 1) {
      R[v] = r0[0];
      R[v + stride] = r1[0];
    } else {
      *(V *)(R + v * VEC) = *(const V *)r0;
      *(V *)(R + (v + stride) * VEC) = *(const V *)r1;
    }
  }
  if (v < nvec) {
    T a0[VEC], b0[VEC], r0[VEC];
    if (VEC == 1) {
      a0[0] = A[v];
      if (B) b0[0] = B[v];
    } else {
      *(V *)a0 = *(const V *)(A + v * VEC);
      if (B) *(V *)b0 = *(const V *)(B + v * VEC);
    }
    compute(v * VEC, a0, b0, r0);
    if (VEC == 1)
      R[v] = r0[0];
    else
      *(V *)(R + v * VEC) = *(const V *)r0;
  }
  // tail (n not a multiple of VEC)
  if (VEC > 1 && blockIdx.x == 0 && (int64_t)threadIdx.x < g.n % VEC) {
    int64_t i = nvec * VEC + threadIdx.x;
    const M c = mg_of<T>(g, col_of(i));
    int64_t b = B ? (int64_t)B[i] : g.bs;
    R[i] = elem_op<T, OP>((int64_t)A[i], b, q_of<T>(g, c), c, g.diag);
  }
}

template <typename T, int OP, int VEC, bool HOIST>
__global__ void __launch_bounds__(256) modop_dense_kernel(const __grid_constant__ ModopArgs g) {
  modop_dense_body<T, OP, VEC, HOIST>(g);
}

template <int VEC, bool HOIST>
__global__ void __launch_bounds__(256, dense_blocks_per_sm<int64_t, OP_MUL>())
    modop_dense_mul64_kernel(const __grid_constant__ ModopArgs g) {
  modop_dense_body<int64_t, OP_MUL, VEC, HOIST>(g);
}

// ---------------------------------------------------- general kernel
// Any strides (broadcast axes have stride 0), axes merged on the host where
// every operand allows.  Each thread takes kGenU elements a block-width
// apart per iteration and issues all their loads before the arithmetic, so
// enough bytes are in flight to cover HBM latency.
constexpr int kGenU = 4;

template <typename T, int OP>
__global__ void __launch_bounds__(256) modop_general_kernel(const __grid_constant__ ModopArgs g) {
  typedef typename MGOf<T>::type M;
  const T *A = (const T *)g.ap;
  const T *B = (const T *)g.bp;
  T *R = (T *)g.rp;
  const int64_t step = (int64_t)gridDim.x * blockDim.x * kGenU;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x * kGenU + threadIdx.x; base < g.n; base += step) {
    int64_t oa[kGenU], ob[kGenU], orr[kGenU], opd[kGenU];
#pragma unroll
    for (int u = 0; u < kGenU; ++u) {
      const int64_t idx = base + (int64_t)u * blockDim.x;
      oa[u] = ob[u] = orr[u] = opd[u] = 0;
      if (idx >= g.n) continue;
      if (g.fd.fast) {
        uint32_t rem = (uint32_t)idx;
#pragma unroll
        for (int k = 0; k < HEAL_MAX_DIMS; ++k) {  // unrolled: per-axis parameters at fixed offsets
          const int i = HEAL_MAX_DIMS - 1 - k;
          if (i >= g.r.ndim) continue;
          const uint32_t q = fastdiv(rem, g.fd.fd[i]);
          const int64_t c = rem - q * (uint32_t)g.r.dims[i];
          rem = q;
          oa[u] += c * g.a.strides[i];
          ob[u] += c * g.b.strides[i];
          opd[u] += c * g.pd.strides[i];
          orr[u] += c * g.r.strides[i];
        }
      } else {
        int64_t rem = idx;
        for (int i = g.r.ndim - 1; i >= 0; --i) {
          const int64_t d = g.r.dims[i];
          const int64_t c = rem % d;
          rem /= d;
          oa[u] += c * g.a.strides[i];
          ob[u] += c * g.b.strides[i];
          opd[u] += c * g.pd.strides[i];
          orr[u] += c * g.r.strides[i];
        }
      }
    }
    int64_t av[kGenU], bv[kGenU];
    M cv[kGenU];
#pragma unroll
    for (int u = 0; u < kGenU; ++u) {
      const bool in = base + (int64_t)u * blockDim.x < g.n;
      av[u] = in ? (int64_t)A[oa[u]] : 0;
      bv[u] = (in && B) ? (int64_t)B[ob[u]] : g.bs;
      cv[u] = mg_of<T>(g, in ? opd[u] : 0);
    }
#pragma unroll
    for (int u = 0; u < kGenU; ++u)
      if (base + (int64_t)u * blockDim.x < g.n)
        R[orr[u]] = elem_op<T, OP>(av[u], bv[u], q_of<T>(g, cv[u]), cv[u], g.diag);
  }
}

// ------------------------------------------------ vector kernel
// The general kernel's work in units of VEC elements of the innermost axis
// (16 bytes of result): a result that is contiguous there, with operands
// that are contiguous (vector loads) or broadcast (one load) along it — a
// plaintext or diagonal broadcast over the ciphertext's polynomials or
// slots.  The views hold the innermost axis divided by VEC, with its strides
// multiplied by VEC, so one decomposition gives a unit's first element; its
// other elements follow at vs_* apart.
constexpr int kVecU = 4;

template <typename T, int OP, int VEC, typename Off>
__global__ void __launch_bounds__(256) modop_vec_kernel(const __grid_constant__ ModopArgs g) {
  typedef typename VecOf<T>::type V;
  typedef typename MGOf<T>::type M;
  const T *A = (const T *)g.ap;
  const T *B = (const T *)g.bp;
  T *R = (T *)g.rp;
  const int64_t units = g.n / VEC;
  const int64_t step = (int64_t)gridDim.x * blockDim.x * kVecU;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x * kVecU + threadIdx.x; base < units; base += step) {
    Off oa[kVecU], ob[kVecU], orr[kVecU], opd[kVecU];
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      const int64_t idx = base + (int64_t)u * blockDim.x;
      oa[u] = ob[u] = orr[u] = opd[u] = 0;
      if (idx >= units) continue;
      if (g.fd.fast) {
        uint32_t rem = (uint32_t)idx;
#pragma unroll
        for (int k = 0; k < HEAL_MAX_DIMS; ++k) {  // unrolled: per-axis parameters at fixed offsets
          const int i = HEAL_MAX_DIMS - 1 - k;
          if (i >= g.r.ndim) continue;
          const uint32_t q = fastdiv(rem, g.fd.fd[i]);
          const Off c = (Off)(rem - q * (uint32_t)g.r.dims[i]);
          rem = q;
          oa[u] += c * (Off)g.a.strides[i];
          ob[u] += c * (Off)g.b.strides[i];
          opd[u] += c * (Off)g.pd.strides[i];
          orr[u] += c * (Off)g.r.strides[i];
        }
      } else {
        int64_t rem = idx;
        for (int i = g.r.ndim - 1; i >= 0; --i) {
          const int64_t c = rem % g.r.dims[i];
          rem /= g.r.dims[i];
          oa[u] += (Off)(c * g.a.strides[i]);
          ob[u] += (Off)(c * g.b.strides[i]);
          opd[u] += (Off)(c * g.pd.strides[i]);
          orr[u] += (Off)(c * g.r.strides[i]);
        }
      }
    }
    T av[kVecU][VEC], bv[kVecU][VEC];
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      if (base + (int64_t)u * blockDim.x >= units) continue;
      if (g.vs_a) {
        *(V *)av[u] = *(const V *)(A + oa[u]);
      } else {
        const T x = A[oa[u]];
#pragma unroll
        for (int j = 0; j < VEC; ++j) av[u][j] = x;
      }
      if (B && g.vs_b) {
        *(V *)bv[u] = *(const V *)(B + ob[u]);
      } else {
        const T x = B ? B[ob[u]] : (T)g.bs;
#pragma unroll
        for (int j = 0; j < VEC; ++j) bv[u][j] = x;
      }
    }
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      if (base + (int64_t)u * blockDim.x >= units) continue;
      T rv[VEC];
#pragma unroll
      for (int j = 0; j < VEC; ++j) {
        const M c = mg_of<T>(g, opd[u] + j * g.vs_pd);
        const int64_t b = B ? (int64_t)bv[u][j] : g.bs;
        rv[j] = elem_op<T, OP>((int64_t)av[u][j], b, q_of<T>(g, c), c, g.diag);
      }
      *(V *)(R + orr[u]) = *(const V *)rv;
    }
  }
}

// Reduction constants of every modulus element, written into a caller-given
// array (the allocation-free modmul's fixed scratch).
__global__ void mod_table_kernel_noalloc(const void *p, int dtype, View v, int64_t n, void *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t off = 0, idx = i;
    for (int d = v.ndim - 1; d >= 0; --d) {
      off += (idx % v.dims[d]) * v.strides[d];
      idx /= v.dims[d];
    }
    if (dtype == HEAL_INT32)
      ((MG32 *)out)[i] = mg32_make((int64_t)((const int32_t *)p)[off]);
    else
      ((MG64 *)out)[i] = mg64_make(((const int64_t *)p)[off]);
  }
}

// ----------------------------------------------------------- host side
static int grid_for(int64_t work, int threads, int per_sm) {
  int64_t want = (work + threads - 1) / threads;
  int64_t cap = (int64_t)std::max(device_sm_count(), 1) * per_sm;
  return (int)std::max<int64_t>(1, std::min(want, cap));
}

// View of `t` in the coordinates of `r` (right-aligned, stride 0 on size-1
// axes, as at_with_broadcast reads it).
static View bcast_view(const heal_tensor &t, const heal_tensor &r) {
  View v = make_view(r);
  int off = r.ndim - t.ndim;
  for (int j = 0; j < r.ndim; ++j) {
    int i = j - off;
    v.strides[j] = (i < 0 || t.dims[i] == 1) ? 0 : t.strides[i];
  }
  return v;
}

// dense row-major strides of `t` mapped into r's coordinates
static View bcast_dense_view(const heal_tensor &t, const heal_tensor &r) {
  heal_tensor d = t;
  int64_t s = 1;
  for (int i = t.ndim - 1; i >= 0; --i) {
    d.strides[i] = s;
    s *= t.dims[i];
  }
  return bcast_view(d, r);
}

static bool dense_rowmajor(const heal_tensor &t) {
  int64_t s = 1;
  for (int i = t.ndim - 1; i >= 0; --i) {
    if (t.dims[i] != 1 && t.strides[i] != s) return false;
    s *= t.dims[i];
  }
  return true;
}

static int check_bcast(const heal_tensor &t, const heal_tensor &r, const char *label) {
  // CHECK_DIMS_BROADCASTABLE (modop_impl.cpp:89-101)
  if (t.ndim > r.ndim) return set_error(HEAL_ERR_INVALID_ARGUMENT, std::string(label) + " has more dims than result.");
  for (int i = 1; i <= t.ndim; ++i) {
    int64_t td = t.dims[t.ndim - i], rd = r.dims[r.ndim - i];
    if (td != 1 && td != rd)
      return set_error(HEAL_ERR_INVALID_ARGUMENT, std::string(label) + " not broadcast-compatible with result.");
  }
  return HEAL_OK;
}

static int check_p(const heal_tensor &p, const heal_tensor &r) {
  // CHECK_DIMS_MATCH_LAST (modop_impl.cpp:84-87), then the bounds at() applies
  // to at_with_broadcast's indices (device_memory_impl.cpp:100-103,116-124).
  if (p.ndim != 1 && (p.ndim == 0 || r.ndim == 0 || p.dims[p.ndim - 1] != r.dims[r.ndim - 1]))
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "Last dimension of p must match last dimension of result.");
  if (p.ndim > r.ndim) return set_error(HEAL_ERR_INVALID_ARGUMENT, "p has more dims than result.");
  if (numel(r) == 0) return HEAL_OK;
  int off = r.ndim - p.ndim;
  for (int i = 0; i < p.ndim; ++i)
    if (p.dims[i] != 1 && p.dims[i] < r.dims[i + off]) return set_error(HEAL_ERR_OUT_OF_RANGE, "Index out of bounds.");
  return HEAL_OK;
}

// Blocks for the dense kernel: about `want`, rounded to a multiple of the
// modulus period so that every thread keeps its moduli (0 when impossible).
static int64_t hoist_blocks(int64_t last, int vec, int64_t want) {
  if (last <= 0) return 0;
  int64_t per = 256 * (int64_t)vec, a = last, b = per;
  while (b) {
    int64_t t = a % b;
    a = b;
    b = t;
  }
  const int64_t unit = last / a;  // blocks per period
  if (unit > want) return 0;
  return (want / unit) * unit;
}

// Switches merged general-kernel views to the vector kernel's units when
// the result is contiguous on its innermost axis and each operand is
// contiguous (in aligned 16-byte vectors) or broadcast there.
static bool vector_units(ModopArgs &g, size_t elem) {
  const int vec = (int)(16 / elem);
  const int in = g.r.ndim - 1;
  if (in < 0 || !inner_vectors(g.r, vec, g.rp, elem)) return false;
  auto operand = [&](const View &v, const void *base) {
    return v.strides[in] == 0 || inner_vectors(v, vec, base, elem);
  };
  if (!operand(g.a, g.ap) || (g.bp && !operand(g.b, g.bp))) return false;
  if (g.pd.strides[in] != 0 && g.pd.strides[in] != 1) return false;
  g.off32 = view_off32(g.r) && view_off32(g.a) && view_off32(g.b) && view_off32(g.pd);
  g.vs_a = (int)g.a.strides[in];
  g.vs_b = g.bp ? (int)g.b.strides[in] : 0;
  g.vs_pd = (int)g.pd.strides[in];
  View *vs[5] = {&g.r, &g.a, &g.b, &g.p, &g.pd};
  for (View *v : vs) {
    v->dims[in] /= vec;
    v->strides[in] *= vec;
  }
  return true;
}

template <typename T, int OP, int VEC>
static void launch_dense(ModopArgs &g, cudaStream_t s, int64_t want_blocks) {
  const int64_t vecs = (g.n / VEC + 1) / 2 + 1;  // two vectors per thread per iteration
  const int64_t want = std::max<int64_t>(1, std::min<int64_t>(want_blocks, (vecs + 255) / 256));
  const int64_t hb = g.p_per_last ? hoist_blocks(g.last, VEC, want_blocks) : want;
  if constexpr (dense_wide_mul<T, OP>()) {
    if (hb > 0)
      modop_dense_mul64_kernel<VEC, true><<<(unsigned)hb, 256, 0, s>>>(g);
    else
      modop_dense_mul64_kernel<VEC, false><<<(unsigned)want, 256, 0, s>>>(g);
  } else {
    if (hb > 0)
      modop_dense_kernel<T, OP, VEC, true><<<(unsigned)hb, 256, 0, s>>>(g);
    else
      modop_dense_kernel<T, OP, VEC, false><<<(unsigned)want, 256, 0, s>>>(g);
  }
}

enum Kind { KIND_GENERAL = 0, KIND_DENSE = 1, KIND_VEC = 2 };

template <typename T, int OP>
static int launch(ModopArgs &g, int kind) {
  cudaStream_t s = stream();
  if (kind == KIND_VEC) {
    constexpr int VEC = 16 / sizeof(T);
    const int grid = grid_for((g.n / VEC + kVecU - 1) / kVecU, 256, 8);
    if (g.off32)
      modop_vec_kernel<T, OP, VEC, int32_t><<<grid, 256, 0, s>>>(g);
    else
      modop_vec_kernel<T, OP, VEC, int64_t><<<grid, 256, 0, s>>>(g);
  } else if (kind == KIND_DENSE) {
    bool aligned = ((uintptr_t)g.ap % 16 == 0) && ((uintptr_t)g.rp % 16 == 0) && (!g.bp || (uintptr_t)g.bp % 16 == 0);
    const int64_t want = (int64_t)std::max(device_sm_count(), 1) * dense_blocks_per_sm<T, OP>();
    if (aligned)
      launch_dense<T, OP, 16 / sizeof(T)>(g, s, want);
    else
      launch_dense<T, OP, 1>(g, s, want);
  } else {
    modop_general_kernel<T, OP><<<grid_for((g.n + kGenU - 1) / kGenU, 256, 8), 256, 0, s>>>(g);
  }
  return check_launch("modop");
}

// a, b (tensor or scalar), p (tensor or scalar) -> result
static int modop(int op, const heal_tensor *a, const heal_tensor *b, int64_t bs, const heal_tensor *p, int64_t ps,
                 const heal_tensor *r) {
  clear_error();
  HEAL_CHECK(check_desc(a, "a", true));
  if (b) HEAL_CHECK(check_desc(b, "b", true));
  if (p) HEAL_CHECK(check_desc(p, "p", true));
  HEAL_CHECK(check_desc(r, "result", true));
  HEAL_CHECK(ensure_init());
  const int dt = r->dtype;
  if (a->dtype != dt || (b && b->dtype != dt) || (p && p->dtype != dt))
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "all tensors must have the element type of result");
  if (op == OP_MOD) {
    // CHECK_SAME_DIMS (modop_impl.cpp:183-186)
    if (!same_dims(*a, *r)) return set_error(HEAL_ERR_INVALID_ARGUMENT, "a must have exactly the same shape as result.");
    if (b && !same_dims(*b, *r))
      return set_error(HEAL_ERR_INVALID_ARGUMENT, "b must have exactly the same shape as result.");
  } else {
    HEAL_CHECK(check_bcast(*a, *r, "a"));
    if (b) HEAL_CHECK(check_bcast(*b, *r, "b"));
    if (p) HEAL_CHECK(check_p(*p, *r));
  }
  const int64_t n = numel(*r);
  if (n == 0) return HEAL_OK;

  // inputs that overlap the result in another layout are copied first
  heal_tensor A = *a, B = b ? *b : heal_tensor(), P = p ? *p : heal_tensor();
  void *owned[3] = {nullptr, nullptr, nullptr};
  auto detach = [&](heal_tensor &t, int slot) -> int {
    if (overlaps(t, *r) && !identical_view(t, *r)) return materialize(t, &t, &owned[slot]);
    return HEAL_OK;
  };
  int rc = detach(A, 0);
  if (!rc && b) rc = detach(B, 1);
  if (!rc && p) rc = detach(P, 2);

  ModopArgs g;
  memset(&g, 0, sizeof g);
  if (!rc) {
    g.r = make_view(*r);
    g.a = bcast_view(A, *r);
    g.b = b ? bcast_view(B, *r) : make_view(*r);
    g.p = p ? bcast_view(P, *r) : make_view(*r);
    g.pd = p ? bcast_dense_view(P, *r) : make_view(*r);
    if (!b)
      for (int i = 0; i < HEAL_MAX_DIMS; ++i) g.b.strides[i] = 0;
    if (!p)
      for (int i = 0; i < HEAL_MAX_DIMS; ++i) g.p.strides[i] = g.pd.strides[i] = 0;
    g.ap = A.data;
    g.bp = b ? B.data : nullptr;
    g.pp = p ? P.data : nullptr;
    g.rp = r->data;
    g.bs = dt == HEAL_INT32 ? (int64_t)(int32_t)bs : bs;
    g.ps = dt == HEAL_INT32 ? (int64_t)(int32_t)ps : ps;
    g.n = n;
    g.diag = diag_device();
    g.last = r->ndim ? r->dims[r->ndim - 1] : 1;
    if (op != OP_MOD) {
      if (p) {
        ModTable mt;
        rc = mod_table(P, &mt);
        g.ptab = mt.consts;
      } else {
        g.pc64 = mg64_make(g.ps);
        g.pc32 = mg32_make(g.ps);
      }
    }
  }
  if (!rc) {
    // dense: result, a, b row-major with result's shape; p scalar or [k] on
    // the last axis (k == last or broadcast 1)
    bool dense = dense_rowmajor(*r) && same_dims(A, *r) && dense_rowmajor(A) &&
                 (!b || (same_dims(B, *r) && dense_rowmajor(B))) && n < (int64_t)UINT32_MAX && r->ndim > 0;
    if (dense && p) {
      bool vec_last = P.ndim == 1 && (P.dims[0] == 1 || g.last <= P.dims[0]);
      dense = vec_last && P.strides[0] == 1;
      g.p_per_last = vec_last && P.dims[0] != 1;
    }
    if (dense && g.last > 0 && g.last < (int64_t)UINT32_MAX) g.last_div = fastdiv_make((uint32_t)g.last);
    else dense = dense && !g.p_per_last;
    g.b_stream = dense && b && A.data == r->data && B.data != r->data;
    int kind = dense ? KIND_DENSE : KIND_GENERAL;
    if (!dense) {
      // general kernel: merge axes that every operand walks linearly
      View *vs[4] = {&g.r, &g.a, &g.b, &g.pd};
      coalesce_views(vs, 4, 0u, nullptr);
      if (vector_units(g, elem_size(dt))) kind = KIND_VEC;
      make_fast_dims(g.r, kind == KIND_VEC ? n / (16 / elem_size(dt)) : n, &g.fd);
      g.off32 = g.off32 && g.fd.fast;
    }
    if (op == OP_MOD) {
      // mod_tt / tc / ct: a and b play the roles of dividend and divisor
      rc = dt == HEAL_INT32 ? launch<int32_t, OP_MOD>(g, kind) : launch<int64_t, OP_MOD>(g, kind);
    } else if (dt == HEAL_INT32) {
      rc = op == OP_MUL ? launch<int32_t, OP_MUL>(g, kind)
           : op == OP_SUM ? launch<int32_t, OP_SUM>(g, kind) : launch<int32_t, OP_NEG>(g, kind);
    } else {
      rc = op == OP_MUL ? launch<int64_t, OP_MUL>(g, kind)
           : op == OP_SUM ? launch<int64_t, OP_SUM>(g, kind) : launch<int64_t, OP_NEG>(g, kind);
    }
  }
  for (void *o : owned) scratch_free(o);
  if (!rc) mark_written(r->data);
  return rc;
}

// mod_ct: scalar dividend, tensor divisor — run as a general kernel over b
static int mod_ct(int64_t as, const heal_tensor *b, const heal_tensor *r) {
  clear_error();
  HEAL_CHECK(check_desc(b, "b", true));
  HEAL_CHECK(check_desc(r, "result", true));
  HEAL_CHECK(ensure_init());
  if (b->dtype != r->dtype) return set_error(HEAL_ERR_INVALID_ARGUMENT, "all tensors must have the element type of result");
  if (!same_dims(*b, *r)) return set_error(HEAL_ERR_INVALID_ARGUMENT, "b must have exactly the same shape as result.");
  const int64_t n = numel(*r);
  if (n == 0) return HEAL_OK;
  // a scalar broadcast as a stride-0 view over b's shape is the dividend
  heal_tensor B = *b;
  void *owned = nullptr;
  if (overlaps(B, *r) && !identical_view(B, *r)) HEAL_CHECK(materialize(B, &B, &owned));
  ModopArgs g;
  memset(&g, 0, sizeof g);
  g.r = make_view(*r);
  g.b = make_view(B);
  g.a = make_view(*r);
  for (int i = 0; i < HEAL_MAX_DIMS; ++i) g.a.strides[i] = 0;
  g.p = g.pd = g.a;
  g.n = n;
  g.diag = diag_device();
  g.rp = r->data;
  g.bp = B.data;
  int rc;
  // the dividend lives in a one-element device buffer
  void *sbuf;
  HEAL_CHECK(scratch_alloc(8, &sbuf));
  int64_t v64 = as;
  int32_t v32 = (int32_t)as;
  rc = cudaMemcpyAsync(sbuf, r->dtype == HEAL_INT32 ? (const void *)&v32 : (const void *)&v64,
                       elem_size(r->dtype), cudaMemcpyHostToDevice, stream()) == cudaSuccess
           ? HEAL_OK
           : set_error(HEAL_ERR_CUDA, "mod_ct: copy failed");
  g.ap = sbuf;
  if (!rc) rc = r->dtype == HEAL_INT32 ? launch<int32_t, OP_MOD>(g, KIND_GENERAL) : launch<int64_t, OP_MOD>(g, KIND_GENERAL);
  scratch_free(sbuf);
  scratch_free(owned);
  if (!rc) mark_written(r->data);
  return rc;
}

// ================================================ allocation-free modmul
// Some callers cannot let a library allocate device memory: a serving
// process that reserves HBM for its resident ciphertexts and keys up front
// and fails any later cudaMalloc, a host runtime (Go, Java, ...) that owns
// every device buffer through its own pool, or a latency-bound loop that
// must not stall in the allocator.  heal_modmul_ttt_noalloc serves them:
// the table it needs (the reduction constants of each modulus, which
// heal_modmul_ttt caches in pool memory) lives in this fixed array instead.
// Every GPU that loads the library keeps the array (128 KiB of constants and
// one diagnostics record) until the process exits.
constexpr int64_t kNoAllocMaxModuli = 4096;
constexpr size_t kNoAllocTableBytes = (size_t)kNoAllocMaxModuli * sizeof(MG64);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocTableBytes + sizeof(Diag)];

struct NoAllocDevice {
  void *scratch = nullptr;  // device address of g_noalloc_scratch
  int sms = 0;
};
static std::mutex g_noalloc_mu;
static NoAllocDevice g_noalloc_dev[64];

// First call on a device: resolve the array's device address (the host-side
// symbol is not one) with that device current.  This happens on the first
// call per device, which should come before any stream capture.
static int noalloc_setup(NoAllocDevice **out) {
  int dev = 0;
  HEAL_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(HEAL_ERR_RUNTIME, "heal_modmul_ttt_noalloc: device ordinal above 63");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocDevice &d = g_noalloc_dev[dev];
  if (!d.scratch) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    HEAL_TRY_CUDA(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
    d.scratch = ptr;
  }
  *out = &d;
  return HEAL_OK;
}

template <typename T>
static int noalloc_launch(ModopArgs &g, bool dense, cudaStream_t s, int sms) {
  auto grid = [&](int64_t work) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, (int64_t)std::max(sms, 1) * 8));
  };
  if (dense) {
    const int vec = 16 / sizeof(T);
    bool aligned = ((uintptr_t)g.ap % 16 == 0) && ((uintptr_t)g.rp % 16 == 0) && ((uintptr_t)g.bp % 16 == 0);
    const int64_t want = (int64_t)std::max(sms, 1) * dense_blocks_per_sm<T, OP_MUL>();
    (void)vec;
    if (aligned)
      launch_dense<T, OP_MUL, 16 / sizeof(T)>(g, s, want);
    else
      launch_dense<T, OP_MUL, 1>(g, s, want);
  } else {
    modop_general_kernel<T, OP_MUL><<<grid(g.n), 256, 0, s>>>(g);
  }
  return check_launch("modmul_ttt_noalloc");
}

static int modmul_noalloc(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, const heal_tensor *r,
                          void *stream_ptr) {
  clear_error();
  HEAL_CHECK(check_desc(a, "a", true));
  HEAL_CHECK(check_desc(b, "b", true));
  HEAL_CHECK(check_desc(p, "p", true));
  HEAL_CHECK(check_desc(r, "result", true));
  const int dt = r->dtype;
  if (a->dtype != dt || b->dtype != dt || p->dtype != dt)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "all tensors must have the element type of result");
  HEAL_CHECK(check_bcast(*a, *r, "a"));
  HEAL_CHECK(check_bcast(*b, *r, "b"));
  HEAL_CHECK(check_p(*p, *r));
  const int64_t np = numel(*p);
  if (np > kNoAllocMaxModuli)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_modmul_ttt_noalloc: p has " + std::to_string(np) +
                                                    " elements; at most 4096 are supported");
  for (const heal_tensor *in : {a, b, p})
    if (overlaps(*in, *r) && !identical_view(*in, *r))
      return set_error(HEAL_ERR_INVALID_ARGUMENT,
                       "heal_modmul_ttt_noalloc: result overlaps an input in another layout (that needs a copy)");
  const int64_t n = numel(*r);
  if (n == 0) return HEAL_OK;
  // the launch checks below read the calling thread's last CUDA error: one
  // left pending by an earlier call (another library, another stream) is
  // reported as that, not as a failure of this call's launches
  const cudaError_t pending = cudaGetLastError();
  if (pending != cudaSuccess)
    return cuda_fail(pending, "heal_modmul_ttt_noalloc: a CUDA error left pending by an earlier call on this thread");
  NoAllocDevice *dev = nullptr;
  HEAL_CHECK(noalloc_setup(&dev));
  cudaStream_t s = (cudaStream_t)stream_ptr;
  unsigned char *scratch = (unsigned char *)dev->scratch;

  // the constants of this call's moduli, written over the previous call's
  const int threads = 128;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((np + threads - 1) / threads, 1024));
  mod_table_kernel_noalloc<<<blocks, threads, 0, s>>>(p->data, p->dtype, make_view(*p), np, scratch);
  HEAL_CHECK(check_launch("modmul_ttt_noalloc constants"));

  ModopArgs g;
  memset(&g, 0, sizeof g);
  g.r = make_view(*r);
  g.a = bcast_view(*a, *r);
  g.b = bcast_view(*b, *r);
  g.p = bcast_view(*p, *r);
  g.pd = bcast_dense_view(*p, *r);
  g.ap = a->data;
  g.bp = b->data;
  g.pp = p->data;
  g.rp = r->data;
  g.ptab = scratch;
  g.n = n;
  g.diag = (Diag *)(scratch + kNoAllocTableBytes);  // written, never read back here
  g.last = r->ndim ? r->dims[r->ndim - 1] : 1;
  bool dense = dense_rowmajor(*r) && same_dims(*a, *r) && dense_rowmajor(*a) && same_dims(*b, *r) &&
               dense_rowmajor(*b) && n < (int64_t)UINT32_MAX && r->ndim > 0;
  if (dense) {
    bool vec_last = p->ndim == 1 && (p->dims[0] == 1 || g.last <= p->dims[0]);
    dense = vec_last && p->strides[0] == 1;
    g.p_per_last = vec_last && p->dims[0] != 1;
  }
  if (dense && g.last > 0 && g.last < (int64_t)UINT32_MAX)
    g.last_div = fastdiv_make((uint32_t)g.last);
  else
    dense = dense && !g.p_per_last;
  int rc = dt == HEAL_INT32 ? noalloc_launch<int32_t>(g, dense, s, dev->sms)
                            : noalloc_launch<int64_t>(g, dense, s, dev->sms);
  if (!rc) mark_written(r->data);
  return rc;
}

}  // namespace heal

using namespace heal;

extern "C" {

int heal_modmul_ttt(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, const heal_tensor *r) {
  if (!p) return set_error(HEAL_ERR_INVALID_ARGUMENT, "p pointer must not be null.");
  if (!b) return set_error(HEAL_ERR_INVALID_ARGUMENT, "b pointer must not be null.");
  return modop(OP_MUL, a, b, 0, p, 0, r);
}
int heal_modmul_ttc(const heal_tensor *a, const heal_tensor *b, int64_t p, const heal_tensor *r) {
  if (!b) return set_error(HEAL_ERR_INVALID_ARGUMENT, "b pointer must not be null.");
  return modop(OP_MUL, a, b, 0, nullptr, p, r);
}
int heal_modmul_tct(const heal_tensor *a, int64_t b, const heal_tensor *p, const heal_tensor *r) {
  if (!p) return set_error(HEAL_ERR_INVALID_ARGUMENT, "p pointer must not be null.");
  return modop(OP_MUL, a, nullptr, b, p, 0, r);
}
int heal_modmul_tcc(const heal_tensor *a, int64_t b, int64_t p, const heal_tensor *r) {
  return modop(OP_MUL, a, nullptr, b, nullptr, p, r);
}
int heal_modsum_ttt(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, const heal_tensor *r) {
  if (!p) return set_error(HEAL_ERR_INVALID_ARGUMENT, "p pointer must not be null.");
  if (!b) return set_error(HEAL_ERR_INVALID_ARGUMENT, "b pointer must not be null.");
  return modop(OP_SUM, a, b, 0, p, 0, r);
}
int heal_modsum_ttc(const heal_tensor *a, const heal_tensor *b, int64_t p, const heal_tensor *r) {
  if (!b) return set_error(HEAL_ERR_INVALID_ARGUMENT, "b pointer must not be null.");
  return modop(OP_SUM, a, b, 0, nullptr, p, r);
}
int heal_modsum_tct(const heal_tensor *a, int64_t b, const heal_tensor *p, const heal_tensor *r) {
  if (!p) return set_error(HEAL_ERR_INVALID_ARGUMENT, "p pointer must not be null.");
  return modop(OP_SUM, a, nullptr, b, p, 0, r);
}
int heal_modsum_tcc(const heal_tensor *a, int64_t b, int64_t p, const heal_tensor *r) {
  return modop(OP_SUM, a, nullptr, b, nullptr, p, r);
}
int heal_modneg_tt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *r) {
  if (!p) return set_error(HEAL_ERR_INVALID_ARGUMENT, "p pointer must not be null.");
  return modop(OP_NEG, a, nullptr, 0, p, 0, r);
}
int heal_modneg_tc(const heal_tensor *a, int64_t p, const heal_tensor *r) {
  return modop(OP_NEG, a, nullptr, 0, nullptr, p, r);
}
int heal_mod_tt(const heal_tensor *a, const heal_tensor *b, const heal_tensor *r) {
  if (!a) return set_error(HEAL_ERR_INVALID_ARGUMENT, "a pointer must not be null.");
  if (!b) return set_error(HEAL_ERR_INVALID_ARGUMENT, "b pointer must not be null.");
  return modop(OP_MOD, a, b, 0, nullptr, 0, r);
}
int heal_mod_tc(const heal_tensor *a, int64_t b, const heal_tensor *r) {
  if (!a) return set_error(HEAL_ERR_INVALID_ARGUMENT, "a pointer must not be null.");
  return modop(OP_MOD, a, nullptr, b, nullptr, 0, r);
}
int heal_mod_ct(int64_t a, const heal_tensor *b, const heal_tensor *r) {
  if (!b) return set_error(HEAL_ERR_INVALID_ARGUMENT, "b pointer must not be null.");
  return mod_ct(a, b, r);
}
int heal_modmul_ttt_noalloc(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p,
                            const heal_tensor *result, void *stream) {
  return modmul_noalloc(a, b, p, result, stream);
}

}  // extern "C"
