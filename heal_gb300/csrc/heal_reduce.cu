// heal_reduce.cu — axis_modsum, g_decomposition and permute.
//
//  axis_modsum   (HEAL include/axis_modsum.h:24-30; axis_modsum_impl.cpp)
//                one thread per output element; the reduction runs in the
//                reference's order, sum = (sum + a_r) % q, so negative
//                operands give the same truncated residues.
//  g_decomposition (include/g_decomposition.h:24-30; g_decomposition_impl.cpp)
//                on dense tensors one thread per 16-byte vector of inputs, its
//                digits written as 16-byte stores; one thread per input element
//                otherwise; `value % base` and
//                `value /= base` act on the value converted to uint64 (base is
//                a size_t), the quotient stored back in T.
//  permute       (include/permute.h:33-40; permute_impl.cpp) a gather of
//                whole rows along perm_axis.
// All three are HBM-bound streams; index arithmetic uses 32-bit invariant
// division whenever the index space fits 32 bits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <type_traits>

#include "heal_internal.h"

namespace heal {

static int grid_for(int64_t work, int threads, int per_sm) {
  int64_t want = (work + threads - 1) / threads;
  int64_t cap = (int64_t)std::max(device_sm_count(), 1) * per_sm;
  return (int)std::max<int64_t>(1, std::min(want, cap));
}

static bool dense_rowmajor(const heal_tensor &t) {
  int64_t s = 1;
  for (int i = t.ndim - 1; i >= 0; --i) {
    if (t.dims[i] != 1 && t.strides[i] != s) return false;
    s *= t.dims[i];
  }
  return true;
}

// ============================================================ axis_modsum
struct AxisArgs {
  View r;          // result view
  View ai;         // a strides in result coordinates
  int64_t ax_len, ax_stride;
  int64_t p_stride;  // p stride, indexed by the last input coordinate
  int last_from_axis;  // the last input coordinate is result's last one
  const void *a, *p;
  void *out;
  int64_t n;
  Diag *diag;
  int fast;                       // n and every dim below 2^32: 32-bit index math
  int literal;                    // reference compatibility: the running sum wraps in the element type
  FastDiv fd[HEAL_MAX_DIMS];      // division by each result dim
};

template <typename T>
__global__ void __launch_bounds__(256) axis_modsum_kernel(const __grid_constant__ AxisArgs g) {
  const T *A = (const T *)g.a;
  const T *P = (const T *)g.p;
  T *R = (T *)g.out;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < g.n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t oa = 0, orr = 0, last = 0;
    if (g.fast) {
      uint32_t rem = (uint32_t)idx;
#pragma unroll
      for (int k = 0; k < HEAL_MAX_DIMS; ++k) {  // unrolled: per-axis parameters at fixed offsets
        const int i = HEAL_MAX_DIMS - 1 - k;
        if (i >= g.r.ndim) continue;
        const uint32_t qd = fastdiv(rem, g.fd[i]);
        const int64_t c = rem - qd * (uint32_t)g.r.dims[i];
        rem = qd;
        if (i == g.r.ndim - 1) last = c;
        oa += c * g.ai.strides[i];
        orr += c * g.r.strides[i];
      }
    } else {
      int64_t rem = idx;
      for (int i = g.r.ndim - 1; i >= 0; --i) {
        int64_t d = g.r.dims[i];
        int64_t c = rem % d;
        rem /= d;
        if (i == g.r.ndim - 1) last = c;
        oa += c * g.ai.strides[i];
        orr += c * g.r.strides[i];
      }
    }
    const int64_t q = (int64_t)P[last * g.p_stride];
    if (q == 0) {
      atomicAdd(&g.diag->zero_mod, 1ull);
      R[orr] = 0;
      continue;
    }
    // the reference's running sum, in order; on long axes the loads go out
    // kBatch at a time (full batches, then the remainder one by one)
    constexpr int kBatch = 4;
    int64_t sum = 0;
    auto step = [&](int64_t v) {
      if (g.literal) {  // (sum + a_r) in the element type, then % (axis_modsum_impl.cpp:70)
        const i128 x = (i128)sum + (i128)v;
        sum = crem128(sizeof(T) == 4 ? (i128)(int32_t)(uint32_t)(uint64_t)x : (i128)(int64_t)(uint64_t)x, q);
      } else if (sum >= 0 && v >= 0 && q > 0) {
        uint64_t x = (uint64_t)sum + (uint64_t)v;
        sum = v < q ? (int64_t)(x >= (uint64_t)q ? x - (uint64_t)q : x) : (int64_t)(x % (uint64_t)q);
      } else {
        sum = crem128((i128)sum + (i128)v, q);
      }
    };
    const T *pa = A + oa;
    int64_t k = 0;
    for (; k + kBatch <= g.ax_len; k += kBatch) {
      int64_t v[kBatch];
#pragma unroll
      for (int j = 0; j < kBatch; ++j) v[j] = (int64_t)pa[(k + j) * g.ax_stride];
#pragma unroll
      for (int j = 0; j < kBatch; ++j) step(v[j]);
    }
    for (; k < g.ax_len; ++k) step((int64_t)pa[k * g.ax_stride]);
    R[orr] = (T)sum;
  }
}

// The reference's running sum of one output: sum = (sum + v) % q, C
// semantics for values outside [0, q).
__device__ __forceinline__ int64_t running_step(int64_t sum, int64_t v, int64_t q) {
  if (sum >= 0 && v >= 0 && q > 0) {
    uint64_t x = (uint64_t)sum + (uint64_t)v;
    return v < q ? (int64_t)(x >= (uint64_t)q ? x - (uint64_t)q : x) : (int64_t)(x % (uint64_t)q);
  }
  return crem128((i128)sum + (i128)v, q);
}

// Reduced axis innermost in memory: output e of a dense row-major result sums
// a[e * D + k], k < D (the digit axis of a moved [.., L, D] view).  A thread
// takes VEC = 16 / sizeof(T) consecutive outputs: their VEC * D inputs are D
// aligned 16-byte vectors, and the VEC results one 16-byte store.
struct BlockSumArgs {
  const void *a, *p;
  void *out;
  int64_t nvec;       // outputs / VEC
  int64_t p_stride;
  uint32_t last;      // result's last dimension (modulus index = e mod last)
  FastDiv last_div;
  Diag *diag;
};

template <typename T, int D>
__global__ void __launch_bounds__(256) axis_modsum_blocks_kernel(const __grid_constant__ BlockSumArgs g) {
  constexpr int VEC = 16 / sizeof(T);
  const uint4 *A = (const uint4 *)g.a;
  uint4 *R = (uint4 *)g.out;
  const T *P = (const T *)g.p;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < g.nvec;
       v += (int64_t)gridDim.x * blockDim.x) {
    union { uint4 w[D]; T x[VEC * D]; } in;
#pragma unroll
    for (int k = 0; k < D; ++k) in.w[k] = A[v * D + k];
    union { uint4 w; T x[VEC]; } out;
    const uint32_t e0 = (uint32_t)(v * VEC);
#pragma unroll
    for (int u = 0; u < VEC; ++u) {
      const uint32_t e = e0 + u;
      const uint32_t t = e - fastdiv(e, g.last_div) * g.last;
      const int64_t q = (int64_t)P[t * g.p_stride];
      int64_t sum = 0;
      if (q == 0) {
        atomicAdd(&g.diag->zero_mod, 1ull);
      } else {
#pragma unroll
        for (int k = 0; k < D; ++k) sum = running_step(sum, (int64_t)in.x[u * D + k], q);
      }
      out.x[u] = (T)sum;
    }
    R[v] = out.w;
  }
}

template <typename T>
static bool launch_blocks(const BlockSumArgs &g, int64_t D, int grid) {
  switch (D) {
    case 2: axis_modsum_blocks_kernel<T, 2><<<grid, 256, 0, stream()>>>(g); return true;
    case 3: axis_modsum_blocks_kernel<T, 3><<<grid, 256, 0, stream()>>>(g); return true;
    case 4: axis_modsum_blocks_kernel<T, 4><<<grid, 256, 0, stream()>>>(g); return true;
    default: return false;
  }
}

static int axis_modsum(const heal_tensor *a, const heal_tensor *p, const heal_tensor *r, int64_t axis) {
  clear_error();
  HEAL_CHECK(check_desc(a, "a", true));
  HEAL_CHECK(check_desc(p, "p", true));
  HEAL_CHECK(check_desc(r, "result", true));
  HEAL_CHECK(ensure_init());
  if (a->dtype != r->dtype || p->dtype != r->dtype)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "all tensors must have the element type of result");
  // axis_modsum_impl.cpp:19-33
  if (p->ndim != 1) return set_error(HEAL_ERR_INVALID_ARGUMENT, "p must be a 1D tensor of shape [k]");
  const int nd = a->ndim;
  if (axis < 0 || axis >= nd - 1)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "axis must be in range [0, ndim - 2] (can't reduce across last axis)");
  if (a->dims[nd - 1] != p->dims[0])
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "Last dimension of a must match shape of p");
  if (r->ndim != nd - 1)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "Result must have the shape of a with the reduced axis removed.");
  const int64_t n = numel(*r);
  for (int i = 0, j = 0; i < nd; ++i) {
    if (i == axis) continue;
    if (n > 0 && r->dims[j] > a->dims[i]) return set_error(HEAL_ERR_OUT_OF_RANGE, "Index out of bounds.");
    ++j;
  }
  if (n == 0) return HEAL_OK;
  heal_tensor A = *a, P = *p;
  void *oa = nullptr, *op = nullptr;
  int rc = HEAL_OK;
  if (overlaps(A, *r)) rc = materialize(A, &A, &oa);
  if (!rc && overlaps(P, *r)) rc = materialize(P, &P, &op);
  if (!rc) {
    AxisArgs g;
    memset(&g, 0, sizeof g);
    g.r = make_view(*r);
    g.ai = make_view(*r);
    for (int i = 0, j = 0; i < nd; ++i) {
      if (i == axis) continue;
      g.ai.strides[j++] = A.strides[i];
    }
    g.ax_len = A.dims[axis];
    g.ax_stride = A.strides[axis];
    g.p_stride = P.strides[0];
    g.a = A.data;
    g.p = P.data;
    g.out = r->data;
    g.n = n;
    g.diag = diag_device();
    g.fast = n < (int64_t)UINT32_MAX;
    g.literal = reference_compat();
    for (int i = 0; i < r->ndim; ++i) {
      if (r->dims[i] >= (int64_t)UINT32_MAX) g.fast = 0;
      else g.fd[i] = fastdiv_make((uint32_t)std::max<int64_t>(r->dims[i], 1));
    }
    // contiguous blocks: a unit-stride reduced axis of 2..4 elements, a's other
    // axes D times the strides of a dense row-major result, 16-byte aligned
    const int es = elem_size(r->dtype), vec = 16 / es;
    const int64_t D = g.ax_len;
    bool blocks = !g.literal && g.ax_stride == 1 && D >= 2 && D <= 4 && r->ndim > 0 && dense_rowmajor(*r) &&
                  n % vec == 0 &&
                  n < (int64_t)UINT32_MAX && (uintptr_t)A.data % 16 == 0 && (uintptr_t)r->data % 16 == 0;
    for (int i = 0; i < r->ndim && blocks; ++i) blocks = r->dims[i] == 1 || g.ai.strides[i] == D * r->strides[i];
    if (blocks) {
      BlockSumArgs bg;
      bg.a = A.data;
      bg.p = P.data;
      bg.out = r->data;
      bg.nvec = n / vec;
      bg.p_stride = P.strides[0];
      bg.last = (uint32_t)r->dims[r->ndim - 1];
      bg.last_div = fastdiv_make(bg.last);
      bg.diag = g.diag;
      const int grid = grid_for(bg.nvec, 256, 8);
      blocks = r->dtype == HEAL_INT32 ? launch_blocks<int32_t>(bg, D, grid) : launch_blocks<int64_t>(bg, D, grid);
    }
    if (blocks) {
      // launched above
    } else if (r->dtype == HEAL_INT32)
      axis_modsum_kernel<int32_t><<<grid_for(n, 256, 8), 256, 0, stream()>>>(g);
    else
      axis_modsum_kernel<int64_t><<<grid_for(n, 256, 8), 256, 0, stream()>>>(g);
    rc = check_launch("axis_modsum");
  }
  scratch_free(oa);
  scratch_free(op);
  if (!rc) mark_written(r->data);
  return rc;
}

// ======================================================== g_decomposition
struct GdecArgs {
  View a;          // input view
  int64_t r_strides[HEAL_MAX_DIMS + 1];  // result strides (a's axes, then digit axis)
  const void *in;
  void *out;
  int64_t n;
  uint64_t power, bits;
  int dense;       // a and result row-major
  Diag *diag;
};


// Dense layout, power PW <= 8: each thread decomposes the VEC elements of one
// 16-byte vector.  A warp stages the digits of its 32 vectors in shared
// memory and writes them back as contiguous 512-byte runs (a thread's own
// VEC * PW digits sit 16 * PW bytes apart from its neighbour's).
template <typename T, int PW>
__global__ void __launch_bounds__(256) gdec_vec_kernel(const __grid_constant__ GdecArgs g) {
  typedef typename std::conditional<sizeof(T) == 8, longlong2, int4>::type V;
  constexpr int VEC = 16 / sizeof(T);
  __shared__ __align__(16) T stage[8][32 * VEC * PW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T *st = stage[warp];
  const T *A = (const T *)g.in;
  T *R = (T *)g.out;
  const uint64_t mask = g.bits >= 64 ? ~0ull : ((1ull << g.bits) - 1);
  const int64_t nvec = g.n / VEC;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t v0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + warp) * 32; v0 < nvec; v0 += nwarps * 32) {
    const int64_t v = v0 + lane;
    const int valid = (int)(nvec - v0 < 32 ? nvec - v0 : 32);
    if (v < nvec) {
      T x[VEC], out[VEC * PW];
      *(V *)x = *(const V *)(A + v * VEC);
#pragma unroll
      for (int e = 0; e < VEC; ++e) {
#pragma unroll
        for (int d = 0; d < PW; ++d) out[e * PW + d] = (T)(int64_t)gdec_digit<T>((int64_t)x[e], d, g.bits, mask);
        const int64_t rest = (int64_t)gdec_digit<T>((int64_t)x[e], PW, g.bits, ~0ull);
        // the residual after PW steps, as the reference's `value > 0` sees it
        const int64_t resid = sizeof(T) == 4 ? (int64_t)(int32_t)(uint32_t)rest : rest;
        if (resid > 0) {
          unsigned long long slot = atomicAdd(&g.diag->count, 1ull);
          if (slot < (unsigned long long)kDiagRecords) {
            DiagRecord &rec = g.diag->rec[slot];
            int64_t rem = v * VEC + e;
            for (int i = g.a.ndim - 1; i >= 0; --i) {
              rec.coord[i] = rem % g.a.dims[i];
              rem /= g.a.dims[i];
            }
            rec.ndim = g.a.ndim;
            rec.kind = 1;
            rec.base_bits = g.bits;
            rec.power = g.power;
          }
        }
      }
#pragma unroll
      for (int k = 0; k < PW; ++k) *(V *)(st + (lane * PW + k) * VEC) = *(const V *)(out + k * VEC);
    }
    __syncwarp();
    for (int j = lane; j < valid * PW; j += 32) *(V *)(R + (v0 * PW + j) * VEC) = *(const V *)(st + j * VEC);
    __syncwarp();
  }
}

template <typename T>
__global__ void __launch_bounds__(256) gdec_kernel(const __grid_constant__ GdecArgs g) {
  const T *A = (const T *)g.in;
  T *R = (T *)g.out;
  const uint64_t mask = g.bits >= 64 ? ~0ull : ((1ull << g.bits) - 1);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < g.n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t ia, ir;
    if (g.dense) {
      ia = idx;
      ir = idx * (int64_t)g.power;
    } else {
      int64_t rem = idx;
      ia = 0;
      ir = 0;
      for (int i = g.a.ndim - 1; i >= 0; --i) {
        int64_t d = g.a.dims[i];
        int64_t c = rem % d;
        rem /= d;
        ia += c * g.a.strides[i];
        ir += c * g.r_strides[i];
      }
    }
    const int64_t ds = g.dense ? 1 : g.r_strides[g.a.ndim];
    int64_t value = (int64_t)A[ia];
    for (uint64_t d = 0; d < g.power; ++d) {
      uint64_t uv = (uint64_t)value;
      R[ir + (int64_t)d * ds] = (T)(int64_t)(uv & mask);
      uint64_t q = uv >> g.bits;
      value = sizeof(T) == 4 ? (int64_t)(int32_t)(uint32_t)q : (int64_t)q;
    }
    if (value > 0) {
      unsigned long long slot = atomicAdd(&g.diag->count, 1ull);
      if (slot < (unsigned long long)kDiagRecords) {
        DiagRecord &rec = g.diag->rec[slot];
        int64_t rem = idx;
        for (int i = g.a.ndim - 1; i >= 0; --i) {
          rec.coord[i] = rem % g.a.dims[i];
          rem /= g.a.dims[i];
        }
        rec.ndim = g.a.ndim;
        rec.kind = 1;
        rec.base_bits = g.bits;
        rec.power = g.power;
      }
    }
  }
}

static int g_decomposition(const heal_tensor *a, const heal_tensor *r, uint64_t power, uint64_t bits) {
  clear_error();
  HEAL_CHECK(check_desc(a, "a", true));
  HEAL_CHECK(check_desc(r, "result", true));
  HEAL_CHECK(ensure_init());
  if (a->dtype != r->dtype) return set_error(HEAL_ERR_INVALID_ARGUMENT, "all tensors must have the element type of result");
  // g_decomposition_impl.cpp:23-26
  bool ok = r->ndim == a->ndim + 1 && r->dims[r->ndim - 1] == (int64_t)power;
  for (int i = 0; ok && i < a->ndim; ++i) ok = a->dims[i] == r->dims[i];
  if (!ok) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Output must have shape a.shape + [power]");
  if (bits >= 64) return set_error(HEAL_ERR_INVALID_ARGUMENT, "base_bits must be below 64");
  const int64_t n = numel(*a);
  if (n == 0) return HEAL_OK;
  heal_tensor A = *a;
  void *oa = nullptr;
  int rc = HEAL_OK;
  if (overlaps(A, *r)) rc = materialize(A, &A, &oa);
  if (!rc) {
    GdecArgs g;
    memset(&g, 0, sizeof g);
    g.a = make_view(A);
    for (int i = 0; i < r->ndim; ++i) g.r_strides[i] = r->strides[i];
    g.in = A.data;
    g.out = r->data;
    g.n = n;
    g.power = power;
    g.bits = bits;
    g.dense = dense_rowmajor(A) && dense_rowmajor(*r);
    g.diag = diag_device();
    const int vec = 16 / elem_size(r->dtype);
    const bool vec_ok = g.dense && power >= 1 && power <= 8 && bits < 64 && n % vec == 0 &&
                        (r->dtype == HEAL_INT64 || bits <= 32) &&
                        (uintptr_t)A.data % 16 == 0 && (uintptr_t)r->data % 16 == 0;
    if (vec_ok) {
      const int grid = grid_for(n / vec, 256, 8);
#define HEAL_GDEC_CASE(PW)                                                                 \
  case PW:                                                                                 \
    if (r->dtype == HEAL_INT32)                                                            \
      gdec_vec_kernel<int32_t, PW><<<grid, 256, 0, stream()>>>(g);                         \
    else                                                                                   \
      gdec_vec_kernel<int64_t, PW><<<grid, 256, 0, stream()>>>(g);                         \
    break;
      switch ((int)power) {
        HEAL_GDEC_CASE(1)
        HEAL_GDEC_CASE(2)
        HEAL_GDEC_CASE(3)
        HEAL_GDEC_CASE(4)
        HEAL_GDEC_CASE(5)
        HEAL_GDEC_CASE(6)
        HEAL_GDEC_CASE(7)
        HEAL_GDEC_CASE(8)
      }
#undef HEAL_GDEC_CASE
    } else if (r->dtype == HEAL_INT32) {
      gdec_kernel<int32_t><<<grid_for(n, 256, 8), 256, 0, stream()>>>(g);
    } else {
      gdec_kernel<int64_t><<<grid_for(n, 256, 8), 256, 0, stream()>>>(g);
    }
    rc = check_launch("g_decomposition");
  }
  scratch_free(oa);
  if (!rc) mark_written(r->data);
  return rc;
}

// ================================================================ permute
struct PermuteArgs {
  View r, a;
  int ew, pa;
  int64_t m;
  int64_t ps0, ps1;  // perms strides
  const void *src, *perms;
  int perms_dtype;
  void *out;
  int64_t n;
  // row-major fast path: idx = (pre * m + pm) * post + inner
  int dense;
  int64_t post;
  int64_t ew_div, ew_mod;  // ew coordinate = (x / ew_div) % l with x = pre or inner
  int ew_in_post;
  int fast;                 // n below 2^32: 32-bit divisions below
  FastDiv f_post, f_m, f_ewdiv, f_ewmod;
  FastDims fd;              // general path: 32-bit decomposition of r's coordinates
};

__device__ __forceinline__ int64_t perm_at(const PermuteArgs &g, int64_t e, int64_t pm) {
  return g.perms_dtype == HEAL_INT32 ? (int64_t)((const int32_t *)g.perms)[e * g.ps0 + pm * g.ps1]
                                     : ((const int64_t *)g.perms)[e * g.ps0 + pm * g.ps1];
}

// row-major a and result: idx = (pre * m + pm) * post + inner, in units of T
// (an element, or a 16-byte vector of a row when rows are whole vectors)
template <typename T>
__global__ void __launch_bounds__(256) permute_dense_kernel(const __grid_constant__ PermuteArgs g) {
  const T *A = (const T *)g.src;
  T *R = (T *)g.out;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < g.n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t inner, pm, pre, e;
    if (g.fast) {
      const uint32_t x = (uint32_t)idx;
      const uint32_t rest = fastdiv(x, g.f_post);
      inner = x - rest * (uint32_t)g.post;
      const uint32_t pr = fastdiv(rest, g.f_m);
      pm = rest - pr * (uint32_t)g.m;
      pre = pr;
      const uint32_t y = fastdiv((uint32_t)(g.ew_in_post ? inner : pre), g.f_ewdiv);
      e = y - fastdiv(y, g.f_ewmod) * (uint32_t)g.ew_mod;
    } else {
      inner = idx % g.post;
      const int64_t rest = idx / g.post;
      pm = rest % g.m;
      pre = rest / g.m;
      e = ((g.ew_in_post ? inner : pre) / g.ew_div) % g.ew_mod;
    }
    R[idx] = A[(pre * g.m + perm_at(g, e, pm)) * g.post + inner];
  }
}

// any strides (axes merged on the host except the two it reads); kGenU
// elements per thread per iteration, loads issued together; Off is int32_t
// when every offset of a and the result fits 32 bits
constexpr int kGenU = 4;

template <typename T, typename Off>
__global__ void __launch_bounds__(256) permute_general_kernel(const __grid_constant__ PermuteArgs g) {
  const T *A = (const T *)g.src;
  T *R = (T *)g.out;
  const int64_t step = (int64_t)gridDim.x * blockDim.x * kGenU;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x * kGenU + threadIdx.x; base < g.n; base += step) {
    Off src[kGenU], dst[kGenU];
#pragma unroll
    for (int u = 0; u < kGenU; ++u) {
      const int64_t idx = base + (int64_t)u * blockDim.x;
      int64_t e = 0, pm = 0;
      Off s = 0, d = 0;
      if (idx < g.n) {
        if (g.fd.fast) {
          uint32_t rem = (uint32_t)idx;
#pragma unroll
          for (int k = 0; k < HEAL_MAX_DIMS; ++k) {  // unrolled: per-axis parameters at fixed offsets
            const int i = HEAL_MAX_DIMS - 1 - k;
            if (i >= g.r.ndim) continue;
            const uint32_t q = fastdiv(rem, g.fd.fd[i]);
            const uint32_t c = rem - q * (uint32_t)g.r.dims[i];
            rem = q;
            if (i == g.ew) e = c;
            if (i == g.pa) pm = c;
            else s += (Off)c * (Off)g.a.strides[i];
            d += (Off)c * (Off)g.r.strides[i];
          }
        } else {
          int64_t rem = idx;
          for (int i = g.r.ndim - 1; i >= 0; --i) {
            const int64_t c = rem % g.r.dims[i];
            rem /= g.r.dims[i];
            if (i == g.ew) e = c;
            if (i == g.pa) pm = c;
            else s += (Off)(c * g.a.strides[i]);
            d += (Off)(c * g.r.strides[i]);
          }
        }
        s += (Off)perm_at(g, e, pm) * (Off)g.a.strides[g.pa];
      }
      src[u] = s;
      dst[u] = d;
    }
    T v[kGenU];
#pragma unroll
    for (int u = 0; u < kGenU; ++u)
      if (base + (int64_t)u * blockDim.x < g.n) v[u] = A[src[u]];
#pragma unroll
    for (int u = 0; u < kGenU; ++u)
      if (base + (int64_t)u * blockDim.x < g.n) R[dst[u]] = v[u];
  }
}

static int permute(const heal_tensor *a, const heal_tensor *perms, const heal_tensor *r, int64_t ew, int64_t pa) {
  clear_error();
  HEAL_CHECK(check_desc(a, "a", true));
  HEAL_CHECK(check_desc(perms, "perms", true));
  HEAL_CHECK(check_desc(r, "result", true));
  HEAL_CHECK(ensure_init());
  if (a->dtype != r->dtype) return set_error(HEAL_ERR_INVALID_ARGUMENT, "all tensors must have the element type of result");
  // permute_impl.cpp:19-35
  const int nd = a->ndim;
  if (!same_dims(*a, *r)) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Result shape must match input shape.");
  if (ew < 0 || ew >= nd || pa < 0 || pa >= nd) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Axis out of bounds.");
  if (ew == pa) return set_error(HEAL_ERR_INVALID_ARGUMENT, "elementwise_axis and perm_axis must be different.");
  const int64_t l = a->dims[ew], m = a->dims[pa];
  if (perms->ndim != 2 || perms->dims[0] != l || perms->dims[1] != m)
    return set_error(HEAL_ERR_INVALID_ARGUMENT,
                     "Perms must have shape [l, m] where l and m match a.shape at elementwise and perm axes.");
  const int64_t n = numel(*a);
  if (n == 0) return HEAL_OK;
  bool valid = false;
  HEAL_CHECK(perms_valid(*perms, m, &valid));
  if (!valid) return set_error(HEAL_ERR_OUT_OF_RANGE, "Permutation index out of bounds.");
  heal_tensor A = *a, PR = *perms;
  void *oa = nullptr, *op = nullptr;
  int rc = HEAL_OK;
  if (overlaps(A, *r)) rc = materialize(A, &A, &oa);
  if (!rc && overlaps(PR, *r)) rc = materialize(PR, &PR, &op);
  if (!rc) {
    PermuteArgs g;
    memset(&g, 0, sizeof g);
    g.r = make_view(*r);
    g.a = make_view(A);
    g.ew = (int)ew;
    g.pa = (int)pa;
    g.m = m;
    g.ps0 = PR.strides[0];
    g.ps1 = PR.strides[1];
    g.src = A.data;
    g.perms = PR.data;
    g.perms_dtype = PR.dtype;
    g.out = r->data;
    g.n = n;
    g.dense = dense_rowmajor(A) && dense_rowmajor(*r);
    if (g.dense) {
      int64_t post = 1;
      for (int i = (int)pa + 1; i < nd; ++i) post *= a->dims[i];
      g.post = post;
      g.ew_in_post = ew > pa;
      int64_t div = 1;
      if (ew > pa) {
        for (int i = (int)ew + 1; i < nd; ++i) div *= a->dims[i];
      } else {
        for (int i = (int)ew + 1; i < (int)pa; ++i) div *= a->dims[i];
      }
      g.ew_div = div;
      g.ew_mod = l;
      g.fast = n < (int64_t)UINT32_MAX && post < (int64_t)UINT32_MAX && m < (int64_t)UINT32_MAX &&
               div < (int64_t)UINT32_MAX && l < (int64_t)UINT32_MAX && post > 0 && m > 0 && l > 0;
      if (g.fast) {
        g.f_post = fastdiv_make((uint32_t)post);
        g.f_m = fastdiv_make((uint32_t)m);
        g.f_ewdiv = fastdiv_make((uint32_t)div);
        g.f_ewmod = fastdiv_make((uint32_t)l);
      }
    }
    const int vec = 16 / elem_size(r->dtype);
    bool gen_vec = false, off32 = false;
    if (!g.dense) {
      // general path: merge the axes other than the two whose coordinates it reads
      View *vs[2] = {&g.r, &g.a};
      int map[HEAL_MAX_DIMS];
      coalesce_views(vs, 2, (1u << ew) | (1u << pa), map);
      g.ew = map[ew];
      g.pa = map[pa];
      // an innermost axis that is neither read axis and is contiguous in
      // aligned 16-byte vectors in both a and the result (a ciphertext's
      // limbs under a broadcast or transposed stack) moves as vectors: the
      // views are rescaled to units of one vector
      const int in = g.r.ndim - 1;
      off32 = view_off32(g.r) && view_off32(g.a);
      gen_vec = in != g.ew && in != g.pa && inner_vectors(g.r, vec, r->data, elem_size(r->dtype)) &&
                inner_vectors(g.a, vec, A.data, elem_size(r->dtype));
      if (gen_vec) {
        for (View *v : vs) {
          v->dims[in] /= vec;
          for (int i = 0; i < in; ++i) v->strides[i] /= vec;
        }
        g.n = n / vec;
      }
      make_fast_dims(g.r, g.n, &g.fd);
      off32 = off32 && g.fd.fast;
    }
    // rows of 16-byte vectors: the gathered blocks (`post` elements) are
    // whole aligned vectors and a vector never straddles two elementwise
    // coordinates; the same kernel then moves one vector per index
    const bool rows = g.dense && g.fast && g.post % vec == 0 && (!g.ew_in_post || g.ew_div % vec == 0) &&
                      (uintptr_t)A.data % 16 == 0 && (uintptr_t)r->data % 16 == 0;
    if (rows) {
      g.post /= vec;
      if (g.ew_in_post) g.ew_div /= vec;
      g.n = n / vec;
      g.f_post = fastdiv_make((uint32_t)g.post);
      g.f_ewdiv = fastdiv_make((uint32_t)g.ew_div);
      permute_dense_kernel<uint4><<<grid_for(g.n, 256, 8), 256, 0, stream()>>>(g);
    } else if (g.dense) {
      if (r->dtype == HEAL_INT32)
        permute_dense_kernel<int32_t><<<grid_for(n, 256, 8), 256, 0, stream()>>>(g);
      else
        permute_dense_kernel<int64_t><<<grid_for(n, 256, 8), 256, 0, stream()>>>(g);
    } else {
      const int grid = grid_for((g.n + kGenU - 1) / kGenU, 256, 8);
      auto go = [&](auto t_tag) {
        typedef decltype(t_tag) TT;
        if (off32)
          permute_general_kernel<TT, int32_t><<<grid, 256, 0, stream()>>>(g);
        else
          permute_general_kernel<TT, int64_t><<<grid, 256, 0, stream()>>>(g);
      };
      if (gen_vec) go(uint4());
      else if (r->dtype == HEAL_INT32) go(int32_t());
      else go(int64_t());
    }
    rc = check_launch("permute");
  }
  scratch_free(oa);
  scratch_free(op);
  if (!rc) mark_written(r->data);
  return rc;
}

}  // namespace heal

using namespace heal;

extern "C" {

int heal_axis_modsum(const heal_tensor *a, const heal_tensor *p, const heal_tensor *result, int64_t axis) {
  return axis_modsum(a, p, result, axis);
}

int heal_g_decomposition(const heal_tensor *a, const heal_tensor *result, uint64_t power, uint64_t base_bits) {
  return g_decomposition(a, result, power, base_bits);
}

int heal_permute(const heal_tensor *a, const heal_tensor *perms, const heal_tensor *result, int64_t elementwise_axis,
                 int64_t perm_axis) {
  return permute(a, perms, result, elementwise_axis, perm_axis);
}

}  // extern "C"
