// heal_view.h — strided views of HEAL tensors in kernel arguments, and the
// host-side merging of their axes.  Plain C++ (no CUDA) so host tests can
// compile it.
#pragma once
#include <stdint.h>
#include <string.h>

#include "../../include/heal_gb300.h"
#include "heal_arith.h"

namespace heal {

struct View {
  int64_t dims[HEAL_MAX_DIMS];
  int64_t strides[HEAL_MAX_DIMS];
  int32_t ndim;
};

inline View make_view(const heal_tensor &t) {
  View v;
  v.ndim = t.ndim;
  for (int i = 0; i < HEAL_MAX_DIMS; ++i) {
    v.dims[i] = i < t.ndim ? t.dims[i] : 1;
    v.strides[i] = i < t.ndim ? t.strides[i] : 0;
  }
  return v;
}

// Views of one coordinate space (same ndim and dims), merged where they
// allow: an axis joins its inner neighbour when every view's stride on it
// equals the neighbour's stride times the neighbour's length, and size-1
// axes are dropped.  Axes in `keep` (bit i = axis i), whose coordinates a
// kernel reads, stay whole and are never dropped or merged.  map (optional)
// receives the new index of every old axis (-1 if dropped).  At least one
// axis remains.  At most 8 views; more are left as they are.
inline void coalesce_views(View *const *views, int nviews, unsigned keep, int *map) {
  if (nviews < 1 || nviews > 8) return;
  const int nd = views[0]->ndim;
  int64_t dims[HEAL_MAX_DIMS], st[8][HEAL_MAX_DIMS];
  bool kept[HEAL_MAX_DIMS];
  int grp[HEAL_MAX_DIMS];
  int ng = 0;  // groups, innermost first
  for (int i = nd - 1; i >= 0; --i) {
    const bool k = (keep >> i) & 1u;
    const int64_t d = views[0]->dims[i];
    if (d == 1 && !k) {
      grp[i] = -1;
      continue;
    }
    if (ng > 0 && !k && !kept[ng - 1]) {
      bool lin = true;
      for (int v = 0; v < nviews; ++v) lin = lin && views[v]->strides[i] == st[v][ng - 1] * dims[ng - 1];
      if (lin) {
        dims[ng - 1] *= d;
        grp[i] = ng - 1;
        continue;
      }
    }
    dims[ng] = d;
    kept[ng] = k;
    for (int v = 0; v < nviews; ++v) st[v][ng] = views[v]->strides[i];
    grp[i] = ng++;
  }
  if (ng == 0) {  // every axis had length 1
    dims[0] = 1;
    for (int v = 0; v < nviews; ++v) st[v][0] = 0;
    ng = 1;
  }
  for (int v = 0; v < nviews; ++v) {
    View &w = *views[v];
    w.ndim = ng;
    for (int j = 0; j < HEAL_MAX_DIMS; ++j) {
      w.dims[j] = j < ng ? dims[ng - 1 - j] : 1;
      w.strides[j] = j < ng ? st[v][ng - 1 - j] : 0;
    }
  }
  if (map)
    for (int i = 0; i < nd; ++i) map[i] = grp[i] < 0 ? -1 : ng - 1 - grp[i];
}

// Divisions by every dim of a coordinate space, for 32-bit index
// decomposition when its element count and dims are below 2^32.
// True when a kernel may move `v`'s innermost axis in vectors of `vec`
// elements of `elem` bytes from `base`: the axis is contiguous, its length is
// a multiple of vec, and every vector starts on a vec * elem byte boundary
// (the base aligned, every other stride a multiple of vec).
inline bool inner_vectors(const View &v, int vec, const void *base, size_t elem) {
  if (v.ndim < 1 || vec < 1) return false;
  const int in = v.ndim - 1;
  if (v.strides[in] != 1 || v.dims[in] % vec) return false;
  if ((uintptr_t)base % ((uintptr_t)vec * elem)) return false;
  for (int i = 0; i < in; ++i)
    if (v.strides[i] % vec) return false;
  return true;
}

// True when every offset of `v` fits a signed 32-bit integer: strides
// non-negative and the largest offset below 2^31 - 1.
inline bool view_off32(const View &v) {
  int64_t span = 0;
  for (int i = 0; i < v.ndim; ++i) {
    if (v.strides[i] < 0 || v.dims[i] < 1) return false;
    if (v.strides[i] && (v.dims[i] - 1) > (INT32_MAX - 1 - span) / v.strides[i]) return false;
    span += (v.dims[i] - 1) * v.strides[i];
  }
  return span < INT32_MAX;
}

struct FastDims {
  int fast;
  FastDiv fd[HEAL_MAX_DIMS];
};

inline void make_fast_dims(const View &v, int64_t n, FastDims *out) {
  memset(out, 0, sizeof *out);
  bool ok = n < (int64_t)UINT32_MAX;
  for (int i = 0; i < v.ndim && ok; ++i) ok = v.dims[i] >= 1 && v.dims[i] < (int64_t)UINT32_MAX;
  out->fast = ok;
  if (ok)
    for (int i = 0; i < v.ndim; ++i) out->fd[i] = fastdiv_make((uint32_t)v.dims[i]);
}

}  // namespace heal
