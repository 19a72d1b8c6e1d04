// Randomised check of heal_view.h: for views of one coordinate space, the
// offsets (and the coordinates of kept axes) computed through the merged
// views, by 64-bit and by FastDiv decomposition, equal those of the
// original views for every linear index.  Prints "ok <cases>" or the first
// mismatch.
#include <cstdio>
#include <random>

#include "../../heal_gb300/csrc/heal_view.h"
using namespace heal;

int main() {
  std::mt19937_64 rng(12345);
  auto pick = [&](int lo, int hi) { return (int)(lo + rng() % (uint64_t)(hi - lo + 1)); };
  int cases = 0;
  for (int it = 0; it < 20000; ++it) {
    const int nd = pick(0, 7), nv = pick(1, 5);
    View v[5];
    int64_t dims[HEAL_MAX_DIMS];
    for (int i = 0; i < nd; ++i) dims[i] = pick(0, 9) < 3 ? 1 : pick(2, 5);
    for (int k = 0; k < nv; ++k) {
      v[k].ndim = nd;
      // strides: dense row-major, broadcast (0), permuted dense, or random
      const int kind = pick(0, 3);
      int64_t s = 1;
      for (int i = nd - 1; i >= 0; --i) {
        v[k].dims[i] = dims[i];
        if (kind == 0) v[k].strides[i] = s;
        else if (kind == 1) v[k].strides[i] = pick(0, 1) ? 0 : s;
        else if (kind == 2) v[k].strides[i] = s * pick(1, 3);
        else v[k].strides[i] = pick(0, 40);
        s *= dims[i];
      }
      for (int i = nd; i < HEAL_MAX_DIMS; ++i) v[k].dims[i] = 1, v[k].strides[i] = 0;
    }
    unsigned keep = 0;
    for (int i = 0; i < nd; ++i)
      if (pick(0, 5) == 0) keep |= 1u << i;
    View w[5];
    View *ptr[5];
    for (int k = 0; k < nv; ++k) w[k] = v[k], ptr[k] = &w[k];
    int map[HEAL_MAX_DIMS];
    coalesce_views(ptr, nv, keep, map);
    int64_t n = 1;
    for (int i = 0; i < nd; ++i) n *= dims[i];
    int64_t m = 1;
    for (int j = 0; j < w[0].ndim; ++j) m *= w[0].dims[j];
    if (m != n) {
      printf("element count %lld != %lld (case %d)\n", (long long)m, (long long)n, it);
      return 1;
    }
    FastDims fd;
    make_fast_dims(w[0], n, &fd);
    if (!fd.fast) {
      printf("fast path refused (case %d)\n", it);
      return 1;
    }
    for (int64_t idx = 0; idx < n; ++idx) {
      int64_t c[HEAL_MAX_DIMS], rem = idx;
      for (int i = nd - 1; i >= 0; --i) c[i] = rem % dims[i], rem /= dims[i];
      int64_t c2[HEAL_MAX_DIMS], c3[HEAL_MAX_DIMS];
      rem = idx;
      uint32_t r32 = (uint32_t)idx;
      for (int j = w[0].ndim - 1; j >= 0; --j) {
        c2[j] = rem % w[0].dims[j], rem /= w[0].dims[j];
        const uint32_t q = fastdiv(r32, fd.fd[j]);
        c3[j] = r32 - q * (uint32_t)w[0].dims[j];
        r32 = q;
      }
      for (int i = 0; i < nd; ++i)
        if (((keep >> i) & 1u) && (map[i] < 0 || c2[map[i]] != c[i] || c3[map[i]] != c[i])) {
          printf("kept axis %d coordinate differs (case %d)\n", i, it);
          return 1;
        }
      for (int k = 0; k < nv; ++k) {
        int64_t o = 0, o2 = 0, o3 = 0;
        for (int i = 0; i < nd; ++i) o += c[i] * v[k].strides[i];
        for (int j = 0; j < w[k].ndim; ++j) o2 += c2[j] * w[k].strides[j], o3 += c3[j] * w[k].strides[j];
        if (o != o2 || o != o3) {
          printf("offset of view %d differs at index %lld (case %d)\n", k, (long long)idx, it);
          return 1;
        }
      }
    }
    ++cases;
  }
  // inner_vectors: contiguous innermost axis, whole vectors, aligned starts
  {
    View a;
    memset(&a, 0, sizeof a);
    a.ndim = 3;
    a.dims[0] = 4, a.dims[1] = 6, a.dims[2] = 8;
    a.strides[0] = 48, a.strides[1] = 8, a.strides[2] = 1;
    alignas(16) static int64_t buf[512];
    const bool want[6] = {true, false, false, false, false, true};
    bool got[6];
    got[0] = inner_vectors(a, 2, buf, 8);
    got[1] = inner_vectors(a, 2, buf + 1, 8);  // start off the 16-byte grid
    View b = a;
    b.strides[1] = 9;                           // a row start off the grid
    got[2] = inner_vectors(b, 2, buf, 8);
    b = a;
    b.dims[2] = 7;                              // a partial vector per row
    got[3] = inner_vectors(b, 2, buf, 8);
    b = a;
    b.strides[2] = 2;                           // a strided innermost axis
    got[4] = inner_vectors(b, 2, buf, 8);
    b = a;
    b.strides[0] = 0;                           // broadcast outer axis
    got[5] = inner_vectors(b, 2, buf, 8);
    for (int i = 0; i < 6; ++i)
      if (got[i] != want[i]) {
        printf("inner_vectors case %d: got %d\n", i, (int)got[i]);
        return 1;
      }
  }
  printf("ok %d\n", cases);
  return 0;
}
