// heal_runtime.cu — library state, HBM allocation, host<->device copies,
// stride-only metadata edits, the strided gather, diagnostics and the caches
// of tables derived from constant tensors (moduli, twiddles, permutations).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "heal_internal.h"

namespace heal {

// ================================================================== errors
static thread_local std::string g_last_error;
// Counts API calls: a table derived from memory the backend did not allocate
// is reused only within the call that built it.
static std::atomic<uint64_t> g_epoch{1};

int set_error(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}
void clear_error() {
  g_last_error.clear();
  g_epoch.fetch_add(1, std::memory_order_relaxed);
}

int cuda_fail(cudaError_t e, const char *what) {
  int code = (e == cudaErrorMemoryAllocation) ? HEAL_ERR_BAD_ALLOC : HEAL_ERR_CUDA;
  return set_error(code, std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

// ================================================================= runtime
struct Runtime {
  bool ready = false;
  bool capturing = false;
  uint64_t capture_start = 0;  // launch count when the capture began
  cudaStream_t origin = nullptr;         // the stream the capture began on
  std::vector<cudaStream_t> branches;    // branch streams, kept for reuse
  int forked = 0;                        // branches joined to this capture
  cudaEvent_t join = nullptr;
  int device = -1;
  int sms = 0;
  cudaStream_t own = nullptr;
  cudaStream_t cur = nullptr;
  Diag *diag = nullptr;
  std::atomic<uint64_t> launches{0};
};
static Runtime g_rt;
static std::recursive_mutex g_mu;

struct Alloc {
  size_t bytes;
  uint64_t gen;
};
static std::map<uintptr_t, Alloc> g_allocs;
static std::atomic<uint64_t> g_gen{1};

static int init_device(int device) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  if (g_rt.ready) {
    if (device != g_rt.device) return set_error(HEAL_ERR_RUNTIME, "heal_init: the backend is bound to another device");
    return HEAL_OK;
  }
  HEAL_TRY_CUDA(cudaSetDevice(device));
  HEAL_TRY_CUDA(cudaDeviceGetAttribute(&g_rt.sms, cudaDevAttrMultiProcessorCount, device));
  HEAL_TRY_CUDA(cudaStreamCreateWithFlags(&g_rt.own, cudaStreamNonBlocking));
  cudaMemPool_t pool;
  HEAL_TRY_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t keep = UINT64_MAX;  // keep freed blocks cached in the pool
  HEAL_TRY_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  HEAL_TRY_CUDA(cudaMalloc(&g_rt.diag, sizeof(Diag)));
  HEAL_TRY_CUDA(cudaMemset(g_rt.diag, 0, sizeof(Diag)));
  g_rt.cur = g_rt.own;
  g_rt.device = device;
  g_rt.ready = true;
  return HEAL_OK;
}

int ensure_init() {
  if (g_rt.ready) return HEAL_OK;
  int dev = 0;
  HEAL_TRY_CUDA(cudaGetDevice(&dev));
  return init_device(dev);
}

cudaStream_t stream() { return g_rt.cur; }

// the sample implementation's wraparound instead of exact results (heal_set_reference_compat)
std::atomic<bool> g_reference_compat{false};
bool reference_compat() { return g_reference_compat.load(); }
int device_sm_count() { return g_rt.sms; }
void note_launch(int n) { g_rt.launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }
Diag *diag_device() { return g_rt.diag; }

int check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  note_launch();
  return HEAL_OK;
}

bool capturing() { return g_rt.capturing; }

int scratch_alloc(size_t bytes, void **out) {
  *out = nullptr;
  if (bytes == 0) return HEAL_OK;
  HEAL_TRY_CUDA(cudaMallocAsync(out, bytes, stream()));
  return HEAL_OK;
}
void scratch_free(void *p) {
  if (p) cudaFreeAsync(p, stream());
}

static std::map<uintptr_t, Alloc>::iterator find_alloc(const void *p) {
  uintptr_t a = (uintptr_t)p;
  auto it = g_allocs.upper_bound(a);
  if (it == g_allocs.begin()) return g_allocs.end();
  --it;
  if (a >= it->first && a < it->first + std::max<size_t>(it->second.bytes, 1)) return it;
  return g_allocs.end();
}

uint64_t generation_of(const void *p) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  auto it = find_alloc(p);
  return it == g_allocs.end() ? 0 : it->second.gen;
}

void mark_written(const void *p) {
  if (!p) return;
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  auto it = find_alloc(p);
  if (it != g_allocs.end()) it->second.gen = g_gen.fetch_add(1);
}

// ============================================================ diagnostics
// Prints the warnings recorded on the device since the last flush; returns
// HEAL_ERR_RUNTIME when a heal_keyswitch_batch dependency wait ran out.
static int flush_diag() {
  if (!g_rt.ready) return HEAL_OK;
  Diag h;
  if (cudaMemcpyAsync(&h, g_rt.diag, sizeof(Diag), cudaMemcpyDeviceToHost, stream()) != cudaSuccess ||
      cudaStreamSynchronize(stream()) != cudaSuccess)
    return HEAL_OK;
  if (h.count == 0 && h.zero_mod == 0 && h.wait_timeouts == 0) return HEAL_OK;
  unsigned long long shown = std::min<unsigned long long>(h.count, kDiagRecords);
  for (unsigned long long i = 0; i < shown; ++i) {
    const DiagRecord &r = h.rec[i];
    if (r.kind != 1) continue;
    std::string c;
    for (int d = 0; d < r.ndim; ++d) c += std::to_string(r.coord[d]) + " ";
    fprintf(stderr, "Warning: value at %sexceeds capacity with base_bits=%llu and power=%llu\n", c.c_str(),
            (unsigned long long)r.base_bits, (unsigned long long)r.power);
  }
  if (h.count > shown)
    fprintf(stderr, "Warning: %llu more values exceeded the decomposition capacity\n", h.count - shown);
  if (h.zero_mod)
    fprintf(stderr, "Warning: %llu elements had a zero modulus or divisor; their results were set to 0\n",
            h.zero_mod);
  cudaMemsetAsync(g_rt.diag, 0, sizeof(Diag), stream());
  cudaStreamSynchronize(stream());
  if (h.wait_timeouts)
    return set_error(HEAL_ERR_RUNTIME, "heal_keyswitch_batch: " + std::to_string(h.wait_timeouts) +
                                           " dependency waits ran out; the results of that batch are incomplete");
  return HEAL_OK;
}

// ================================================================ helpers
int64_t numel(const heal_tensor &t) {
  int64_t n = 1;
  for (int i = 0; i < t.ndim; ++i) n *= t.dims[i];
  return n;
}
bool same_dims(const heal_tensor &a, const heal_tensor &b) {
  if (a.ndim != b.ndim) return false;
  for (int i = 0; i < a.ndim; ++i)
    if (a.dims[i] != b.dims[i]) return false;
  return true;
}
int elem_size(int dtype) { return dtype == HEAL_INT32 ? 4 : 8; }

int check_desc(const heal_tensor *t, const char *label, bool integer_only) {
  if (!t) return set_error(HEAL_ERR_INVALID_ARGUMENT, std::string(label) + " pointer must not be null.");
  if (t->ndim < 0 || t->ndim > HEAL_MAX_DIMS)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, std::string(label) + ": unsupported number of dimensions");
  if (t->dtype != HEAL_INT32 && t->dtype != HEAL_INT64 && (integer_only || t->dtype != HEAL_FLOAT64))
    return set_error(HEAL_ERR_INVALID_ARGUMENT, std::string(label) + ": unsupported element type");
  for (int i = 0; i < t->ndim; ++i)
    if (t->dims[i] < 0) return set_error(HEAL_ERR_INVALID_ARGUMENT, std::string(label) + ": negative dimension");
  if (numel(*t) > 0 && !t->data)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, std::string(label) + ": null data for a non-empty tensor");
  return HEAL_OK;
}

void byte_range(const heal_tensor &t, uintptr_t *lo, uintptr_t *hi) {
  *lo = *hi = 0;
  if (numel(t) == 0) return;
  int64_t mn = 0, mx = 0;
  for (int i = 0; i < t.ndim; ++i) {
    int64_t e = (t.dims[i] - 1) * t.strides[i];
    if (e < 0) mn += e; else mx += e;
  }
  int es = elem_size(t.dtype);
  *lo = (uintptr_t)t.data + mn * es;
  *hi = (uintptr_t)t.data + (mx + 1) * es;
}

bool overlaps(const heal_tensor &a, const heal_tensor &b) {
  uintptr_t al, ah, bl, bh;
  byte_range(a, &al, &ah);
  byte_range(b, &bl, &bh);
  if (al == ah || bl == bh) return false;
  return al < bh && bl < ah;
}

bool identical_view(const heal_tensor &a, const heal_tensor &b) {
  if (a.data != b.data || a.dtype != b.dtype || !same_dims(a, b)) return false;
  for (int i = 0; i < a.ndim; ++i)
    if (a.dims[i] > 1 && a.strides[i] != b.strides[i]) return false;
  return true;
}

// ========================================================= strided gather
struct CopyArgs {
  View src, dst;
  FastDims fd;
  int64_t n;
  const char *s;
  char *d;
};

// kCopyU elements per thread per iteration, loads issued together
constexpr int kCopyU = 4;

template <typename W>
__global__ void __launch_bounds__(256) copy_strided_kernel(const __grid_constant__ CopyArgs a) {
  const W *src = (const W *)a.s;
  W *dst = (W *)a.d;
  const int64_t step = (int64_t)gridDim.x * blockDim.x * kCopyU;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x * kCopyU + threadIdx.x; base < a.n; base += step) {
    int64_t so[kCopyU], dofs[kCopyU];
#pragma unroll
    for (int u = 0; u < kCopyU; ++u) {
      const int64_t idx = base + (int64_t)u * blockDim.x;
      so[u] = dofs[u] = 0;
      if (idx >= a.n) continue;
      if (a.fd.fast) {
        uint32_t rem = (uint32_t)idx;
#pragma unroll
        for (int k = 0; k < HEAL_MAX_DIMS; ++k) {  // unrolled: per-axis parameters at fixed offsets
          const int i = HEAL_MAX_DIMS - 1 - k;
          if (i >= a.dst.ndim) continue;
          const uint32_t q = fastdiv(rem, a.fd.fd[i]);
          const int64_t c = rem - q * (uint32_t)a.dst.dims[i];
          rem = q;
          so[u] += c * a.src.strides[i];
          dofs[u] += c * a.dst.strides[i];
        }
      } else {
        int64_t rem = idx;
        for (int i = a.dst.ndim - 1; i >= 0; --i) {
          const int64_t d = a.dst.dims[i];
          const int64_t c = rem % d;
          rem /= d;
          so[u] += c * a.src.strides[i];
          dofs[u] += c * a.dst.strides[i];
        }
      }
    }
    W v[kCopyU];
#pragma unroll
    for (int u = 0; u < kCopyU; ++u)
      if (base + (int64_t)u * blockDim.x < a.n) v[u] = src[so[u]];
#pragma unroll
    for (int u = 0; u < kCopyU; ++u)
      if (base + (int64_t)u * blockDim.x < a.n) dst[dofs[u]] = v[u];
  }
}

static int grid_for(int64_t n, int threads) {
  int64_t want = (n + threads - 1) / threads;
  int64_t cap = (int64_t)std::max(device_sm_count(), 1) * 16;
  return (int)std::max<int64_t>(1, std::min(want, cap));
}

int copy_strided_impl(const heal_tensor &src, const heal_tensor &dst) {
  int64_t n = numel(dst);
  if (n == 0) return HEAL_OK;
  CopyArgs a;
  a.src = make_view(src);
  a.dst = make_view(dst);
  View *vs[2] = {&a.src, &a.dst};
  coalesce_views(vs, 2, 0u, nullptr);
  make_fast_dims(a.dst, n, &a.fd);
  a.n = n;
  a.s = (const char *)src.data;
  a.d = (char *)dst.data;
  // 16-byte vectors when both innermost axes are unit-stride rows of whole,
  // aligned vectors: the same kernel then moves one vector per index
  const int es = elem_size(src.dtype), vec = 16 / es;
  const int in = a.dst.ndim - 1;
  bool v16 = ((uintptr_t)a.s % 16 == 0) && ((uintptr_t)a.d % 16 == 0) && a.src.strides[in] == 1 &&
             a.dst.strides[in] == 1 && a.dst.dims[in] % vec == 0;
  for (int i = 0; i < in && v16; ++i) v16 = a.src.strides[i] % vec == 0 && a.dst.strides[i] % vec == 0;
  if (v16) {
    a.dst.dims[in] /= vec;
    a.src.dims[in] = a.dst.dims[in];
    for (int i = 0; i < in; ++i) {
      a.src.strides[i] /= vec;
      a.dst.strides[i] /= vec;
    }
    a.n = n / vec;
    make_fast_dims(a.dst, a.n, &a.fd);
    copy_strided_kernel<uint4><<<grid_for((a.n + kCopyU - 1) / kCopyU, 256), 256, 0, stream()>>>(a);
  } else {
    const int64_t work = (n + kCopyU - 1) / kCopyU;
    if (es == 4)
      copy_strided_kernel<uint32_t><<<grid_for(work, 256), 256, 0, stream()>>>(a);
    else
      copy_strided_kernel<uint64_t><<<grid_for(work, 256), 256, 0, stream()>>>(a);
  }
  HEAL_CHECK(check_launch("copy_strided"));
  mark_written(dst.data);
  return HEAL_OK;
}

int materialize(const heal_tensor &t_in, heal_tensor *out, void **owned) {
  const heal_tensor t = t_in;  // `out` may alias `t_in`
  *out = t;
  *owned = nullptr;
  int64_t n = numel(t);
  HEAL_CHECK(scratch_alloc((size_t)std::max<int64_t>(n, 1) * elem_size(t.dtype), owned));
  out->data = *owned;
  int64_t s = 1;
  for (int i = t.ndim - 1; i >= 0; --i) {
    out->strides[i] = s;
    s *= t.dims[i];
  }
  return copy_strided_impl(t, *out);
}

// ===================================================== derived-table cache
// Entries are keyed by the descriptors of the tensors they derive from and
// stay valid while the write generations of those tensors' allocations do.
// Memory not allocated by heal_alloc has no generation: its entries are
// rebuilt on every use (the previous buffer is freed stream-ordered).
//
// Streams: an entry records an event on the stream that built it and the
// streams that have used it.  A lookup from another stream first waits for
// that event (the build may still be running there); dropping an entry that
// another stream has used waits for the device before its buffers are freed.
struct CacheEntry {
  std::vector<std::pair<const void *, uint64_t>> deps;
  uint64_t epoch = 0;
  std::vector<void *> bufs;
  int64_t i0 = 0, i1 = 0;
  bool b0 = false, b1 = false;
  uint64_t used = 0;
  cudaEvent_t ready = nullptr;        // recorded after the build was enqueued
  std::vector<cudaStream_t> users;    // streams that have used the tables
  bool complete = false;              // false while (or if) the build did not finish
};
static std::unordered_map<std::string, CacheEntry> g_cache;
static uint64_t g_cache_clock = 0;
// A ragged batch touches five tables per distinct (m, k) shape (moduli
// constants, moduli summary, twiddles, inverse twiddles, m_inv): 4096 entries
// keep every shape of a few hundred ciphertexts resident for graph capture.
constexpr size_t kCacheMax = 4096;

// Cache key: the kind, then per tensor its data pointer, dtype, ndim and
// dims / strides as raw bytes (fixed widths, ndim before the dims, so no two
// different argument lists give the same key), then `extra`.  Built on every
// call that uses a derived table, so without any formatting.
static std::string key_of(const char *kind, std::initializer_list<const heal_tensor *> ts, int64_t extra = 0) {
  std::string k(kind);
  k.reserve(k.size() + 16 + ts.size() * (24 + 16 * HEAL_MAX_DIMS));
  auto put = [&k](const void *p, size_t n) { k.append((const char *)p, n); };
  for (const heal_tensor *t : ts) {
    k.push_back('|');
    put(&t->data, sizeof t->data);
    put(&t->dtype, sizeof t->dtype);
    put(&t->ndim, sizeof t->ndim);
    const int nd = std::max(0, std::min<int>(t->ndim, HEAL_MAX_DIMS));
    put(t->dims, nd * sizeof(int64_t));
    put(t->strides, nd * sizeof(int64_t));
  }
  k.push_back('#');
  put(&extra, sizeof extra);
  return k;
}

static void drop_entry(CacheEntry &e) {
  bool foreign = !e.complete;  // another stream may still be reading (or building) the tables
  for (cudaStream_t s : e.users) foreign = foreign || s != stream();
  if (foreign && !e.bufs.empty()) cudaDeviceSynchronize();
  for (void *b : e.bufs) scratch_free(b);
  e.bufs.clear();
  if (e.ready) cudaEventDestroy(e.ready);
  e.ready = nullptr;
  e.users.clear();
}

// Called once an entry's build is enqueued on the current stream.
static void entry_built(CacheEntry &e) {
  if (!e.ready && cudaEventCreateWithFlags(&e.ready, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    e.ready = nullptr;
  }
  if (e.ready) cudaEventRecord(e.ready, stream());
  e.users.assign(1, stream());
  e.complete = true;
}

static int refuse_in_capture(const char *what) {
  return set_error(HEAL_ERR_RUNTIME, std::string(what) +
                                         ": the table for this tensor is not cached yet; run the call once before "
                                         "capturing it in a graph");
}

// Returns the valid entry for `key`, or nullptr (after dropping a stale one;
// while a graph is being captured a stale entry is left alone).
static CacheEntry *cache_lookup(const std::string &key) {
  auto it = g_cache.find(key);
  if (it == g_cache.end()) return nullptr;
  bool ok = it->second.complete;  // a build that returned early left an incomplete entry
  if (!ok && g_rt.capturing) return nullptr;
  for (auto &d : it->second.deps) {
    uint64_t g = generation_of(d.first);
    if (g != d.second || (g == 0 && it->second.epoch != g_epoch.load())) ok = false;
  }
  if (!ok) {
    if (g_rt.capturing) return nullptr;
    drop_entry(it->second);
    g_cache.erase(it);
    return nullptr;
  }
  CacheEntry &e = it->second;
  e.used = ++g_cache_clock;
  const cudaStream_t s = stream();
  if (!g_rt.capturing && std::find(e.users.begin(), e.users.end(), s) == e.users.end()) {
    if (e.ready) cudaStreamWaitEvent(s, e.ready, 0);  // the build may still run on its own stream
    e.users.push_back(s);
  }
  return &e;
}

static CacheEntry &cache_insert(const std::string &key, std::initializer_list<const void *> deps) {
  if (g_cache.size() >= kCacheMax) {  // evict the least recently used entry
    auto victim = g_cache.begin();
    for (auto it = g_cache.begin(); it != g_cache.end(); ++it)
      if (it->second.used < victim->second.used) victim = it;
    drop_entry(victim->second);
    g_cache.erase(victim);
  }
  CacheEntry &e = g_cache[key];
  drop_entry(e);
  e = CacheEntry();
  for (const void *d : deps) e.deps.push_back({d, generation_of(d)});
  e.epoch = g_epoch.load();
  e.used = ++g_cache_clock;
  return e;
}

static void cache_forget(uintptr_t base, size_t bytes) {
  for (auto it = g_cache.begin(); it != g_cache.end();) {
    bool hit = false;
    for (auto &d : it->second.deps) {
      uintptr_t a = (uintptr_t)d.first;
      if (a >= base && a < base + std::max<size_t>(bytes, 1)) hit = true;
    }
    if (hit) {
      drop_entry(it->second);
      it = g_cache.erase(it);
    } else {
      ++it;
    }
  }
}

template <typename T>
__device__ __forceinline__ int64_t load_elem(const void *base, int64_t off) {
  return (int64_t)((const T *)base)[off];
}
__device__ __forceinline__ int64_t load_any(const void *base, int dtype, int64_t off) {
  return dtype == HEAL_INT32 ? load_elem<int32_t>(base, off) : load_elem<int64_t>(base, off);
}
__device__ __forceinline__ int64_t view_offset(const View &v, int64_t idx) {
  int64_t off = 0;
  for (int i = v.ndim - 1; i >= 0; --i) {
    int64_t d = v.dims[i];
    off += (idx % d) * v.strides[i];
    idx /= d;
  }
  return off;
}

// ---------------------------------------------------------------- moduli
__global__ void mod_table_kernel(const void *p, int dtype, View v, int64_t n, void *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = load_any(p, dtype, view_offset(v, i));
    if (dtype == HEAL_INT32)
      ((MG32 *)out)[i] = mg32_make(q);
    else
      ((MG64 *)out)[i] = mg64_make(q);
  }
}

int mod_table(const heal_tensor &p, ModTable *out) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  std::string key = key_of("mod", {&p});
  CacheEntry *e = cache_lookup(key);
  if (!e && g_rt.capturing) return refuse_in_capture("modulus constants");
  if (!e) {
    CacheEntry &n = cache_insert(key, {p.data});
    int64_t cnt = numel(p);
    size_t es = p.dtype == HEAL_INT32 ? sizeof(MG32) : sizeof(MG64);
    void *buf;
    HEAL_CHECK(scratch_alloc(std::max<size_t>(1, cnt) * es, &buf));
    n.bufs.push_back(buf);
    n.i0 = cnt;
    if (cnt) {
      mod_table_kernel<<<grid_for(cnt, 128), 128, 0, stream()>>>(p.data, p.dtype, make_view(p), cnt, buf);
      HEAL_CHECK(check_launch("mod_table"));
    }
    entry_built(n);
    e = &n;
  }
  out->consts = e->bufs[0];
  out->count = e->i0;
  return HEAL_OK;
}

struct MinMax {
  unsigned long long min_enc, max_enc;  // order-preserving encodings of int64
};
__device__ __forceinline__ unsigned long long enc64(int64_t x) { return (unsigned long long)x ^ 0x8000000000000000ull; }
static int64_t dec64(unsigned long long x) { return (int64_t)(x ^ 0x8000000000000000ull); }

__global__ void mod_info_kernel(const void *p, int dtype, int64_t stride, int64_t k, int64_t *q, uint64_t *qone,
                                MinMax *mm) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t v = load_any(p, dtype, i * stride);
    q[i] = v;
    // floor(2^64 / q); 2^64 - 1 stands in for q = 1 (the Shoup bound still holds)
    qone[i] = v > 1 ? (uint64_t)((((u128)1) << 64) / (u128)(uint64_t)v) : ~0ull;
    atomicMin(&mm->min_enc, enc64(v));
    atomicMax(&mm->max_enc, enc64(v));
  }
}

int mod_info(const heal_tensor &p, ModInfo *out) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  std::string key = key_of("modinfo", {&p});
  CacheEntry *e = cache_lookup(key);
  if (!e && g_rt.capturing) return refuse_in_capture("mod_info");
  if (!e) {
    CacheEntry &n = cache_insert(key, {p.data});
    int64_t k = p.ndim ? p.dims[0] : 1;
    void *buf, *mmb;
    HEAL_CHECK(scratch_alloc(2 * sizeof(int64_t) * std::max<int64_t>(k, 1), &buf));  // q, then floor(2^64 / q)
    n.bufs.push_back(buf);
    HEAL_CHECK(scratch_alloc(sizeof(MinMax), &mmb));
    MinMax init = {~0ull, 0ull};
    HEAL_TRY_CUDA(cudaMemcpyAsync(mmb, &init, sizeof init, cudaMemcpyHostToDevice, stream()));
    if (k) {
      mod_info_kernel<<<grid_for(k, 128), 128, 0, stream()>>>(p.data, p.dtype, p.ndim ? p.strides[0] : 0, k,
                                                              (int64_t *)buf, (uint64_t *)buf + k, (MinMax *)mmb);
      HEAL_CHECK(check_launch("mod_info"));
    }
    MinMax h;
    HEAL_TRY_CUDA(cudaMemcpyAsync(&h, mmb, sizeof h, cudaMemcpyDeviceToHost, stream()));
    HEAL_TRY_CUDA(cudaStreamSynchronize(stream()));
    scratch_free(mmb);
    n.i0 = k ? dec64(h.min_enc) : 1;
    n.i1 = k ? dec64(h.max_enc) : 1;
    entry_built(n);
    e = &n;
  }
  out->min_q = e->i0;
  out->max_q = e->i1;
  out->q = (const int64_t *)e->bufs[0];
  out->qone = (const uint64_t *)e->bufs[0] + std::max<int64_t>(p.ndim ? p.dims[0] : 1, 1);
  return HEAL_OK;
}

// ------------------------------------------------------------- twiddles
struct TwArgs {
  const void *tw;
  int tw_dtype;
  int64_t tw_s0, tw_s1;
  const int64_t *q;
  const int32_t *rows;  // compact row -> source row (null: identity)
  int64_t k, m;         // k = rows in the output table
  void *pairs;
  int *neg;
};

template <bool WIDE>
__global__ void twiddle_kernel(TwArgs a) {
  int64_t n = a.k * a.m;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t u = i / a.m, j = i - u * a.m;
    int64_t t = a.rows ? (int64_t)a.rows[u] : u;
    int64_t s = load_any(a.tw, a.tw_dtype, t * a.tw_s0 + j * a.tw_s1);
    int64_t q = a.q[t];
    if (s < 0) atomicOr(a.neg, 1);
    uint64_t mag = s < 0 ? (uint64_t)0 - (uint64_t)s : (uint64_t)s;
    uint64_t w = q > 0 ? mag % (uint64_t)q : 0;
    if (WIDE) {
      ulonglong2 pr;
      pr.x = w;
      pr.y = q > 0 ? shoup64_companion(w, (uint64_t)q) : 0;
      ((ulonglong2 *)a.pairs)[i] = pr;
    } else {
      uint2 pr;
      pr.x = (uint32_t)w;
      pr.y = q > 0 ? shoup32_companion((uint32_t)w, (uint32_t)q) : 0;
      ((uint2 *)a.pairs)[i] = pr;
    }
  }
}

static int build_pairs(const void *tw, int tw_dtype, int64_t s0, int64_t s1, const int64_t *q, const int32_t *rows,
                       int64_t k, int64_t m, int wide, CacheEntry &n) {
  void *pairs, *flag;
  size_t es = wide ? sizeof(ulonglong2) : sizeof(uint2);
  HEAL_CHECK(scratch_alloc(std::max<int64_t>(k * m, 1) * es, &pairs));
  n.bufs.push_back(pairs);
  HEAL_CHECK(scratch_alloc(sizeof(int), &flag));
  n.bufs.push_back(flag);
  HEAL_TRY_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), stream()));
  if (k * m) {
    TwArgs a{tw, tw_dtype, s0, s1, q, rows, k, m, pairs, (int *)flag};
    if (wide)
      twiddle_kernel<true><<<grid_for(k * m, 256), 256, 0, stream()>>>(a);
    else
      twiddle_kernel<false><<<grid_for(k * m, 256), 256, 0, stream()>>>(a);
    HEAL_CHECK(check_launch("twiddle_table"));
  }
  return HEAL_OK;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// one block per twiddle row: an order-aware hash of the row and its modulus
__global__ void row_hash_kernel(const void *tw, int dtype, int64_t s0, int64_t s1, const int64_t *q, int64_t m,
                                unsigned long long *h) {
  const int64_t t = blockIdx.x;
  unsigned long long acc = 0;
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x)
    acc += mix64((unsigned long long)load_any(tw, dtype, t * s0 + j * s1) ^ ((unsigned long long)j * 0x9E3779B97F4A7C15ull));
  if (threadIdx.x == 0) acc += mix64((unsigned long long)q[t] + 0x5851F42D4C957F2Dull);
  atomicAdd(&h[t], acc);
}

// rows whose hash matched their representative: compare every element
__global__ void row_verify_kernel(const void *tw, int dtype, int64_t s0, int64_t s1, const int64_t *q, int64_t m,
                                  const int32_t *rep, int *bad) {
  const int64_t t = blockIdx.x;
  const int64_t r = rep[t];
  if (r == t) return;
  if (q[t] != q[r]) {
    if (threadIdx.x == 0) bad[t] = 1;
    return;
  }
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x)
    if (load_any(tw, dtype, t * s0 + j * s1) != load_any(tw, dtype, r * s0 + j * s1)) bad[t] = 1;
}

int twiddle_table(const heal_tensor &tw, const heal_tensor &p, int wide, TwiddleTable *out) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  ModInfo mi;
  HEAL_CHECK(mod_info(p, &mi));
  std::string key = key_of("tw", {&tw, &p}, wide);
  CacheEntry *e = cache_lookup(key);
  if (!e && g_rt.capturing) return refuse_in_capture("twiddle table");
  if (!e) {
    CacheEntry &n = cache_insert(key, {tw.data, p.data});
    const int64_t k = tw.dims[0], m = tw.dims[1];
    // rows with equal content and modulus (tiled moduli, repeated
    // ciphertext components) share one row of the Shoup table
    std::vector<int32_t> rep(k);
    for (int64_t t = 0; t < k; ++t) rep[t] = (int32_t)t;
    if (k > 1 && m > 0) {
      void *hb, *rb, *bb;
      HEAL_CHECK(scratch_alloc(sizeof(unsigned long long) * k, &hb));
      HEAL_TRY_CUDA(cudaMemsetAsync(hb, 0, sizeof(unsigned long long) * k, stream()));
      row_hash_kernel<<<(unsigned)k, 256, 0, stream()>>>(tw.data, tw.dtype, tw.strides[0], tw.strides[1], mi.q, m,
                                                       (unsigned long long *)hb);
      HEAL_CHECK(check_launch("row_hash"));
      std::vector<unsigned long long> hh(k);
      HEAL_TRY_CUDA(cudaMemcpyAsync(hh.data(), hb, sizeof(unsigned long long) * k, cudaMemcpyDeviceToHost, stream()));
      HEAL_TRY_CUDA(cudaStreamSynchronize(stream()));
      scratch_free(hb);
      std::unordered_map<unsigned long long, int32_t> first;
      bool any = false;
      for (int64_t t = 0; t < k; ++t) {
        auto it = first.find(hh[t]);
        if (it == first.end()) {
          first[hh[t]] = (int32_t)t;
        } else {
          rep[t] = it->second;
          any = true;
        }
      }
      if (any) {
        HEAL_CHECK(scratch_alloc(sizeof(int32_t) * k, &rb));
        HEAL_CHECK(scratch_alloc(sizeof(int) * k, &bb));
        HEAL_TRY_CUDA(cudaMemcpyAsync(rb, rep.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice, stream()));
        HEAL_TRY_CUDA(cudaMemsetAsync(bb, 0, sizeof(int) * k, stream()));
        row_verify_kernel<<<(unsigned)k, 256, 0, stream()>>>(tw.data, tw.dtype, tw.strides[0], tw.strides[1], mi.q, m,
                                                           (const int32_t *)rb, (int *)bb);
        HEAL_CHECK(check_launch("row_verify"));
        std::vector<int> bad(k);
        HEAL_TRY_CUDA(cudaMemcpyAsync(bad.data(), bb, sizeof(int) * k, cudaMemcpyDeviceToHost, stream()));
        HEAL_TRY_CUDA(cudaStreamSynchronize(stream()));
        scratch_free(rb);
        scratch_free(bb);
        for (int64_t t = 0; t < k; ++t)
          if (bad[t]) rep[t] = (int32_t)t;
      }
    }
    std::vector<int32_t> rows, rowmap(k);
    std::vector<int32_t> compact(k, -1);
    for (int64_t t = 0; t < k; ++t) {
      if (rep[t] == t) {
        compact[t] = (int32_t)rows.size();
        rows.push_back((int32_t)t);
      }
    }
    for (int64_t t = 0; t < k; ++t) rowmap[t] = compact[rep[t]];
    void *rows_d, *map_d;
    HEAL_CHECK(scratch_alloc(sizeof(int32_t) * std::max<size_t>(rows.size(), 1), &rows_d));
    HEAL_CHECK(scratch_alloc(sizeof(int32_t) * std::max<int64_t>(k, 1), &map_d));
    if (!rows.empty())
      HEAL_TRY_CUDA(cudaMemcpyAsync(rows_d, rows.data(), sizeof(int32_t) * rows.size(), cudaMemcpyHostToDevice, stream()));
    if (k) HEAL_TRY_CUDA(cudaMemcpyAsync(map_d, rowmap.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice, stream()));
    HEAL_CHECK(build_pairs(tw.data, tw.dtype, tw.strides[0], tw.strides[1], mi.q, (const int32_t *)rows_d,
                           (int64_t)rows.size(), m, wide, n));
    n.bufs.push_back(map_d);   // bufs: pairs, neg flag, rowmap
    // the host vectors above must outlive the copies that read them
    HEAL_TRY_CUDA(cudaStreamSynchronize(stream()));
    scratch_free(rows_d);
    n.i0 = (int64_t)rows.size();
    entry_built(n);
    e = &n;
  }
  out->pairs = e->bufs[0];
  out->neg_flag = (const int *)e->bufs[1];
  out->rowmap = (const int32_t *)e->bufs[2];
  out->wide = wide;
  return HEAL_OK;
}

int minv_table(const heal_tensor &minv, const heal_tensor &p, int64_t k, int wide, TwiddleTable *out) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  ModInfo mi;
  HEAL_CHECK(mod_info(p, &mi));
  std::string key = key_of("minv", {&minv, &p}, wide * 1000003 + k);
  CacheEntry *e = cache_lookup(key);
  if (!e) {
    CacheEntry &n = cache_insert(key, {minv.data, p.data});
    HEAL_CHECK(build_pairs(minv.data, minv.dtype, minv.strides[0], 0, mi.q, nullptr, k, 1, wide, n));
    entry_built(n);
    e = &n;
  }
  out->pairs = e->bufs[0];
  out->neg_flag = (const int *)e->bufs[1];
  out->rowmap = nullptr;
  out->wide = wide;
  return HEAL_OK;
}

// ---------------------------------------------------------- permutations
struct PermCounts {
  unsigned long long bad, distinct;
  unsigned long long not_bitrev;  // entries differing from the bit reversal of their index
};

__global__ void perm_kernel(const void *perm, int dtype, int64_t stride, int64_t m, int logm, int32_t *perm32,
                            int32_t *inv32, PermCounts *cnt) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < m; u += (int64_t)gridDim.x * blockDim.x) {
    int64_t v = load_any(perm, dtype, u * stride);
    if (v < 0 || v >= m) {
      atomicAdd(&cnt->bad, 1ull);
      perm32[u] = 0;
      continue;
    }
    perm32[u] = (int32_t)v;
    int old = atomicMax(&inv32[v], (int)u);
    if (old < 0) atomicAdd(&cnt->distinct, 1ull);
    if (logm > 0 && v != (int64_t)(__brev((uint32_t)u) >> (32 - logm))) atomicAdd(&cnt->not_bitrev, 1ull);
  }
}

int perm_info(const heal_tensor &perm, PermInfo *out) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  std::string key = key_of("perm", {&perm});
  CacheEntry *e = cache_lookup(key);
  if (!e && g_rt.capturing) return refuse_in_capture("permutation table");
  if (!e) {
    CacheEntry &n = cache_insert(key, {perm.data});
    int64_t m = perm.dims[0];
    if (m > INT32_MAX) return set_error(HEAL_ERR_INVALID_ARGUMENT, "transform length too large");
    void *p32, *i32, *cnt;
    HEAL_CHECK(scratch_alloc(sizeof(int32_t) * std::max<int64_t>(m, 1), &p32));
    n.bufs.push_back(p32);
    HEAL_CHECK(scratch_alloc(sizeof(int32_t) * std::max<int64_t>(m, 1), &i32));
    n.bufs.push_back(i32);
    HEAL_CHECK(scratch_alloc(sizeof(PermCounts), &cnt));
    HEAL_TRY_CUDA(cudaMemsetAsync(i32, 0xFF, sizeof(int32_t) * std::max<int64_t>(m, 1), stream()));
    HEAL_TRY_CUDA(cudaMemsetAsync(cnt, 0, sizeof(PermCounts), stream()));
    if (m) {
      int logm = 0;
      while (((int64_t)1 << logm) < m) ++logm;
      if (((int64_t)1 << logm) != m) logm = 0;  // bit reversal only for power-of-two lengths
      perm_kernel<<<grid_for(m, 256), 256, 0, stream()>>>(perm.data, perm.dtype, perm.strides[0], m, logm,
                                                           (int32_t *)p32, (int32_t *)i32, (PermCounts *)cnt);
      n.i0 = logm;
      HEAL_CHECK(check_launch("perm_info"));
    }
    PermCounts h;
    HEAL_TRY_CUDA(cudaMemcpyAsync(&h, cnt, sizeof h, cudaMemcpyDeviceToHost, stream()));
    HEAL_TRY_CUDA(cudaStreamSynchronize(stream()));
    scratch_free(cnt);
    n.b0 = h.distinct == (unsigned long long)m && h.bad == 0;
    n.b1 = h.bad != 0;
    n.i1 = (m > 1 && n.i0 > 0 && n.b0 && h.not_bitrev == 0) ? n.i0 : 0;
    entry_built(n);
    e = &n;
  }
  out->perm32 = (const int32_t *)e->bufs[0];
  out->inv32 = (const int32_t *)e->bufs[1];
  out->bijective = e->b0;
  out->bad = e->b1;
  out->bitrev_log = (int)e->i1;
  return HEAL_OK;
}

__global__ void perms_check_kernel(const void *perms, int dtype, int64_t s0, int64_t s1, int64_t l, int64_t m,
                                   unsigned long long *bad) {
  int64_t n = l * m;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / m, c = i - r * m;
    int64_t v = load_any(perms, dtype, r * s0 + c * s1);
    if (v < 0 || v >= m) atomicAdd(bad, 1ull);
  }
}

int perms_valid(const heal_tensor &perms, int64_t m, bool *ok) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  std::string key = key_of("perms", {&perms}, m);
  CacheEntry *e = cache_lookup(key);
  if (!e && g_rt.capturing) return refuse_in_capture("permutation check");
  if (!e) {
    CacheEntry &n = cache_insert(key, {perms.data});
    void *cnt;
    HEAL_CHECK(scratch_alloc(sizeof(unsigned long long), &cnt));
    HEAL_TRY_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), stream()));
    int64_t l = perms.dims[0];
    if (l * m) {
      perms_check_kernel<<<grid_for(l * m, 256), 256, 0, stream()>>>(perms.data, perms.dtype, perms.strides[0],
                                                                     perms.strides[1], l, m,
                                                                     (unsigned long long *)cnt);
      HEAL_CHECK(check_launch("perms_check"));
    }
    unsigned long long h = 0;
    HEAL_TRY_CUDA(cudaMemcpyAsync(&h, cnt, sizeof h, cudaMemcpyDeviceToHost, stream()));
    HEAL_TRY_CUDA(cudaStreamSynchronize(stream()));
    scratch_free(cnt);
    n.b0 = h == 0;
    entry_built(n);
    e = &n;
  }
  *ok = e->b0;
  return HEAL_OK;
}

}  // namespace heal

using namespace heal;

// ============================================================== C ABI
extern "C" {

int heal_init(int device) {
  clear_error();
  return init_device(device);
}

const char *heal_last_error(void) { return g_last_error.c_str(); }

struct HealGraph {
  cudaGraphExec_t exec;
  uint64_t kernels;  // kernel launches recorded in the graph
};

int heal_graph_begin(void) {
  clear_error();
  HEAL_CHECK(ensure_init());
  if (g_rt.capturing) return set_error(HEAL_ERR_RUNTIME, "heal_graph_begin: already capturing");
  HEAL_TRY_CUDA(cudaStreamBeginCapture(stream(), cudaStreamCaptureModeThreadLocal));
  g_rt.capturing = true;
  g_rt.capture_start = g_rt.launches.load();
  g_rt.origin = stream();
  g_rt.forked = 0;
  return HEAL_OK;
}

int heal_graph_fork(int n) {
  clear_error();
  if (!g_rt.capturing) return set_error(HEAL_ERR_RUNTIME, "heal_graph_fork: not capturing");
  if (g_rt.forked) return set_error(HEAL_ERR_RUNTIME, "heal_graph_fork: this capture is already forked");
  if (n < 1 || n > HEAL_GRAPH_MAX_BRANCHES)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_graph_fork: n must be in [1, " + std::to_string(HEAL_GRAPH_MAX_BRANCHES) + "]");
  if (!g_rt.join) HEAL_TRY_CUDA(cudaEventCreateWithFlags(&g_rt.join, cudaEventDisableTiming));
  while ((int)g_rt.branches.size() < n) {
    cudaStream_t s;
    HEAL_TRY_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    g_rt.branches.push_back(s);
  }
  HEAL_TRY_CUDA(cudaEventRecord(g_rt.join, g_rt.origin));
  for (int i = 0; i < n; ++i) HEAL_TRY_CUDA(cudaStreamWaitEvent(g_rt.branches[i], g_rt.join, 0));
  g_rt.forked = n;
  return HEAL_OK;
}

int heal_graph_branch(int i) {
  clear_error();
  if (!g_rt.capturing) return set_error(HEAL_ERR_RUNTIME, "heal_graph_branch: not capturing");
  if (i < -1 || i >= g_rt.forked)
    return set_error(HEAL_ERR_OUT_OF_RANGE, "heal_graph_branch: branch " + std::to_string(i) + " was not forked");
  g_rt.cur = i < 0 ? g_rt.origin : g_rt.branches[i];
  return HEAL_OK;
}

int heal_graph_end(void **graph) {
  clear_error();
  if (!graph) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_graph_end: graph must not be null");
  *graph = nullptr;
  if (!g_rt.capturing) return set_error(HEAL_ERR_RUNTIME, "heal_graph_end: not capturing");
  g_rt.capturing = false;
  const uint64_t recorded = g_rt.launches.load() - g_rt.capture_start;
  g_rt.launches.fetch_sub(recorded);  // counted again at every replay
  // join every branch back into the stream the capture began on
  cudaError_t je = cudaSuccess;
  for (int i = 0; i < g_rt.forked && je == cudaSuccess; ++i) {
    je = cudaEventRecord(g_rt.join, g_rt.branches[i]);
    if (je == cudaSuccess) je = cudaStreamWaitEvent(g_rt.origin, g_rt.join, 0);
  }
  g_rt.forked = 0;
  g_rt.cur = g_rt.origin;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(g_rt.origin, &g);
  if (je != cudaSuccess || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_fail(je != cudaSuccess ? je : e, "heal_graph_end");
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  *graph = new HealGraph{exec, recorded};
  return HEAL_OK;
}

int heal_graph_launch(void *graph) {
  if (!graph) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_graph_launch: graph must not be null");
  HealGraph *hg = (HealGraph *)graph;
  HEAL_TRY_CUDA(cudaGraphLaunch(hg->exec, stream()));
  note_launch((int)hg->kernels);
  return HEAL_OK;
}

int heal_graph_destroy(void *graph) {
  if (!graph) return HEAL_OK;
  HealGraph *hg = (HealGraph *)graph;
  cudaGraphExecDestroy(hg->exec);
  delete hg;
  return HEAL_OK;
}

// calls that wait for the GPU or change the allocation registry cannot be
// recorded into a graph
static int refuse_sync(const char *what) {
  return set_error(HEAL_ERR_RUNTIME, std::string(what) + ": not allowed while a graph is being captured");
}

int heal_synchronize(void) {
  HEAL_CHECK(ensure_init());
  if (g_rt.capturing) return refuse_sync("heal_synchronize");
  HEAL_TRY_CUDA(cudaStreamSynchronize(stream()));
  return flush_diag();
}

void *heal_get_stream(void) {
  if (ensure_init()) return nullptr;
  return (void *)stream();
}

int heal_set_stream(void *s) {
  HEAL_CHECK(ensure_init());
  g_rt.cur = s ? (cudaStream_t)s : g_rt.own;
  return HEAL_OK;
}

uint64_t heal_kernel_launch_count(void) { return g_rt.launches.load(); }

int heal_set_reference_compat(int on) {
  g_reference_compat.store(on != 0);
  return HEAL_OK;
}

int heal_get_reference_compat(void) { return g_reference_compat.load() ? 1 : 0; }

int heal_alloc(size_t bytes, int zero, void **out) {
  if (!out) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_alloc: out must not be null");
  *out = nullptr;
  HEAL_CHECK(ensure_init());
  if (g_rt.capturing) return refuse_sync("heal_alloc");
  if (bytes == 0) return HEAL_OK;
  void *p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes, stream());
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(HEAL_ERR_BAD_ALLOC, "heal_alloc: out of device memory");
  }
  if (zero) HEAL_TRY_CUDA(cudaMemsetAsync(p, 0, bytes, stream()));
  {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    g_allocs[(uintptr_t)p] = Alloc{bytes, g_gen.fetch_add(1)};
  }
  *out = p;
  return HEAL_OK;
}

int heal_free(void *ptr) {
  if (!ptr) return HEAL_OK;
  HEAL_CHECK(ensure_init());
  if (g_rt.capturing) return refuse_sync("heal_free");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  auto it = g_allocs.find((uintptr_t)ptr);
  if (it == g_allocs.end()) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_free: pointer not from heal_alloc");
  cache_forget(it->first, it->second.bytes);
  g_allocs.erase(it);
  HEAL_TRY_CUDA(cudaFreeAsync(ptr, stream()));
  return HEAL_OK;
}

static bool is_pinned(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

int heal_h2d(void *dst, const void *src, size_t bytes) {
  HEAL_CHECK(ensure_init());
  if (g_rt.capturing) return refuse_sync("heal_h2d");
  if (!bytes) return HEAL_OK;
  HEAL_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, stream()));
  if (!is_pinned(src)) HEAL_TRY_CUDA(cudaStreamSynchronize(stream()));
  mark_written(dst);
  return HEAL_OK;
}

int heal_d2h(void *dst, const void *src, size_t bytes) {
  HEAL_CHECK(ensure_init());
  if (g_rt.capturing) return refuse_sync("heal_d2h");
  if (bytes) HEAL_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, stream()));
  HEAL_TRY_CUDA(cudaStreamSynchronize(stream()));
  return flush_diag();
}

int heal_h2d_async(void *dst, const void *src, size_t bytes) {
  HEAL_CHECK(ensure_init());
  if (bytes) HEAL_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream()));
  mark_written(dst);
  return HEAL_OK;
}

int heal_d2h_async(void *dst, const void *src, size_t bytes) {
  HEAL_CHECK(ensure_init());
  if (bytes) HEAL_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream()));
  return HEAL_OK;
}

int heal_host_alloc(size_t bytes, void **out) {
  HEAL_CHECK(ensure_init());
  *out = nullptr;
  if (!bytes) return HEAL_OK;
  HEAL_TRY_CUDA(cudaMallocHost(out, bytes));
  return HEAL_OK;
}

int heal_host_free(void *ptr) {
  if (ptr) HEAL_TRY_CUDA(cudaFreeHost(ptr));
  return HEAL_OK;
}

int heal_mark_modified(void *ptr) {
  mark_written(ptr);
  return HEAL_OK;
}

int heal_copy_strided(const heal_tensor *src, const heal_tensor *dst) {
  clear_error();
  HEAL_CHECK(ensure_init());
  HEAL_CHECK(check_desc(src, "src", false));
  HEAL_CHECK(check_desc(dst, "dst", false));
  if (!same_dims(*src, *dst) || elem_size(src->dtype) != elem_size(dst->dtype))
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_copy_strided: shapes or element types differ");
  if (overlaps(*src, *dst) && !identical_view(*src, *dst)) {
    heal_tensor tmp;
    void *owned;
    HEAL_CHECK(materialize(*src, &tmp, &owned));
    int rc = copy_strided_impl(tmp, *dst);
    scratch_free(owned);
    return rc;
  }
  if (identical_view(*src, *dst)) return HEAL_OK;
  return copy_strided_impl(*src, *dst);
}

// ------------------------------------------------- stride-only metadata
int heal_tensor_reshape(heal_tensor *t, int32_t new_ndim, const int64_t *new_dims) {
  if (!t || new_ndim < 0 || new_ndim > HEAL_MAX_DIMS || (new_ndim && !new_dims))
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "reshape: unsupported number of dimensions");
  // DeviceTensor::reshape (device_memory_impl.cpp:42-84): the element count
  // excludes stride-0 axes; the new strides are row-major.
  int64_t new_total = 1, cur_total = 1;
  for (int i = 0; i < new_ndim; ++i) new_total *= new_dims[i];
  for (int i = 0; i < t->ndim; ++i)
    if (t->strides[i] != 0) cur_total *= t->dims[i];
  if (new_total != cur_total)
    return set_error(HEAL_ERR_INVALID_ARGUMENT,
                     "Total size of new shape must match number of elements (excluding broadcasted dims).");
  int64_t s = 1;
  for (int i = new_ndim - 1; i >= 0; --i) {
    t->dims[i] = new_dims[i];
    t->strides[i] = s;
    s *= new_dims[i];
  }
  t->ndim = new_ndim;
  return HEAL_OK;
}

int heal_tensor_expand(heal_tensor *t, int64_t axis, int64_t repeats) {
  // expand (memory_virtual_ops_impl.cpp:7-40)
  if (repeats <= 0) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Repeat count must be positive.");
  int64_t nd = t->ndim;
  if (axis < 0) axis += nd;
  if (axis < 0 || axis >= nd) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Invalid repeat dimension.");
  if (t->dims[axis] != 1) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Can only expand a dimension of size 1.");
  t->dims[axis] *= repeats;
  t->strides[axis] = 0;
  return HEAL_OK;
}

int heal_tensor_squeeze(heal_tensor *t, int64_t axis) {
  // squeeze (memory_virtual_ops_impl.cpp:42-65)
  int64_t nd = t->ndim;
  if (axis < 0) axis += nd;
  if (axis < 0 || axis >= nd) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Invalid squeeze dimension.");
  if (t->dims[axis] != 1) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Can only squeeze dimensions of size 1.");
  for (int64_t i = axis; i + 1 < nd; ++i) {
    t->dims[i] = t->dims[i + 1];
    t->strides[i] = t->strides[i + 1];
  }
  t->ndim = (int32_t)(nd - 1);
  return HEAL_OK;
}

int heal_tensor_unsqueeze(heal_tensor *t, int64_t axis) {
  // unsqueeze (memory_virtual_ops_impl.cpp:67-86): inserts dim 1, stride 0
  int64_t nd = t->ndim;
  if (axis < 0) axis += nd + 1;
  if (axis < 0 || axis > nd) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Invalid unsqueeze dimension.");
  if (nd >= HEAL_MAX_DIMS) return set_error(HEAL_ERR_INVALID_ARGUMENT, "unsqueeze: too many dimensions");
  for (int64_t i = nd; i > axis; --i) {
    t->dims[i] = t->dims[i - 1];
    t->strides[i] = t->strides[i - 1];
  }
  t->dims[axis] = 1;
  t->strides[axis] = 0;
  t->ndim = (int32_t)(nd + 1);
  return HEAL_OK;
}

int heal_tensor_moveaxis(heal_tensor *t, int64_t src, int64_t dst) {
  int64_t nd = t->ndim;
  if (src < 0) src += nd;
  if (dst < 0) dst += nd;
  if (src < 0 || src >= nd || dst < 0 || dst >= nd)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "Invalid moveaxis dimension.");
  int64_t d = t->dims[src], s = t->strides[src];
  if (src < dst) {
    for (int64_t i = src; i < dst; ++i) {
      t->dims[i] = t->dims[i + 1];
      t->strides[i] = t->strides[i + 1];
    }
  } else {
    for (int64_t i = src; i > dst; --i) {
      t->dims[i] = t->dims[i - 1];
      t->strides[i] = t->strides[i - 1];
    }
  }
  t->dims[dst] = d;
  t->strides[dst] = s;
  return HEAL_OK;
}

int heal_tensor_slice(heal_tensor *t, int64_t axis, int64_t start, int64_t stop, int64_t step) {
  int64_t nd = t->ndim;
  if (axis < 0) axis += nd;
  if (axis < 0 || axis >= nd) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Invalid slice dimension.");
  if (step <= 0) return set_error(HEAL_ERR_INVALID_ARGUMENT, "Slice step must be positive.");
  int64_t d = t->dims[axis];
  if (start < 0) start += d;
  if (stop < 0) stop += d;
  start = std::min(std::max<int64_t>(start, 0), d);
  stop = std::min(std::max<int64_t>(stop, 0), d);
  int64_t len = stop > start ? (stop - start + step - 1) / step : 0;
  if (len > 0 && t->data) t->data = (char *)t->data + start * t->strides[axis] * elem_size(t->dtype);
  t->dims[axis] = len;
  t->strides[axis] *= step;
  return HEAL_OK;
}

int heal_tensor_is_contiguous(const heal_tensor *t) {
  // DeviceTensor::is_contiguous (device_memory_impl.cpp:31-40)
  int64_t expected = 1;
  for (int i = t->ndim - 1; i >= 0; --i) {
    if (t->dims[i] == 1) continue;
    if (t->strides[i] != expected) return 0;
    expected *= t->dims[i];
  }
  return 1;
}

int64_t heal_tensor_span(const heal_tensor *t) {
  if (numel(*t) == 0) return 0;
  int64_t s = 1;
  for (int i = 0; i < t->ndim; ++i) s += (t->dims[i] - 1) * t->strides[i];
  return s;
}

}  // extern "C"
