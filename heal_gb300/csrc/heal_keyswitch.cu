// heal_keyswitch.cu — heal_keyswitch_batch: the fused keyswitch step (INTT,
// g_decomposition + NTT of the digits, modmul -> axis_modsum -> permute) of
// many ciphertexts of any ring degree and limb count in one persistent launch.
//
// Each job is the three calls of a fused keyswitch step
// (heal_gb300.chain.KeyswitchChain.run_fused):
//   heal_intt(ct, p, perm, inv_twiddles, m_inv) -> x
//   heal_g_decomposition_ntt(x, power, base_bits, p_digits, perm, twiddles_digits) -> digits
//   heal_modmul_axis_sum_permute(tail_a, tail_b, p, tail_axis, galois, elementwise_axis, perm_axis) -> result
// (example_impl/ntt_impl.cpp:69-170, g_decomposition_impl.cpp:10-67,
// modop_impl.cpp:44-101, axis_modsum_impl.cpp:12-76, permute_impl.cpp:8-65).
// The host prepares every call exactly as the call itself does (validation,
// derived tables, the same pass arguments) but records the launches instead
// of making them: five stages per job, the INTT's two passes, the digit
// transform's two passes and the tail.  The transforms are split into two
// passes of 2^6 .. 2^8 points (ring degrees 2^12 .. 2^16), tiles of
// 1024 / P limbs, so that every pass runs on 128 threads.
//
// One kernel then runs all stages of all jobs.  Its CTAs take work items
// (one tile of one stage) from a global counter, a few at a time, in queue
// order: stage k of
// every job before stage k + 1 of any job, each stage's jobs grouped by pass
// length.  An item first waits until every tile of the stage it depends on
// (the previous stage of the same job) has finished; since that stage sits
// earlier in the queue, its items were taken by CTAs that are running, and
// the earliest unfinished item never waits, so the launch always completes.
// A finished tile makes its writes visible device-wide (fence) before it
// counts itself done; the waiting CTA reads the count with acquire
// semantics.  Each wait is bounded: one that runs out counts a timeout in the
// device diagnostics, raises an abort flag that ends every other wait, and
// the next heal_synchronize returns HEAL_ERR_RUNTIME.
//
// Results are bit-identical to the three calls made one job after another.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "heal_internal.h"
#include "heal_ntt_kernels.cuh"
#include "heal_ntt_record.h"
#include "heal_tail.cuh"

namespace heal {

enum { KS_INV = 0, KS_GDEC = 1, KS_FWD = 2, KS_TAIL = 3 };
constexpr int kKsThreads = 128;
constexpr int kKsTailPerThread = 8;                       // result elements per thread and tail item
constexpr int kKsTailItem = kKsThreads * kKsTailPerThread;
// jobs per call: their derived tables (a few per job) stay among the table
// cache's most recent entries until the launch that reads them
constexpr int64_t kKsMaxJobs = 256;

struct KsStage {
  uint32_t first;   // its first item in the queue
  uint32_t ntiles;  // its items
  int32_t dep;      // the stage whose items must all have finished first (-1: none)
  uint32_t hold;    // items of dep beyond its own that the wait also needs (0; the test hook sets 1)
  int32_t kind;     // KS_* | pass length (log2) << 4 | (tail: terms << 8 | 32-bit perms << 12)
  union {
    NttArgs ntt;
    TailArgs tail;
  } u;
};

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <typename PT, int D>
__device__ __forceinline__ void ks_tail(const TailArgs &g, uint32_t tile) {
#pragma unroll
  for (int e = 0; e < kKsTailPerThread; ++e) {
    const uint32_t idx = tile * kKsTailItem + e * kKsThreads + threadIdx.x;
    if (idx < g.n) tail_one<int64_t, PT, D>(g, idx);
  }
}

template <typename PT>
__device__ __forceinline__ void ks_tail_d(const TailArgs &g, uint32_t tile, int d) {
  switch (d) {
    case 1: ks_tail<PT, 1>(g, tile); break;
    case 2: ks_tail<PT, 2>(g, tile); break;
    case 3: ks_tail<PT, 3>(g, tile); break;
    default: ks_tail<PT, 4>(g, tile); break;
  }
}

// One pass tile, out of line: each pass class is register-allocated on its
// own (inlined together into one kernel, their allocations spill).
template <bool INV, int LOGP, bool GDEC>
__device__ __noinline__ void ks_pass(const NttArgs &g, uint32_t tile) {
  ntt_reg_body<int64_t, MODE_W64_GROW, INV, LOGP, GDEC>(g, tile);
}

// One stage's tile.  The transform passes are the register kernel's
// (ntt_reg_body: 64-bit growing ranges, 8 points per thread).
__device__ __forceinline__ void ks_run(const KsStage &st, uint32_t tile) {
  const int cls = st.kind & 15, lp = (st.kind >> 4) & 15;
  switch (cls) {
    case KS_INV:
      if (lp == 6) ks_pass<true, 6, false>(st.u.ntt, tile);
      else if (lp == 7) ks_pass<true, 7, false>(st.u.ntt, tile);
      else ks_pass<true, 8, false>(st.u.ntt, tile);
      break;
    case KS_GDEC:
      if (lp == 6) ks_pass<false, 6, true>(st.u.ntt, tile);
      else if (lp == 7) ks_pass<false, 7, true>(st.u.ntt, tile);
      else ks_pass<false, 8, true>(st.u.ntt, tile);
      break;
    case KS_FWD:
      if (lp == 6) ks_pass<false, 6, false>(st.u.ntt, tile);
      else if (lp == 7) ks_pass<false, 7, false>(st.u.ntt, tile);
      else ks_pass<false, 8, false>(st.u.ntt, tile);
      break;
    default: {
      const int d = (st.kind >> 8) & 15;
      if ((st.kind >> 12) & 1) ks_tail_d<int32_t>(st.u.tail, tile, d);
      else ks_tail_d<int64_t>(st.u.tail, tile, d);
    }
  }
}

// Items are claimed kKsClaim at a time (consecutive items mostly lie in one
// stage); the claim of the next run is issued before the current run's work,
// so its latency hides behind it.  The current stage's arguments stay in
// shared memory until a claim leaves it; a stage's dependency is checked once.
constexpr uint32_t kKsClaim = 4;

// the stage of `item`, searching forward from `from` (items only grow)
__device__ __forceinline__ int ks_find(const KsStage *__restrict__ stages, int nstages, int from, uint32_t item) {
  int lo = from, step = 1;
  while (lo + step < nstages && stages[lo + step].first <= item) {  // gallop
    lo += step;
    step <<= 1;
  }
  int hi = min(lo + step, nstages - 1);
  while (lo < hi) {  // the last stage in [lo, hi] whose first item is <= item
    const int mid = (lo + hi + 1) >> 1;
    if (stages[mid].first <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// state: done[nstages] (finished items per stage), then the queue counter,
// then the abort flag
__global__ void __launch_bounds__(kKsThreads, 8)
    keyswitch_batch_kernel(const KsStage *__restrict__ stages, int nstages, uint32_t nitems, uint32_t *state,
                           uint32_t spin_limit, Diag *diag) {
  __shared__ uint32_t sh_claim;
  __shared__ int sh_stage, sh_ok;
  __shared__ __align__(16) KsStage sh_st;
  uint32_t *done = state;
  uint32_t *next = state + nstages;
  volatile uint32_t *abort_flag = state + nstages + 1;
  int cur = -1;  // stage held in sh_st (uniform)
  uint32_t claim = 0, upcoming = 0;
  if (threadIdx.x == 0) upcoming = atomicAdd(next, kKsClaim);
  for (;;) {
    if (threadIdx.x == 0) {
      claim = upcoming;
      if (claim < nitems) upcoming = atomicAdd(next, kKsClaim);  // the run after this one
      sh_claim = claim;
    }
    __syncthreads();
    claim = sh_claim;
    if (claim >= nitems) return;
    const uint32_t end = min(claim + kKsClaim, nitems);
    for (uint32_t item = claim; item < end; ++item) {
      if (cur < 0 || item >= sh_st.first + sh_st.ntiles) {
        // a new stage: find it, wait for its dependency, load its arguments
        __syncthreads();  // every thread is done with sh_st
        if (threadIdx.x == 0) {
          int ok = !*abort_flag;
          const int s = ks_find(stages, nstages, cur < 0 ? 0 : cur, item);
          const int dep = stages[s].dep;
          if (ok && dep >= 0) {
            const uint32_t need = stages[dep].ntiles + stages[s].hold;
            for (uint32_t it = 0; ld_acquire(done + dep) < need; ++it) {
              if (*abort_flag) {
                ok = 0;
                break;
              }
              if (it >= spin_limit) {  // ran out: report, and end every other wait
                atomicAdd(&diag->wait_timeouts, 1ull);
                atomicExch((uint32_t *)abort_flag, 1u);
                ok = 0;
                break;
              }
              __nanosleep(256);
            }
          }
          sh_stage = s;
          sh_ok = ok;
        }
        __syncthreads();
        if (!sh_ok) return;
        cur = sh_stage;
        {
          const uint32_t *src = reinterpret_cast<const uint32_t *>(stages + cur);
          uint32_t *dst = reinterpret_cast<uint32_t *>(&sh_st);
          for (int i = threadIdx.x; i < (int)(sizeof(KsStage) / 4); i += kKsThreads) dst[i] = src[i];
        }
        __syncthreads();
      }
      ks_run(sh_st, item - sh_st.first);
      __threadfence();  // this tile's writes, device-wide, before it counts as done
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(done + cur, 1u);
    }
  }
}

// ------------------------------------------------------------------ host
// the failure-path test hook (heal_keyswitch_batch_test_wait)
static uint32_t g_ks_spin_limit = 1u << 22;  // about a second of polling (256 ns sleeps)
static int g_ks_stall = 0;
// the recorded call's own status and message, prefixed with the job
static int ks_fail(int code, int64_t job, const char *what) {
  const std::string msg = heal_last_error();
  return set_error(code, "heal_keyswitch_batch: job " + std::to_string(job) + ": " + what + ": " + msg);
}
static int ks_bad(int64_t job, const char *what) {
  return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_keyswitch_batch: job " + std::to_string(job) + ": " + what);
}

// The pass rebuilt for 128 threads: tiles of 1024 / P limbs.
static void ks_retile(NttArgs &a) {
  const int C = (8 * kKsThreads) >> a.p;
  int logC = 0;
  while ((1 << logC) < C) ++logC;
  a.C = C;
  a.logC = logC;
  a.ngroups_t = (a.k + C - 1) / C;
  a.fast_bid = a.ngroups_t < (int64_t)UINT32_MAX && a.l * a.r < (int64_t)UINT32_MAX && a.r < (int64_t)UINT32_MAX;
  if (a.fast_bid) {
    a.fd_groups = fastdiv_make((uint32_t)a.ngroups_t);
    a.fd_nij = fastdiv_make((uint32_t)(a.l * a.r));
    a.fd_r = fastdiv_make((uint32_t)a.r);
  }
}

static int ks_chunk(const heal_keyswitch_job *jobs, int64_t n, int64_t base) {
  struct JobStages {
    KsStage st[5];
  };
  std::vector<JobStages> js((size_t)n);
  std::vector<void *> release;
  int rc = HEAL_OK;
  for (int64_t j = 0; j < n && !rc; ++j) {
    const heal_keyswitch_job &b = jobs[j];
    const int64_t jn = base + j;
    if (b.ct.dtype != HEAL_INT64 || b.ct.ndim != 4) {
      rc = ks_bad(jn, "ct must be an int64 tensor [l, m, r, k]");
      break;
    }
    const int64_t m = b.ct.dims[1];
    int logm = 0;
    while ((int64_t(1) << logm) < m) ++logm;
    if ((int64_t(1) << logm) != m || logm < 12 || logm > 16) {
      rc = ks_bad(jn, "the ring degree must be 2^12 .. 2^16");
      break;
    }
    std::vector<NttRecorded> inv, fwd;
    int code;
    if ((code = ntt_record(true, &b.ct, &b.p, &b.perm, &b.inv_twiddles, &b.m_inv, &b.x, 0, 0, logm / 2, &inv,
                           &release))) {
      rc = ks_fail(code, jn, "intt");
      break;
    }
    if ((code = ntt_record(false, &b.x, &b.p_digits, &b.perm, &b.twiddles_digits, nullptr, &b.digits, b.power,
                           b.base_bits, logm / 2, &fwd, &release))) {
      rc = ks_fail(code, jn, "g_decomposition_ntt");
      break;
    }
    TailRecorded tr;
    if ((code = tail_record(&b.tail_a, &b.tail_b, &b.p, b.tail_axis, &b.galois, b.elementwise_axis, b.perm_axis,
                            &b.result, &tr))) {
      rc = ks_fail(code, jn, "modmul_axis_sum_permute");
      break;
    }
    if (tr.is32) {
      rc = ks_bad(jn, "the tail must be int64");
      break;
    }
    // every pass must be a register-kernel pass of 2^6 .. 2^8 points in 64-bit growing ranges
    const bool shapes = inv.size() == 2 && fwd.size() == 2 && fwd[0].args.gdec_power && !fwd[1].args.gdec_power;
    bool ok = shapes;
    for (const auto *v : {&inv, &fwd})
      for (const NttRecorded &r : *v)
        ok = ok && !r.is32 && r.mode == MODE_W64_GROW && r.args.p >= 6 && r.args.p <= 8 && !r.args.store_gather &&
             (r.args.bitrev || (!r.args.load_map && !r.args.store_scatter));
    if (!ok) {
      rc = ks_bad(jn, "the transforms must run in 64-bit growing ranges (moduli below 2^55) with the bit-reversal "
                      "permutation");
      break;
    }
    const NttRecorded *passes[4] = {&inv[0], &inv[1], &fwd[0], &fwd[1]};
    const int cls[4] = {KS_INV, KS_INV, KS_GDEC, KS_FWD};
    for (int k = 0; k < 4; ++k) {
      KsStage &st = js[j].st[k];
      memset(&st, 0, sizeof st);
      st.u.ntt = passes[k]->args;
      ks_retile(st.u.ntt);
      st.ntiles = (uint32_t)(st.u.ntt.nsets * st.u.ntt.l * st.u.ntt.r * st.u.ntt.ngroups_t);
      st.kind = cls[k] | (st.u.ntt.p << 4);
    }
    KsStage &tl = js[j].st[4];
    memset(&tl, 0, sizeof tl);
    tl.u.tail = tr.args;
    tl.ntiles = (uint32_t)((tr.args.n + kKsTailItem - 1) / kKsTailItem);
    tl.kind = KS_TAIL | (tr.len << 8) | (tr.perms32 << 12);
  }
  if (rc) {
    for (void *p : release) scratch_free(p);
    return rc;
  }
  // queue order: stage k of every job, grouped by pass length, before stage k + 1
  std::vector<KsStage> stages;
  std::vector<int> where((size_t)n * 5);
  for (int k = 0; k < 5; ++k) {
    std::vector<int64_t> order((size_t)n);
    for (int64_t j = 0; j < n; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t x, int64_t y) { return js[x].st[k].kind < js[y].st[k].kind; });
    for (int64_t j : order) {
      where[j * 5 + k] = (int)stages.size();
      stages.push_back(js[j].st[k]);
    }
  }
  uint64_t items = 0;
  for (size_t s = 0; s < stages.size(); ++s) stages[s].first = (uint32_t)items, items += stages[s].ntiles;
  if (items >= 0x7FFFFFFFull) {
    for (void *p : release) scratch_free(p);
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_keyswitch_batch: more than 2^31 tiles in one launch");
  }
  // a stage with no tiles (an empty result) counts as finished at once
  for (int64_t j = 0; j < n; ++j)
    for (int k = 0; k < 5; ++k) {
      KsStage &st = stages[where[j * 5 + k]];
      st.dep = k ? where[j * 5 + k - 1] : -1;
      st.hold = g_ks_stall && k == 4 ? 1u : 0u;  // the test hook: the tails wait for a tile that never comes
    }
  const int nst = (int)stages.size();
  void *dstages = nullptr, *state = nullptr;
  rc = scratch_alloc(sizeof(KsStage) * stages.size(), &dstages);
  if (!rc) rc = scratch_alloc(sizeof(uint32_t) * (nst + 2), &state);
  if (!rc && cudaMemcpyAsync(dstages, stages.data(), sizeof(KsStage) * stages.size(), cudaMemcpyHostToDevice,
                             stream()) != cudaSuccess)
    rc = set_error(HEAL_ERR_RUNTIME, "heal_keyswitch_batch: upload of the work list failed");
  if (!rc && cudaMemsetAsync(state, 0, sizeof(uint32_t) * (nst + 2), stream()) != cudaSuccess)
    rc = set_error(HEAL_ERR_RUNTIME, "heal_keyswitch_batch: clearing the counters failed");
  if (!rc && items) {
    static int per_sm = 0;
    if (!per_sm) {
      const size_t smem = (size_t)8 * kKsThreads * sizeof(int64_t);
      HEAL_TRY_CUDA(cudaFuncSetAttribute(keyswitch_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
      int nb = 0;
      HEAL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, keyswitch_batch_kernel, kKsThreads, smem));
      per_sm = std::max(nb, 1);
    }
    const int64_t grid = std::min<int64_t>((int64_t)items, (int64_t)per_sm * device_sm_count());
    const uint32_t spin_limit = g_ks_spin_limit;
    keyswitch_batch_kernel<<<(unsigned)grid, kKsThreads, (size_t)8 * kKsThreads * sizeof(int64_t), stream()>>>(
        (const KsStage *)dstages, nst, (uint32_t)items, (uint32_t *)state, spin_limit, diag_device());
    rc = check_launch("keyswitch_batch");
  }
  scratch_free(dstages);
  scratch_free(state);
  for (void *p : release) scratch_free(p);  // stream-ordered: after the launch
  return rc;
}

}  // namespace heal

using namespace heal;

extern "C" int heal_keyswitch_batch(const heal_keyswitch_job *jobs, int64_t count) {
  clear_error();
  HEAL_CHECK(ensure_init());
  if (capturing()) return set_error(HEAL_ERR_RUNTIME, "heal_keyswitch_batch: not allowed while a graph is being captured");
  if (count < 0 || (count > 0 && !jobs)) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_keyswitch_batch: no jobs");
  if (count > kKsMaxJobs)
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_keyswitch_batch: at most 256 jobs per call");
  if (count == 0) return HEAL_OK;
  // no job may write memory another job uses
  for (int64_t i = 0; i < count; ++i) {
    const heal_keyswitch_job &a = jobs[i];
    for (const heal_tensor *t : {&a.ct, &a.x, &a.digits, &a.result}) HEAL_CHECK(check_desc(t, "job tensor", true));
  }
  for (int64_t i = 0; i < count; ++i)
    for (int64_t j = 0; j < count; ++j) {
      if (i == j) continue;
      const heal_keyswitch_job &a = jobs[i], &b = jobs[j];
      for (const heal_tensor *w : {&a.x, &a.digits, &a.result})
        for (const heal_tensor *u : {&b.ct, &b.x, &b.digits, &b.result, &b.tail_a})
          if (overlaps(*w, *u))
            return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_keyswitch_batch: job " + std::to_string(i) +
                                                            " writes memory job " + std::to_string(j) + " uses");
    }
  return ks_chunk(jobs, count, 0);
}

extern "C" int heal_keyswitch_batch_test_wait(uint32_t spin_limit, int stall) {
  if (spin_limit == 0) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_keyswitch_batch_test_wait: spin_limit must be positive");
  g_ks_spin_limit = spin_limit;
  g_ks_stall = stall != 0;
  return HEAL_OK;
}
