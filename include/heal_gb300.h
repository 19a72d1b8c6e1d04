/*
 * heal_gb300.h — C ABI of the GB300 HEAL vendor backend.
 *
 * Every entry point is `extern "C"`, takes plain pointers, sizes and tensor
 * descriptors, and returns an `int` status (0 = success).  On failure the
 * message is available from heal_last_error() and the status names the C++
 * exception type the HEAL API throws for it (HEAL_ERR_INVALID_ARGUMENT ->
 * std::invalid_argument, ...).  No torch or CUDA types appear here.
 *
 * Each function cites the HEAL interface it replaces as
 * `path:line` inside the Lattica-ai/heal project.  The C++ templates of
 * `namespace lattica_hw_api` (the include/ headers of HEAL) and the `lattica_hw`
 * Python module are thin layers over these calls.
 *
 * Execution model: one GPU, one library stream (replaceable with
 * heal_set_stream).  Compute calls are stream-ordered and return once the
 * work is enqueued; results are visible to every later call on the same
 * stream, and heal_d2h / heal_synchronize wait for them.  A call validates
 * its arguments on the host before it enqueues anything, so argument errors
 * leave every output untouched.  Tables that depend on data (a permutation's
 * range, a modulus' constants, a twiddle table's Shoup companions) are
 * derived on the GPU the first time a table is used and cached per
 * allocation; the first use of a permutation table synchronises once so that
 * an out-of-range index is reported by the call that uses it.
 */
#ifndef HEAL_GB300_H
#define HEAL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HEAL_MAX_DIMS 8

/* Element types of DeviceTensor<T>: T = int32_t, int64_t, double. */
typedef enum heal_dtype {
  HEAL_INT32 = 0,
  HEAL_INT64 = 1,
  HEAL_FLOAT64 = 2
} heal_dtype;

/* Status codes; each maps to the exception HEAL's C++ API throws. */
typedef enum heal_status {
  HEAL_OK = 0,
  HEAL_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument */
  HEAL_ERR_OUT_OF_RANGE = 2,     /* std::out_of_range     */
  HEAL_ERR_RUNTIME = 3,          /* std::runtime_error    */
  HEAL_ERR_BAD_ALLOC = 4,        /* std::bad_alloc        */
  HEAL_ERR_CUDA = 5              /* CUDA failure (std::runtime_error) */
} heal_status;

/*
 * A strided view of device memory: the fields of HEAL's DeviceTensor<T>
 * (example_impl/device_memory_impl.h:11-34 — dims, strides, data).
 * `data` is the device address of element (0, ..., 0); strides are in
 * elements and may be 0 (a broadcast axis made by expand/unsqueeze).
 */
typedef struct heal_tensor {
  void *data;
  int32_t dtype; /* heal_dtype */
  int32_t ndim;  /* 0 .. HEAL_MAX_DIMS */
  int64_t dims[HEAL_MAX_DIMS];
  int64_t strides[HEAL_MAX_DIMS];
} heal_tensor;

/* ---------------------------------------------------------------- runtime */

/* Selects the CUDA device and creates the library stream and memory pool.
 * Called implicitly by every other entry point with the current device. */
int heal_init(int device);

/* Message of the last failing call on this thread ("" if none). */
const char *heal_last_error(void);

/* Waits for all enqueued work, then prints (to stderr) the diagnostics
 * kernels recorded since the last synchronisation, e.g. the
 * g_decomposition capacity warnings (g_decomposition_impl.cpp:58-65), and
 * returns HEAL_ERR_RUNTIME if a heal_keyswitch_batch dependency wait ran out
 * since then (the report is consumed: the next call returns HEAL_OK). */
int heal_synchronize(void);

/* The stream every compute call is enqueued on (a cudaStream_t). */
void *heal_get_stream(void);
/* Replaces the library stream by a caller's cudaStream_t (NULL restores the
 * library's own stream). */
int heal_set_stream(void *stream);

/* Number of kernels this library has launched since heal_init (a graph
 * replay counts the kernels it contains). */
uint64_t heal_kernel_launch_count(void);

/* Reference-compatibility mode (off by default).  HEAL's sample
 * implementation computes some sums and the INTT's m^-1 scaling in the
 * element type, so they wrap: the int64 INTT for every modulus above about
 * 2^31.5 (ntt_impl.cpp:165), the int32 NTT and INTT butterflies for moduli
 * of 2^30 and above (ntt_impl.cpp:106-107,155-157), the int32 INTT scaling
 * above about 2^15.5, and axis_modsum's running sum for int32 moduli of 2^30
 * and int64 moduli of 2^62 and above (axis_modsum_impl.cpp:70).  This
 * backend computes the mathematically exact results by default.  With
 * on != 0, heal_ntt, heal_intt and heal_axis_modsum reproduce the sample
 * implementation's wraparound instead (every NTT tile then takes the
 * stage-by-stage exact path, so transforms are much slower), so that outputs
 * equal the sample implementation's bit for bit even where it overflows.
 * The extension ops (modmul_axis_sum, g_decomposition_ntt,
 * modmul_axis_sum_permute, the batches) keep the exact semantics.  A process-
 * wide setting; calls already enqueued are not affected. */
int heal_set_reference_compat(int on);
int heal_get_reference_compat(void);

/* CUDA graphs of HEAL calls.  heal_graph_begin starts capturing the library
 * stream; every compute call until heal_graph_end is recorded instead of run,
 * and heal_graph_end returns an instantiated graph that heal_graph_launch
 * replays on the library stream.  The tables the recorded calls derive from
 * their inputs must already be cached (run each call once before capturing);
 * a call that would have to build one fails during capture.  No counterpart
 * in HEAL: a way to issue a fixed sequence of calls with one launch. */
int heal_graph_begin(void);
int heal_graph_end(void **graph);
int heal_graph_launch(void *graph);
int heal_graph_destroy(void *graph);

/* Parallel branches inside one capture.  heal_graph_fork(n), once per
 * capture, starts n branch streams after everything recorded so far;
 * heal_graph_branch(i) sends the calls that follow to branch i (-1: back to
 * the stream the capture began on).  heal_graph_end joins every branch, so a
 * replay ends when all branches have.  Calls on different branches must not
 * write memory another branch reads or writes.  Synchronising calls
 * (heal_synchronize, heal_d2h, heal_h2d, heal_alloc, heal_free) fail while a
 * capture is open. */
#define HEAL_GRAPH_MAX_BRANCHES 64
int heal_graph_fork(int n);
int heal_graph_branch(int i);

/* ------------------------------------------- device memory (HBM residency)
 * Replaces allocate_on_hardware / host_to_device / device_to_host
 * (include/device_memory.h:24-39; example_impl/device_memory_impl.cpp:168-202). */

/* Allocates `bytes` of HBM (stream-ordered pool).  `zero` != 0 clears it,
 * as allocate_on_hardware's calloc does (device_memory_impl.cpp:171). */
int heal_alloc(size_t bytes, int zero, void **out);
/* Releases memory from heal_alloc (stream-ordered). */
int heal_free(void *ptr);
/* Host -> device copy of `bytes` (pageable or pinned host memory).
 * Enqueued on the library stream; returns when the source may be reused. */
int heal_h2d(void *dst_device, const void *src_host, size_t bytes);
/* Device -> host copy; waits for all earlier work on the stream first and
 * reports its diagnostics as heal_synchronize does. */
int heal_d2h(void *dst_host, const void *src_device, size_t bytes);
/* Asynchronous variants for pinned host memory (no wait). */
int heal_h2d_async(void *dst_device, const void *src_host, size_t bytes);
int heal_d2h_async(void *dst_host, const void *src_device, size_t bytes);
/* Pinned host memory for the async copies. */
int heal_host_alloc(size_t bytes, void **out);
int heal_host_free(void *ptr);
/* Declares that memory from heal_alloc was written by something other than
 * this library, so tables derived from it are rebuilt on their next use. */
int heal_mark_modified(void *ptr);

/* Host-side decoding of a transcript's tensor payload: `len` bytes of
 * base64 text at `src` (RFC 4648 standard alphabet, '=' padding) into `dst`
 * (capacity `cap` bytes), split over up to `threads` host threads (<= 0: one
 * per core, at most 16; runs of 256 KB of text at least); *written = the
 * decoded length.  Replaces the base64.b64decode of HEAL's decode_tensor
 * (python_execution/lattica_heal_runtime/serialization.py:31) on the request
 * path of a server that takes transcripts.  Only the canonical encoding is
 * accepted (length a multiple of 4, padding only at the end, no other
 * characters): anything else, or a `dst` too small, returns
 * HEAL_ERR_INVALID_ARGUMENT, and the caller decodes such text leniently.
 * Touches no GPU. */
int heal_base64_decode(const char *src, size_t len, void *dst, size_t cap, size_t *written, int threads);

/* Strided gather of `src` into `dst` (same dims, any strides, any dtype):
 * the copy inside make_contiguous (include/contiguous.h:19-20;
 * example_impl/contiguous_impl.cpp:9-52). */
int heal_copy_strided(const heal_tensor *src, const heal_tensor *dst);

/* ------------------------------------ stride-only metadata (no GPU access)
 * In-place edits of a descriptor, as DeviceTensor::reshape
 * (device_memory_impl.cpp:42-84) and expand / squeeze / unsqueeze
 * (include/memory_virtual_ops.h:39-86; memory_virtual_ops_impl.cpp:7-86). */
int heal_tensor_reshape(heal_tensor *t, int32_t new_ndim, const int64_t *new_dims);
int heal_tensor_expand(heal_tensor *t, int64_t axis, int64_t repeats);
int heal_tensor_squeeze(heal_tensor *t, int64_t axis);
int heal_tensor_unsqueeze(heal_tensor *t, int64_t axis);
/* Extension (no HEAL counterpart; named by DeviceDispatcher.moveaxis,
 * python_execution/lattica_heal_runtime/device_interface.py:84-85):
 * moves axis `src` to position `dst` by permuting dims and strides. */
int heal_tensor_moveaxis(heal_tensor *t, int64_t src, int64_t dst);
/* Extension: basic slice [start, stop) with positive step along `axis`. */
int heal_tensor_slice(heal_tensor *t, int64_t axis, int64_t start, int64_t stop, int64_t step);
/* 1 if dense row-major ignoring size-1 axes (device_memory_impl.cpp:31-40). */
int heal_tensor_is_contiguous(const heal_tensor *t);
/* Elements spanned by the view: 1 + sum((dims[i]-1)*strides[i])
 * (device_memory_impl.cpp:19-23); 0 if any dim is 0. */
int64_t heal_tensor_span(const heal_tensor *t);

/* ------------------------------------------- modular elementwise arithmetic
 * result = (a op b) % p in the double-width type (int32 -> int64,
 * int64 -> __int128) with C's truncating remainder, broadcasting a, b and p
 * against result's shape (include/modop.h:47-111;
 * example_impl/modop_impl.cpp:108-180,238-239).  Scalars are given as
 * int64_t and converted to the element type, as the templates' T scalars. */
int heal_modmul_ttt(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, const heal_tensor *result);
int heal_modmul_ttc(const heal_tensor *a, const heal_tensor *b, int64_t p, const heal_tensor *result);
int heal_modmul_tct(const heal_tensor *a, int64_t b, const heal_tensor *p, const heal_tensor *result);
int heal_modmul_tcc(const heal_tensor *a, int64_t b, int64_t p, const heal_tensor *result);
int heal_modsum_ttt(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, const heal_tensor *result);
int heal_modsum_ttc(const heal_tensor *a, const heal_tensor *b, int64_t p, const heal_tensor *result);
int heal_modsum_tct(const heal_tensor *a, int64_t b, const heal_tensor *p, const heal_tensor *result);
int heal_modsum_tcc(const heal_tensor *a, int64_t b, int64_t p, const heal_tensor *result);

/* result = a % b with C's remainder in the element type, identical shapes
 * (include/modop.h:115-134; modop_impl.cpp:188-235). */
int heal_mod_tt(const heal_tensor *a, const heal_tensor *b, const heal_tensor *result);
int heal_mod_tc(const heal_tensor *a, int64_t b, const heal_tensor *result);
int heal_mod_ct(int64_t a, const heal_tensor *b, const heal_tensor *result);

/* modmul_ttt without any device allocation, for callers that cannot let a
 * library allocate: a serving process that reserves HBM up front and fails
 * later allocations, a foreign host runtime that owns every device buffer,
 * a loop that must not stall in an allocator.  No counterpart in HEAL.
 * Same result as heal_modmul_ttt, on the caller's `stream` (a cudaStream_t;
 * NULL is the default stream).  The moduli's reduction constants go to one
 * fixed device array of this library (at most 4096 moduli: p with more
 * elements is rejected with HEAL_ERR_INVALID_ARGUMENT), which every GPU that
 * loads the library keeps until the process exits.  The first call on a
 * device looks up that array's device address; make it before any stream
 * capture.  All calls share the array and each overwrites it, so calls that
 * overlap on the GPU (on different streams) race.  A result that overlaps
 * an input in another layout is rejected (it would need a temporary copy).
 * A modulus of 0 gives 0, as in heal_modmul_ttt, but without that call's
 * warning at the next synchronisation.  The result is written on `stream`;
 * when another library call then reads it on the library stream (for
 * instance as moduli or twiddles), order the two streams with an event or a
 * synchronisation first.  A CUDA error left pending on the calling thread by
 * an earlier call is returned as HEAL_ERR_RUNTIME before anything runs. */
int heal_modmul_ttt_noalloc(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p,
                            const heal_tensor *result, void *stream);

/* Extension (DeviceDispatcher._modneg_tt / _modneg_tc,
 * device_interface.py:51-54, which have no backend in HEAL):
 * result = (p - a % p) % p in the double-width type, broadcasting like
 * modsum. */
int heal_modneg_tt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *result);
int heal_modneg_tc(const heal_tensor *a, int64_t p, const heal_tensor *result);

/* Reduction of a non-last axis modulo p[k] (include/axis_modsum.h:24-30;
 * example_impl/axis_modsum_impl.cpp:12-76). */
int heal_axis_modsum(const heal_tensor *a, const heal_tensor *p, const heal_tensor *result, int64_t axis);

/* Base-2^base_bits digits of every element into a new last axis of size
 * `power` (include/g_decomposition.h:24-30; g_decomposition_impl.cpp:10-67). */
int heal_g_decomposition(const heal_tensor *a, const heal_tensor *result, uint64_t power, uint64_t base_bits);

/* Batched negacyclic NTT / INTT over [l, m, r, k] with moduli innermost
 * (include/ntt.h:31-52; example_impl/ntt_impl.cpp:69-170).  log2p and mu
 * may be NULL (HEAL declares them optional and its sample ignores them).
 * The inverse scales by m_inv in the double-width type. */
int heal_ntt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm, const heal_tensor *twiddles,
             const heal_tensor *log2p, const heal_tensor *mu, const heal_tensor *result);
int heal_intt(const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm, const heal_tensor *inv_twiddles,
              const heal_tensor *m_inv, const heal_tensor *log2p, const heal_tensor *mu, const heal_tensor *result);

/* NTT plans.  A plan fixes, for one element type (HEAL_INT32 / HEAL_INT64),
 * direction (inverse 0/1), length m and limb count k, the limbs per CTA tile
 * (1, 2, 4, 8 or 16) and where the butterfly network splits into two passes
 * (first_pass_log2: log2 of the first pass's length, 1..12 with
 * log2(m) - first_pass_log2 in 1..12; 0 = one pass, for m <= 4096).  Without
 * a plan a call uses 4 limbs per tile and one pass up to m = 4096, else an
 * even split.  Plans change speed only; every plan gives the same result.
 * No counterpart in HEAL (example_impl has one loop nest). */
int heal_ntt_set_plan(int dtype, int inverse, int64_t m, int64_t k, int tile_limbs, int first_pass_log2);
/* The plan a call of this shape uses: the one set, else the default. */
int heal_ntt_get_plan(int dtype, int inverse, int64_t m, int64_t k, int *tile_limbs, int *first_pass_log2);
int heal_ntt_clear_plans(void);
/* Times every candidate plan on these operands (heal_ntt when inverse == 0,
 * else heal_intt with m_inv) with `reps` calls each and keeps the fastest for
 * this shape, or the default plan unless the fastest beats it by 3% (near-equal
 * plans swap places between runs); `result` is overwritten.  The choice is returned through
 * tile_limbs / first_pass_log2 (either may be null).  Waits for the GPU; fails
 * while a graph is being captured. */
int heal_ntt_autotune(int inverse, const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm,
                      const heal_tensor *twiddles, const heal_tensor *m_inv, const heal_tensor *result, int reps,
                      int *tile_limbs, int *first_pass_log2);

/* Diagnostic (no HEAL counterpart): the sustained rate, in butterflies per
 * second, of the NTT's 64-bit growing-range forward butterfly with its
 * operands held in registers (groups radix-8 groups of 12 butterflies per
 * thread, 8 CTAs of 128 threads per SM): the integer-pipe ceiling that an NTT
 * pass is compared with.  Waits for the GPU; fails while a graph is being
 * captured. */
int heal_ntt_butterfly_peak(int groups, double *butterflies_per_s);

/* Per-row gather along perm_axis with indices perms[l, m]
 * (include/permute.h:33-40; example_impl/permute_impl.cpp:8-65). */
int heal_permute(const heal_tensor *a, const heal_tensor *perms, const heal_tensor *result, int64_t elementwise_axis,
                 int64_t perm_axis);

/* Fused multiply-reduce, the backend op behind HEAL's DeviceDispatcher
 * modmul_axis_sum (python_execution/lattica_heal_runtime/device_interface.py:
 * 67-68, which names the op only).  Defined as the composition
 *   result = axis_modsum(modmul(a', b, p), axis)
 * with a and b broadcast like modmul to a common shape S (result's shape with
 * `axis` re-inserted; axis in [0, ndim(S) - 2]; p of shape [S[-1]]), and
 * a' = a when perms is NULL, else a gathered like permute with
 * elementwise_axis = axis: a'[c] = a[c with c[perm_axis] <- perms[c[axis],
 * c[perm_axis]]], perms of shape [S[axis], S[perm_axis]].  Perms of shape
 * [S[axis], S[perm_axis], S[perm_axis + 1]] (linear across its last two
 * axes) gather over the two axes taken as one flattened axis, a linear
 * across them: permute of a with those axes reshaped into one.
 * Bit-identical to the separate calls; the product is never written.
 * Errors as axis_modsum / permute. */
int heal_modmul_axis_sum(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, const heal_tensor *perms,
                         int64_t perm_axis, const heal_tensor *result, int64_t axis);

/* A ragged batch of transforms in few launches (an extension: HEAL has no
 * batch call).  Job i is the heal_ntt (inverse = 0) or heal_intt
 * (inverse = 1) call with a = jobs[i].a, p, perm, twiddles (the inverse
 * twiddles for inverse = 1), m_inv (read for inverse = 1 only) and result;
 * the jobs may differ in every shape (ring degree, limb count, batch axes),
 * element type and table.  Results are bit-identical to the calls one by
 * one.  No job's result may overlap another job's input or result
 * (invalid_argument; a job's result may alias its own input as in heal_ntt).
 * Every job is validated, with the errors of heal_ntt / heal_intt, before
 * anything is enqueued.  The passes of all jobs are launched grouped by
 * kernel class (element type, arithmetic mode, pass length, tile width), up
 * to 64 passes per launch with their arguments in the launch parameters, so
 * the batch can be recorded in a CUDA graph like any call. */
typedef struct heal_ntt_job {
  heal_tensor a, p, perm, twiddles, m_inv, result;
} heal_ntt_job;
int heal_ntt_batch(int inverse, const heal_ntt_job *jobs, int64_t count);

/* Many fused keyswitch steps, of any ring degree 2^12 .. 2^16 and limb
 * count, in one persistent launch (an extension: HEAL has no such op; each
 * step is the composition of HEAL's intt, g_decomposition, ntt, modmul,
 * axis_modsum and permute, example_impl/ntt_impl.cpp:69-170,
 * g_decomposition_impl.cpp:10-67, modop_impl.cpp:44-101,
 * axis_modsum_impl.cpp:12-76, permute_impl.cpp:8-65).  Job i is the three
 * calls
 *   heal_intt(ct, p, perm, inv_twiddles, m_inv, NULL, NULL, x)
 *   heal_g_decomposition_ntt(x, power, base_bits, p_digits, perm, twiddles_digits, digits)
 *   heal_modmul_axis_sum_permute(tail_a, tail_b, p, tail_axis, galois, elementwise_axis, perm_axis, result)
 * and the results are bit-identical to making them job after job.  Every
 * job is validated, with those calls' errors, before anything is enqueued;
 * beyond them: int64 tensors, moduli below 2^55 (the transforms' 64-bit
 * growing ranges), the bit-reversal permutation, a tail that takes the lean
 * kernel (at most 4 terms), at most 256 jobs, and no job writing (x, digits,
 * result) memory another job uses.  Tiles of all stages of all jobs run in
 * one kernel whose waits on the previous stage of the same job are bounded;
 * a wait that runs out makes the next heal_synchronize return
 * HEAL_ERR_RUNTIME.  Not allowed while a graph is being captured. */
typedef struct heal_keyswitch_job {
  heal_tensor ct, p, perm, inv_twiddles, m_inv, x;
  int64_t power, base_bits;
  heal_tensor p_digits, twiddles_digits, digits;
  heal_tensor tail_a, tail_b;
  int64_t tail_axis;
  heal_tensor galois;
  int64_t elementwise_axis, perm_axis;
  heal_tensor result;
} heal_keyswitch_job;
int heal_keyswitch_batch(const heal_keyswitch_job *jobs, int64_t count);

/* Test hook of heal_keyswitch_batch's failure path (no counterpart in
 * HEAL): later batches give up a dependency wait after spin_limit polls of
 * 256 ns (default 2^22, about a second), and with stall != 0 every job's
 * tail waits for one tile more than its previous stage has, so those waits
 * run out and the next heal_synchronize returns HEAL_ERR_RUNTIME.  Call it
 * again with stall = 0 (and the default limit) to restore normal runs. */
int heal_keyswitch_batch_test_wait(uint32_t spin_limit, int stall);

/* The head of a keyswitch's digit transform in one call (an extension: HEAL
 * has no such op).  Defined as the composition of HEAL's own calls
 *   result = ntt(reshape(g_decomposition(a, power, base_bits),
 *                        [l, m, r, k * power]), p, perm, twiddles)
 * (example_impl/g_decomposition_impl.cpp:10-67, ntt_impl.cpp:69-116) for a of
 * shape [l, m, r, k]: digit limb t * power + d is digit d of source limb t,
 * p has shape [k * power] and twiddles [k * power, m].  The first pass of the
 * transform reads a and extracts each digit as it loads, so the digit tensor
 * is never written.  Bit-identical to the two calls, including
 * g_decomposition's capacity warnings (printed at the next synchronisation).
 * Errors as g_decomposition / ntt; result must have shape [l, m, r, k * power]. */
int heal_g_decomposition_ntt(const heal_tensor *a, int64_t power, int64_t base_bits, const heal_tensor *p,
                             const heal_tensor *perm, const heal_tensor *twiddles, const heal_tensor *result);

/* The tail of a keyswitch in one pass (an extension: HEAL has no such op).
 * Defined as the composition of HEAL's own calls
 *   result = permute(axis_modsum(modmul(a, b, p), axis), perms,
 *                    elementwise_axis, perm_axis)
 * (example_impl/modop_impl.cpp:44-101, axis_modsum_impl.cpp:12-76,
 * permute_impl.cpp:8-65): a and b broadcast like modmul to a common shape S,
 * axis in [0, ndim(S) - 2], p of shape [S[-1]], and elementwise_axis /
 * perm_axis numbered in result's axes (S without `axis`), perms of shape
 * [result.dims[elementwise_axis], result.dims[perm_axis]].  A permutation
 * gathers whole rows along perm_axis, so each result element is the running
 * sum over `axis` of a * b at its source row; the product and the unpermuted
 * sum are never written.  Bit-identical to the three calls.  Errors as
 * modmul / axis_modsum / permute; indices are checked before anything is
 * written. */
int heal_modmul_axis_sum_permute(const heal_tensor *a, const heal_tensor *b, const heal_tensor *p, int64_t axis,
                                 const heal_tensor *perms, int64_t elementwise_axis, int64_t perm_axis,
                                 const heal_tensor *result);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* HEAL_GB300_H */
