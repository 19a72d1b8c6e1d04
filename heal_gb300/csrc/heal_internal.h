// heal_internal.h — shared declarations of the backend's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/heal_gb300.h"
#include "heal_arith.h"

namespace heal {

// ------------------------------------------------------------ error state
int set_error(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
void clear_error();

#define HEAL_TRY_CUDA(call)                                  \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return ::heal::cuda_fail(e_, #call); \
  } while (0)

#define HEAL_CHECK(expr)        \
  do {                          \
    int rc_ = (expr);           \
    if (rc_) return rc_;        \
  } while (0)

// ----------------------------------------------------------------- runtime
int ensure_init();
// heal_set_reference_compat: reproduce the sample implementation's wraparound
bool reference_compat();
cudaStream_t stream();
bool capturing();  // a graph capture is open
int device_sm_count();
void note_launch(int n = 1);
// checks the launch that was just enqueued
int check_launch(const char *what);

// Stream-ordered scratch memory from the library pool (not registered).
int scratch_alloc(size_t bytes, void **out);
void scratch_free(void *p);

// Write generations of allocations made by heal_alloc.  A table derived from
// a tensor stays valid while the generation of the tensor's allocation does.
uint64_t generation_of(const void *p);  // 0 = memory not from heal_alloc
void mark_written(const void *p);

// --------------------------------------------------------- diagnostics
// Records kernels leave for the host; printed at the next synchronisation.
struct DiagRecord {
  int64_t coord[HEAL_MAX_DIMS];
  int32_t ndim;
  int32_t kind;  // 1 = g_decomposition capacity warning, 2 = zero modulus
  uint64_t base_bits, power;
};
constexpr int kDiagRecords = 32;
struct Diag {
  unsigned long long count;  // total events
  unsigned long long zero_mod;
  unsigned long long wait_timeouts;  // dependency waits of heal_keyswitch_batch that ran out
  DiagRecord rec[kDiagRecords];
};
Diag *diag_device();

// --------------------------------------------------------------- helpers
int64_t numel(const heal_tensor &t);
bool same_dims(const heal_tensor &a, const heal_tensor &b);
int elem_size(int dtype);
int check_desc(const heal_tensor *t, const char *label, bool integer_only);
// [lo, hi) byte range the view touches; empty if numel == 0
void byte_range(const heal_tensor &t, uintptr_t *lo, uintptr_t *hi);
bool overlaps(const heal_tensor &a, const heal_tensor &b);
bool identical_view(const heal_tensor &a, const heal_tensor &b);
int copy_strided_impl(const heal_tensor &src, const heal_tensor &dst);
// dense row-major copy of `t` into fresh scratch memory (caller frees)
int materialize(const heal_tensor &t, heal_tensor *out, void **owned);

// ------------------------------------------------------- derived tables
// Möller-Granlund constants of every element of a modulus tensor, in the
// tensor's logical row-major order.  Element type MG64 (int64) or MG32.
struct ModTable {
  const void *consts;
  int64_t count;
};
int mod_table(const heal_tensor &p, ModTable *out);

// Moduli summary of a [k] tensor (first use synchronises once).
struct ModInfo {
  int64_t min_q, max_q;
  const int64_t *q;        // device, [k] int64 copy of the moduli
  const uint64_t *qone;    // device, [k] floor(2^64 / q) (2^64 - 1 for q = 1)
};
int mod_info(const heal_tensor &p, ModInfo *out);

// Shoup companions of a [k, m] twiddle table against moduli p (dense
// [k][m] pairs of 32-bit or 64-bit words) plus a device flag that is set
// when some twiddle is negative (the exact path is then taken).
struct TwiddleTable {
  const void *pairs;
  const int32_t *rowmap;  // limb -> row of `pairs`; rows of equal content are stored once (null: identity)
  const int *neg_flag;
  int wide;
};
int twiddle_table(const heal_tensor &tw, const heal_tensor &p, int wide, TwiddleTable *out);

// Shoup pairs of m_inv[t] mod q_t, flag set when some m_inv is negative.
int minv_table(const heal_tensor &minv, const heal_tensor &p, int64_t k, int wide, TwiddleTable *out);

// A permutation [m] validated once: perm32[u], inv32[v] = largest u with
// perm[u] == v (or -1), whether it is a bijection, and whether it is the
// bit reversal of the index (then kernels compute it instead of loading it).
struct PermInfo {
  const int32_t *perm32;
  const int32_t *inv32;
  bool bijective;
  bool bad;        // some index outside [0, m)
  int bitrev_log;  // log2(m) when perm[u] is the bit reversal of u over log2(m) bits (its own inverse), else 0
};
int perm_info(const heal_tensor &perm, PermInfo *out);

// Per-row gather tables for permute: validated once per perms tensor.
int perms_valid(const heal_tensor &perms, int64_t m, bool *ok);

}  // namespace heal

#include "heal_view.h"
