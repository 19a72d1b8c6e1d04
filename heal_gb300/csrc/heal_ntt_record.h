// heal_ntt_record.h — an NTT / INTT call's passes recorded instead of
// launched (heal_keyswitch_batch runs them inside its persistent kernel).
#pragma once
#include <vector>

#include "heal_ntt_kernels.cuh"

namespace heal {

struct NttRecorded {
  NttArgs args;     // the pass as the register kernel would run it
  int64_t nblocks;  // its tiles
  int mode;         // arithmetic mode (MODE_*)
  bool inv, is32;
};

// Validates and prepares heal_ntt / heal_intt (gdec_power > 0:
// heal_g_decomposition_ntt) as the call itself does, splitting the transform
// after first_log stages (0: the plan's split), and appends its passes to
// *out in order; scratch buffers the passes use go to *release, to be freed
// (stream-ordered) after the passes are enqueued.  Derived tables are built
// (enqueued) as for the call.
int ntt_record(bool inv, const heal_tensor *a, const heal_tensor *p, const heal_tensor *perm, const heal_tensor *tw,
               const heal_tensor *minv, const heal_tensor *res, int64_t gdec_power, int64_t gdec_bits, int first_log,
               std::vector<NttRecorded> *out, std::vector<void *> *release);

}  // namespace heal
