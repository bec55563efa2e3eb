// Library-internal functions shared between translation units; not part of
// the C ABI (include/hitengpu.h).
#pragma once

#include "hitengpu.h"

namespace hg_internal {

// The handle's grow-only device buffer of hg_correct_halo: at least `bytes`
// (allocated, and counted, only when the buffer is smaller).
int correct_buffers(hg_handle* h, long long bytes, void** out);
// hg_reserve from inside the library.
int reserve_refine(hg_handle* h, int N, int dim, int max_hits);
// Record `msg` as the handle's last error and return `code`.
int fail_msg(hg_handle* h, int code, const char* msg);
// The handle's slot for the device corrector's cached graph; free_fn
// releases it when the handle is destroyed.
void** graph_slot(hg_handle* h, void (*free_fn)(void*));
// Add n to the handle's kernel-launch counter.
void count_launches(hg_handle* h, long long n);
// The handle's device ordinal and a tuning value (hg_set_tuning keys).
int device_of(const hg_handle* h);
int tuning(const hg_handle* h, int key);

}  // namespace hg_internal
