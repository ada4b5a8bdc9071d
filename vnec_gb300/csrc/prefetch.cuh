// L2 prefetch of a stream ahead of the sliced kernels' tasks.
//
// Tasks tile the entry arrays in order, so a warp that prefetches the entries
// a fixed distance past its own task's, as many as its own, covers with the
// other warps the whole stream that distance ahead of the tasks running now.
// The lanes issue one `prefetch.global.L2` per 128-byte line: no registers
// stay busy waiting, and the values reach L2 before their task starts.  On
// stream-bound layouts (local columns: stencils, bands; every form, FP64
// included) this takes the latency of HBM off the warps' chains; on
// gather-bound ones (power-law columns) it only adds requests to the L2's
// limiting request rate, so plans enable it by layout.
#pragma once

#include <cstdint>

#include "sliced.h"

namespace vnec {

// Every line holding one of the n items at p (all in bounds).
template <typename T>
__device__ __forceinline__ void prefetch_l2_range(const T* p, long long n, int lane) {
  const char* a = reinterpret_cast<const char*>(p);
  const long long lines = (n * (long long)sizeof(T) + 127) / 128;
  for (long long l = lane; l < lines; l += 32) asm volatile("prefetch.global.L2 [%0];" ::"l"(a + 128 * l));
}

// Lanes 0-3: the descriptor, first column, row slot and shared-pattern line
// of the task about `pf.entries` ahead (row slots only for tasks that have
// them: not CHUNK tasks, whose row_base is a chunk id).
__device__ __forceinline__ void prefetch_l2_task_meta(const SlicedPrefetch& pf, long long w, int base, int row_base,
                                                      bool row_slots, const SlicedTask* tasks,
                                                      const int32_t* first, const int32_t* rowid,
                                                      const uint16_t* pat16, int lane) {
  const char* a = nullptr;
  if (lane == 0) {
    const long long t = w + pf.tasks;
    if (t < pf.n_tasks) a = reinterpret_cast<const char*>(tasks + t);
  } else if (lane == 1 || lane == 2) {
    const long long r = (long long)row_base + pf.rows;
    const int32_t* arr = lane == 1 ? first : rowid;
    if (row_slots && arr && r < pf.n_rows) a = reinterpret_cast<const char*>(arr + r);
  } else if (lane == 3) {
    const long long q = ((long long)base + pf.entries) >> 5;
    if (pat16 && q < (pf.n_entries >> 5)) a = reinterpret_cast<const char*>(pat16 + q);
  }
  if (a) asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
}

}  // namespace vnec
