// The sliced kernels' long-row fix-up: y[row] = the sum of the row's chunk
// sums, for every row cut into chunks.
//
// Blocks [0, g.light) give one thread to each long row of at most
// kHeavyChunks chunks, summed in chunk order.  Blocks [g.light, g.total)
// give one warp to each heavy row (SlicedMatrix::long_heavy): lane l sums
// chunks l, l + 32, ... and a fixed xor tree joins the lanes.  A thread per
// row for every row made the launch as long as the longest row's serial sum
// (R-MAT 2^24: 55,454 long rows, median 2 chunks, longest 233, ~20 us per
// call); heavy rows cluster at the hub end of a power-law matrix, so a warp
// cannot take its own threads' heavy rows in turn either.  The order is
// fixed by the layout: every call gives the same bits.
#pragma once

#include <cstdint>

#include "sliced.h"

namespace vnec {

// out(i, s) stores long row i's sum s.
template <typename V, typename Out>
__device__ __forceinline__ void long_rows_fixup(const int32_t* __restrict__ long_first,
                                                const int32_t* __restrict__ long_heavy, long long num_long,
                                                long long num_heavy, long long heavy_sub, unsigned light_blocks,
                                                const V* __restrict__ chunk_sum, Out out) {
  if (blockIdx.x < light_blocks) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num_long) return;
    const int c0 = long_first[i], c1 = long_first[i + 1];
    if (c1 - c0 > kHeavyChunks) return;  // a warp of the heavy blocks sums it
    V s = V(0);
#pragma unroll 4
    for (int c = c0; c < c1; ++c) s += chunk_sum[c];
    out(i, s);
    return;
  }
  const long long w = ((long long)(blockIdx.x - light_blocks) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= num_heavy) return;  // whole warps: blockDim.x is a multiple of 32
  const long long i = long_heavy[w] - heavy_sub;
  const int c0 = long_first[i], c1 = long_first[i + 1];
  V s = V(0);
  for (int c = c0 + lane; c < c1; c += 32) s += chunk_sum[c];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) out(i, s);
}

}  // namespace vnec
