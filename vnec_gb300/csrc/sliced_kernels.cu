// Sliced row-group SpMV (VNEC-S counterpart, src/operation/src/spmv_vnec_S_for_mxv.c:589-660).
//
// One warp per task (sliced.h).  For a ROWS task of vector width VW the warp
// reads `steps` rows of 32 consecutive entries — 256 B of FP64 values and
// 128 B of columns per step, fully coalesced — so lane l accumulates entries
// of group row l / VW; a VW-lane xor-shuffle reduction finishes each row
// (VW = 1: the reference's cross-row kernel, one lane per row, no reduction).
// CHUNK tasks do the same for 32-wide pieces of long rows and a second launch
// adds the pieces of each long row in chunk order.  Loads of values and
// columns are streamed (read once); x is gathered through the read-only path.
// FP64 work: one FMA per entry plus log2(VW) adds per row.

#include <cuda_runtime.h>

#include <cstdint>

#include "common.h"
#include "sliced.h"

namespace vnec {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarpsPerBlock = 8;

template <typename V> __device__ __forceinline__ V fmav(V a, V b, V c);
template <> __device__ __forceinline__ double fmav<double>(double a, double b, double c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fmav<float>(float a, float b, float c) { return fmaf(a, b, c); }

template <typename V, int U>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
sliced_kernel(const SlicedTask* __restrict__ tasks, long long num_tasks, const V* __restrict__ val,
              const int32_t* __restrict__ col, const int32_t* __restrict__ rowid, const V* __restrict__ x,
              V* __restrict__ y, V* __restrict__ chunk_sum) {
  const long long w = ((long long)blockIdx.x * kWarpsPerBlock) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= num_tasks) return;
  const int4 raw = __ldg(reinterpret_cast<const int4*>(tasks) + w);
  const int base = raw.x, row_base = raw.y, steps = raw.z, meta = raw.w;
  const int kind = meta & 15, vwl = (meta >> 4) & 15, nrows = meta >> 8;
  if (kind == kSlicedZero) {
    if (lane < nrows) y[rowid[row_base + lane]] = V(0);
    return;
  }
  const V* vp = val + base + lane;
  const int32_t* cp = col + base + lane;
  V acc = V(0);
  int k = 0;
  for (; k + U <= steps; k += U) {
    int c[U];
    V v[U], xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      c[u] = __ldcs(cp + (k + u) * 32);
      v[u] = __ldcs(vp + (k + u) * 32);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) xv[u] = __ldg(x + c[u]);
#pragma unroll
    for (int u = 0; u < U; ++u) acc = fmav<V>(v[u], xv[u], acc);
  }
  for (; k < steps; ++k) acc = fmav<V>(__ldcs(vp + k * 32), __ldg(x + __ldcs(cp + k * 32)), acc);
  for (int off = (1 << vwl) >> 1; off > 0; off >>= 1) acc += __shfl_xor_sync(kFull, acc, off);
  if (kind == kSlicedChunk) {
    if (lane == 0) chunk_sum[row_base] = acc;
  } else {
    const int g = lane >> vwl;
    if ((lane & ((1 << vwl) - 1)) == 0 && g < nrows) y[rowid[row_base + g]] = acc;
  }
}

template <typename V>
__global__ void sliced_long_fixup(const int32_t* __restrict__ long_row, const int32_t* __restrict__ long_first,
                                  long long num_long, const V* __restrict__ chunk_sum, V* __restrict__ y) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= num_long) return;
  V s = V(0);
  for (int c = long_first[i]; c < long_first[i + 1]; ++c) s += chunk_sum[c];
  y[long_row[i]] = s;
}

template <typename V>
bool launch(const SlicedMatrix& m, const void* x, void* y, cudaStream_t s, cudaEvent_t* ev) {
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[0], s))) return false;
  if (m.num_tasks > 0) {
    const long long grid = (m.num_tasks + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (grid > 0x7fffffffLL) {
      set_error("sliced: too many tasks for one launch");
      return false;
    }
    sliced_kernel<V, 8><<<(unsigned)grid, kWarpsPerBlock * 32, 0, s>>>(
        m.tasks, m.num_tasks, static_cast<const V*>(m.val), m.col, m.rowid, static_cast<const V*>(x),
        static_cast<V*>(y), static_cast<V*>(m.chunk_sum));
    if (!VNEC_CUDA(cudaGetLastError())) return false;
  }
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[1], s))) return false;
  if (m.num_long > 0) {
    const int b = 128;
    sliced_long_fixup<V><<<(unsigned)((m.num_long + b - 1) / b), b, 0, s>>>(
        m.long_row, m.long_first, m.num_long, static_cast<const V*>(m.chunk_sum), static_cast<V*>(y));
    if (!VNEC_CUDA(cudaGetLastError())) return false;
  }
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[2], s))) return false;
  return true;
}

}  // namespace

bool sliced_spmv(const SlicedMatrix& m, bool fp64, const void* x, void* y, cudaStream_t s, cudaEvent_t* ev) {
  return fp64 ? launch<double>(m, x, y, s, ev) : launch<float>(m, x, y, s, ev);
}

}  // namespace vnec
