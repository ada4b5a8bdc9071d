// Batched multi-right-hand-side SpMV kernel (batch.h): one persistent launch
// over the task list of the block-diagonal concatenation of the batch.
//
// Lane l of a warp serves task slot g = l / L and right-hand sides
// [sub * R, sub * R + R) with sub = l % L, R = k / L.  At every step the warp
// reads the G = 32 / L (value, column) pairs of one step (lanes of a slot read
// the same pair, a broadcast) and each lane gathers R consecutive values of
// row `column` of X with 16-byte vector loads, so the L lanes of a slot read
// the whole k-wide X row.  No cross-lane reduction is needed for ROWS tasks:
// every lane owns its own outputs.  CHUNK tasks (pieces of rows longer than
// the grouping limit) spread entries over the G slots; the slots are summed
// with xor-shuffles in FP64 and the last chunk of a row to arrive (an arrival
// counter per long row, reset by that chunk) adds the row's chunk sums in
// chunk order, so no second kernel is needed.
//
// Precision forms: FP64 (FP64 values, X and FMA) and FP32 (FP32 values, X
// rounded to FP32 once per call by a preceding kernel, FP32 products and
// per-lane accumulation; chunk, slot and long-row sums in FP64).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "batch.h"
#include "common.h"

namespace vnec {
namespace {

constexpr unsigned kFull = 0xffffffffu;

struct BatchArgs {
  const int4* tasks;
  long long num_tasks;
  const void* val;
  const int32_t* col;
  const int32_t* rowid;
  const int32_t* long_row;
  const int32_t* long_first;
  const int32_t* chunk_long;
  double* chunk_sum;
  int* chunk_count;
  const void* x;
  double* y;
  int klog2;  // k = 1 << klog2
  int llog2;  // lanes per slot L = 1 << llog2
};

// R consecutive values of X (16-byte vector loads where R allows).
template <typename V, int R> __device__ __forceinline__ void load_x(const V* p, V (&v)[R]) {
  if constexpr (R == 1) {
    v[0] = __ldg(p);
  } else if constexpr (sizeof(V) == 8) {
#pragma unroll
    for (int i = 0; i < R / 2; ++i) {
      const double2 a = __ldg(reinterpret_cast<const double2*>(p) + i);
      v[2 * i] = a.x;
      v[2 * i + 1] = a.y;
    }
  } else if constexpr (R == 2) {
    const float2 a = __ldg(reinterpret_cast<const float2*>(p));
    v[0] = a.x;
    v[1] = a.y;
  } else {
#pragma unroll
    for (int i = 0; i < R / 4; ++i) {
      const float4 a = __ldg(reinterpret_cast<const float4*>(p) + i);
      v[4 * i] = a.x;
      v[4 * i + 1] = a.y;
      v[4 * i + 2] = a.z;
      v[4 * i + 3] = a.w;
    }
  }
}

template <int R> __device__ __forceinline__ void store_y(double* p, const double (&v)[R]) {
  if constexpr (R == 1) {
    p[0] = v[0];
  } else {
#pragma unroll
    for (int i = 0; i < R / 2; ++i) reinterpret_cast<double2*>(p)[i] = make_double2(v[2 * i], v[2 * i + 1]);
  }
}

__device__ __forceinline__ double fmav(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmav(float a, float b, float c) { return fmaf(a, b, c); }

template <typename V, int R, int U>
__global__ void __launch_bounds__(256) batch_kernel(const BatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int k = 1 << a.klog2;
  const int G = 32 >> a.llog2;
  const int g = lane >> a.llog2, sub = lane & ((1 << a.llog2) - 1);
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  const V* __restrict__ val = static_cast<const V*>(a.val);
  const V* __restrict__ xs = static_cast<const V*>(a.x) + sub * R;
  for (long long t = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < a.num_tasks; t += nw) {
    const int4 raw = __ldg(a.tasks + t);
    const int base = raw.x, row_base = raw.y, steps = raw.z, kind = raw.w & 15, nrows = raw.w >> 8;
    if (kind == kSlicedZero) {
      for (int i = lane; i < (nrows << a.klog2); i += 32)
        a.y[((size_t)__ldg(a.rowid + row_base + (i >> a.klog2)) << a.klog2) + (i & (k - 1))] = 0.0;
      continue;
    }
    const V* vp = val + base + g;
    const int32_t* cp = a.col + base + g;
    V acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = V(0);
    int s = 0;
    for (; s + U <= steps; s += U) {
      int c[U];
      V v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        c[u] = __ldcs(cp + (s + u) * G);
        v[u] = __ldcs(vp + (s + u) * G);
      }
      V xv[U][R];
#pragma unroll
      for (int u = 0; u < U; ++u) load_x<V, R>(xs + ((size_t)c[u] << a.klog2), xv[u]);
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] = fmav(v[u], xv[u][r], acc[r]);
    }
    for (; s < steps; ++s) {
      const int c = __ldcs(cp + s * G);
      const V v = __ldcs(vp + s * G);
      V xv[R];
      load_x<V, R>(xs + ((size_t)c << a.klog2), xv);
#pragma unroll
      for (int r = 0; r < R; ++r) acc[r] = fmav(v, xv[r], acc[r]);
    }
    double d[R];
#pragma unroll
    for (int r = 0; r < R; ++r) d[r] = static_cast<double>(acc[r]);
    if (kind == kSlicedChunk) {
      for (int off = 1 << a.llog2; off < 32; off <<= 1)
#pragma unroll
        for (int r = 0; r < R; ++r) d[r] += __shfl_xor_sync(kFull, d[r], off);
      if (g == 0) store_y<R>(a.chunk_sum + ((size_t)row_base << a.klog2) + sub * R, d);
      __threadfence();
      __syncwarp();
      const int li = __ldg(a.chunk_long + row_base);
      const int c0 = __ldg(a.long_first + li), c1 = __ldg(a.long_first + li + 1);
      int last = 0;
      if (lane == 0) last = atomicAdd(a.chunk_count + li, 1) == c1 - c0 - 1;
      last = __shfl_sync(kFull, last, 0);
      if (last) {
        __threadfence();
        const size_t yrow = (size_t)__ldg(a.long_row + li) << a.klog2;
        for (int j = lane; j < k; j += 32) {
          double sum = 0.0;
          for (int c = c0; c < c1; ++c) sum += __ldcg(a.chunk_sum + ((size_t)c << a.klog2) + j);
          a.y[yrow + j] = sum;
        }
        if (lane == 0) a.chunk_count[li] = 0;
      }
    } else if (g < nrows) {
      store_y<R>(a.y + ((size_t)__ldg(a.rowid + row_base + g) << a.klog2) + sub * R, d);
    }
  }
}

template <typename V, int R> constexpr int unroll_for() { return R >= 4 ? 2 : 8 / R; }

template <typename V, int R> void* kernel_ptr() {
  return reinterpret_cast<void*>(&batch_kernel<V, R, unroll_for<V, R>()>);
}

void* pick_kernel(int precision, int r) {
  const bool f32 = precision == kPrecFP32;
  switch (r) {
    case 1: return f32 ? kernel_ptr<float, 1>() : kernel_ptr<double, 1>();
    case 2: return f32 ? kernel_ptr<float, 2>() : kernel_ptr<double, 2>();
    case 4: return f32 ? kernel_ptr<float, 4>() : kernel_ptr<double, 4>();
    case 8: return f32 ? kernel_ptr<float, 8>() : kernel_ptr<double, 8>();
    default: return nullptr;
  }
}

int log2i(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

}  // namespace

int batch_grid(int precision, int rhs_per_lane, int warps_per_block) {
  void* fn = pick_kernel(precision, rhs_per_lane);
  if (!fn || (warps_per_block != 4 && warps_per_block != 8)) return 0;
  int dev = 0, sms = 0, per_sm = 0;
  if (!VNEC_CUDA(cudaGetDevice(&dev)) ||
      !VNEC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) ||
      !VNEC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, warps_per_block * 32, 0)))
    return 0;
  return sms * std::max(per_sm, 1);
}

bool batch_spmm(const BatchMatrix& m, const double* X, double* Y, cudaStream_t s) {
  if (!batch_supported(m.k, m.lanes)) {
    set_error("batch: unsupported k / lanes");
    return false;
  }
  const int R = m.k / m.lanes;
  const void* xin = X;
  if (m.precision == kPrecFP32) {
    if (m.n_cols > 0 && !round_to_f32(X, m.xbuf, (long long)m.n_cols * m.k, s)) return false;
    xin = m.xbuf;
  }
  if (m.num_tasks == 0) return true;
  BatchArgs a;
  a.tasks = reinterpret_cast<const int4*>(m.tasks);
  a.num_tasks = m.num_tasks;
  a.val = m.precision == kPrecFP32 ? static_cast<const void*>(m.val32) : static_cast<const void*>(m.val);
  a.col = m.col;
  a.rowid = m.rowid;
  a.long_row = m.long_row;
  a.long_first = m.long_first;
  a.chunk_long = m.chunk_long;
  a.chunk_sum = m.chunk_sum;
  a.chunk_count = m.chunk_count;
  a.x = xin;
  a.y = Y;
  a.klog2 = log2i(m.k);
  a.llog2 = log2i(m.lanes);
  void* fn = pick_kernel(m.precision, R);
  const int grid = (int)std::min<long long>(m.grid, std::max<long long>(1, (m.num_tasks + 7) / 8));
  void* args[] = {&a};
  return VNEC_CUDA(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3((unsigned)(m.warps_per_block * 32)), args, 0, s));
}

}  // namespace vnec
