// Sliced row-group SpMV (VNEC-S counterpart, src/operation/src/spmv_vnec_S_for_mxv.c:589-660).
//
// One warp per task (sliced.h).  For a ROWS task of vector width VW the warp
// reads `steps` rows of 32 consecutive entries — 256 B of FP64 values and
// 128 B of columns per step, fully coalesced — so lane l accumulates entries
// of group row l / VW; a VW-lane xor-shuffle reduction finishes each row
// (VW = 1: the reference's cross-row kernel, one lane per row, no reduction).
// CHUNK tasks do the same for 32-wide pieces of long rows and a second launch
// adds the pieces of each long row in chunk order.  Values and columns are
// read once (no L1 allocation, L2 evict-first policy); x is gathered through
// the read-only path with evict-last policies.
// FP64 work: one FMA per entry plus log2(VW) adds per row.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "common.h"
#include "long_rows.cuh"
#include "prefetch.cuh"
#include "sliced.h"

namespace vnec {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarpsPerBlock = 8;

// Loads with explicit cache policies (hint 1): values and columns are read
// once — no L1 allocation, L2 policy evict_first — while x is kept (L1
// evict_last, L2 policy evict_last) so its hot part stays cached across tasks.
struct Policies {
  unsigned long long once, keep;
};
__device__ __forceinline__ Policies make_policies() {
  Policies p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p.once));
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p.keep));
  return p;
}
__device__ __forceinline__ double ld_once(const double* p, unsigned long long pol) {
  double v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ float ld_once(const float* p, unsigned long long pol) {
  float v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ int ld_once(const int* p, unsigned long long pol) {
  int v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double ld_keep(const double* p, unsigned long long pol) {
  double v;
  asm("ld.global.nc.L1::evict_last.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ float ld_keep(const float* p, unsigned long long pol) {
  float v;
  asm("ld.global.nc.L1::evict_last.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}

// Streamed value/column loads with no L1 allocation and no L2 policy.
__device__ __forceinline__ double ld_na(const double* p) {
  double v;
  asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_na(const float* p) {
  float v;
  asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ int ld_na(const int* p) {
  int v;
  asm("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_l1_keep(const double* p) {
  double v;
  asm("ld.global.nc.L1::evict_last.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_l1_keep(const float* p) {
  float v;
  asm("ld.global.nc.L1::evict_last.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}

// Cache-hint variants H: 0 streaming (.cs) loads of values/columns and
// read-only x gathers; 1 explicit L1/L2 policies; 2 values/columns without L1
// allocation; 3 as 2 with x gathers marked L1 evict-last.
template <int H, typename T> __device__ __forceinline__ T ld_stream_h(const T* p, const Policies& pol) {
  if constexpr (H == 0) return __ldcs(p);
  else if constexpr (H == 1) return ld_once(p, pol.once);
  else return ld_na(p);
}
template <int H, typename T> __device__ __forceinline__ T ld_x_h(const T* p, const Policies& pol) {
  if constexpr (H == 0 || H == 2) return __ldg(p);
  else if constexpr (H == 1) return ld_keep(p, pol.keep);
  else return ld_l1_keep(p);
}


template <typename V> __device__ __forceinline__ V fmav(V a, V b, V c);
template <> __device__ __forceinline__ double fmav<double>(double a, double b, double c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fmav<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Dense-block entries (VNEC-D counterpart): 4 consecutive values starting at
// column c; x is read at c..c+3 (guarded by n_cols).
template <typename V> struct Quad;
template <> struct Quad<double> {
  __device__ static void load(const double* p, double (&v)[4]) {
    const double2 a = __ldcs(reinterpret_cast<const double2*>(p));
    const double2 b = __ldcs(reinterpret_cast<const double2*>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
};
template <> struct Quad<float> {
  __device__ static void load(const float* p, float (&v)[4]) {
    const float4 a = __ldcs(reinterpret_cast<const float4*>(p));
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  }
};

template <typename V>
__device__ __forceinline__ V block_dot(const V* vp, int c, const V* __restrict__ x, int n_cols, V acc) {
  V v[4];
  Quad<V>::load(vp, v);
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const V xv = (c + l < n_cols) ? __ldg(x + c + l) : V(0);
    acc = fmav<V>(v[l], xv, acc);
  }
  return acc;
}

template <typename V>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
dense_block_kernel(const SlicedTask* __restrict__ tasks, long long num_tasks, const V* __restrict__ val,
                   const int32_t* __restrict__ col, const int32_t* __restrict__ rowid, const V* __restrict__ x,
                   int n_cols, V* __restrict__ y, V* __restrict__ chunk_sum) {
  const long long w = ((long long)blockIdx.x * kWarpsPerBlock) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= num_tasks) return;
  const int4 raw = __ldg(reinterpret_cast<const int4*>(tasks) + w);
  const int base = raw.x, row_base = raw.y, steps = raw.z, meta = raw.w;
  const int kind = meta & 15, vwl = (meta >> 4) & 15, nrows = (meta >> 8) & 0xff;
  if (kind == kSlicedZero) {
    if (lane < nrows) y[rowid[row_base + lane]] = V(0);
    return;
  }
  const V* vp = val + (size_t)(base + lane) * 4;
  const int32_t* cp = col + base + lane;
  V acc = V(0);
  int k = 0;
  for (; k + 4 <= steps; k += 4) {
    int c[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) c[u] = __ldcs(cp + (k + u) * 32);
#pragma unroll
    for (int u = 0; u < 4; ++u) acc = block_dot<V>(vp + (size_t)(k + u) * 128, c[u], x, n_cols, acc);
  }
  for (; k < steps; ++k) acc = block_dot<V>(vp + (size_t)k * 128, __ldcs(cp + k * 32), x, n_cols, acc);
  for (int off = (1 << vwl) >> 1; off > 0; off >>= 1) acc += __shfl_xor_sync(kFull, acc, off);
  if (kind == kSlicedChunk) {
    if (lane == 0) chunk_sum[row_base] = acc;
  } else {
    const int g = lane >> vwl;
    if ((lane & ((1 << vwl) - 1)) == 0 && g < nrows) y[rowid[row_base + g]] = acc;
  }
}

// Address of x for a (possibly hot-relabelled) column.
template <bool HOT, typename V>
__device__ __forceinline__ const V* x_at(const V* __restrict__ x, const V* __restrict__ xh, int ncols, int c) {
  if constexpr (HOT) return c < ncols ? x + c : xh + (c - ncols);
  else return x + c;
}

// Output of row `row`: the sum, or alpha * sum + beta * z[row] + gamma.
// z is not restrict-qualified: it may alias y (the thread reads z[row] before
// it writes y[row], and no other thread touches that entry).
template <bool EPI, typename V>
__device__ __forceinline__ V epi_out(V acc, int row, const SlicedEpilogue& ep) {
  if constexpr (EPI) {
    const double g = ep.gamma_dev ? fma(ep.gamma_dev_scale, *ep.gamma_dev, ep.gamma) : ep.gamma;
    double r = fma(ep.alpha, static_cast<double>(acc), g);
    if (ep.z) r = fma(ep.beta, static_cast<double>(static_cast<const V*>(ep.z)[row]), r);
    return static_cast<V>(r);
  } else {
    return acc;
  }
}

// One warp task (the body of sliced_kernel and of the DF32 guard kernel).
template <typename V, int U, int H, bool HOT, bool EPI>
__device__ __forceinline__ void sliced_task(long long w, int lane, const SlicedTask* __restrict__ tasks,
                                            const V* __restrict__ val, const int32_t* __restrict__ col,
                                            const int32_t* __restrict__ rowid, const V* __restrict__ x, V* y,
                                            V* __restrict__ chunk_sum, const V* __restrict__ xh, int ncols,
                                            const SlicedEpilogue& ep, const uint16_t* __restrict__ col16,
                                            const int32_t* __restrict__ first,
                                            const SlicedPrefetch& pf = SlicedPrefetch()) {
  const int4 raw = __ldg(reinterpret_cast<const int4*>(tasks) + w);
  const int base = raw.x, row_base = raw.y, steps = raw.z, meta = raw.w;
  const int kind = meta & 15, vwl = (meta >> 4) & 15, nrows = (meta >> 8) & 0xff;
  // The entries and task metadata ahead of this task, into L2 (prefetch.cuh).
  if (pf.entries > 0) {
    prefetch_l2_task_meta(pf, w, base, row_base, kind != kSlicedChunk, tasks, first, rowid, nullptr, lane);
    const long long e0 = base + pf.entries, len = 32LL * steps;
    if (kind != kSlicedZero && e0 + len <= pf.n_entries) {
      prefetch_l2_range(val + e0, len, lane);
      if (meta & kSlicedDelta)
        prefetch_l2_range(col16 + e0, len, lane);
      else
        prefetch_l2_range(col + e0, len, lane);
    }
  }
  if (kind == kSlicedZero) {
    if (lane < nrows) {
      const int row = rowid[row_base + lane];
      y[row] = epi_out<EPI>(V(0), row, ep);
    }
    return;
  }
  if (meta & kSlicedDelta) {
    // One row per lane, columns as 16-bit deltas from the row's first column.
    const V* vp = val + base + lane;
    const uint16_t* dp = col16 + base + lane;
    int c = lane < nrows ? __ldg(first + row_base + lane) : 0;
    V acc = V(0);
    int k = 0;
    for (; k + U <= steps; k += U) {
      int cc[U];
      V v[U], xv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        cc[u] = __ldcs(dp + (k + u) * 32);
        v[u] = __ldcs(vp + (k + u) * 32);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        c += cc[u];
        cc[u] = c;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) xv[u] = __ldg(x_at<HOT>(x, xh, ncols, cc[u]));
#pragma unroll
      for (int u = 0; u < U; ++u) acc = fmav<V>(v[u], xv[u], acc);
    }
    for (; k < steps; ++k) {
      c += __ldcs(dp + k * 32);
      acc = fmav<V>(__ldcs(vp + k * 32), __ldg(x_at<HOT>(x, xh, ncols, c)), acc);
    }
    if (lane < nrows) {
      const int row = rowid[row_base + lane];
      y[row] = epi_out<EPI>(acc, row, ep);
    }
    return;
  }
  const V* vp = val + base + lane;
  const int32_t* cp = col + base + lane;
  Policies pol{0, 0};
  if constexpr (H == 1) pol = make_policies();
  V acc = V(0);
  int k = 0;
  for (; k + U <= steps; k += U) {
    int c[U];
    V v[U], xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      c[u] = ld_stream_h<H>(cp + (k + u) * 32, pol);
      v[u] = ld_stream_h<H>(vp + (k + u) * 32, pol);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) xv[u] = ld_x_h<H>(x_at<HOT>(x, xh, ncols, c[u]), pol);
#pragma unroll
    for (int u = 0; u < U; ++u) acc = fmav<V>(v[u], xv[u], acc);
  }
  for (; k < steps; ++k)
    acc = fmav<V>(ld_stream_h<H>(vp + k * 32, pol),
                  ld_x_h<H>(x_at<HOT>(x, xh, ncols, ld_stream_h<H>(cp + k * 32, pol)), pol), acc);
  for (int off = (1 << vwl) >> 1; off > 0; off >>= 1) acc += __shfl_xor_sync(kFull, acc, off);
  if (kind == kSlicedChunk) {
    if (lane == 0) chunk_sum[row_base] = acc;
  } else {
    const int g = lane >> vwl;
    if ((lane & ((1 << vwl) - 1)) == 0 && g < nrows) {
      const int row = rowid[row_base + g];
      y[row] = epi_out<EPI>(acc, row, ep);
    }
  }
}

template <typename V, int U, int H, bool HOT = false, bool EPI = false>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
sliced_kernel(const SlicedTask* __restrict__ tasks, long long num_tasks, const V* __restrict__ val,
              const int32_t* __restrict__ col, const int32_t* __restrict__ rowid, const V* __restrict__ x,
              V* y, V* __restrict__ chunk_sum, const V* __restrict__ xh = nullptr, int ncols = 0,
              SlicedEpilogue ep = SlicedEpilogue(), const uint16_t* __restrict__ col16 = nullptr,
              const int32_t* __restrict__ first = nullptr, SlicedPrefetch pf = SlicedPrefetch()) {
  const long long w = ((long long)blockIdx.x * kWarpsPerBlock) + (threadIdx.x >> 5);
  if (w >= num_tasks) return;
  sliced_task<V, U, H, HOT, EPI>(w, threadIdx.x & 31, tasks, val, col, rowid, x, y, chunk_sum, xh, ncols, ep, col16,
                                 first, pf);
}

// FP64 recompute of a DF32 call whose x left the split range: a small grid of
// warps striding the task list, so that the launch costs next to nothing in
// the usual case (flag clear: every block returns at once).
template <bool HOT>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
sliced_guard_kernel(const int* __restrict__ guard, const SlicedTask* __restrict__ tasks, long long num_tasks,
                    const double* __restrict__ val, const int32_t* __restrict__ col,
                    const int32_t* __restrict__ rowid, const double* __restrict__ x, double* y,
                    double* __restrict__ chunk_sum, const double* __restrict__ xh, int ncols,
                    const uint16_t* __restrict__ col16, const int32_t* __restrict__ first) {
  if (*reinterpret_cast<const volatile int*>(guard) == 0) return;
  const SlicedEpilogue ep;
  const long long stride = (long long)gridDim.x * kWarpsPerBlock;
  for (long long w = (long long)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); w < num_tasks; w += stride)
    sliced_task<double, 8, 0, HOT, false>(w, threadIdx.x & 31, tasks, val, col, rowid, x, y, chunk_sum, xh, ncols,
                                          ep, col16, first);
}

template <typename V, bool EPI = false>
__global__ void sliced_long_fixup(const int32_t* __restrict__ long_row, const int32_t* __restrict__ long_first,
                                  const int32_t* __restrict__ long_heavy, long long num_long, long long num_heavy,
                                  long long heavy_sub, unsigned light_blocks, const V* __restrict__ chunk_sum, V* y,
                                  SlicedEpilogue ep = SlicedEpilogue()) {
  long_rows_fixup<V>(long_first, long_heavy, num_long, num_heavy, heavy_sub, light_blocks, chunk_sum,
                     [&](long long i, V s) {
                       const int row = long_row[i];
                       y[row] = epi_out<EPI>(s, row, ep);
                     });
}

template <typename V>
__global__ void epilogue_kernel(V* y, long long n, SlicedEpilogue ep) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double g = ep.gamma_dev ? fma(ep.gamma_dev_scale, *ep.gamma_dev, ep.gamma) : ep.gamma;
    double r = fma(ep.alpha, static_cast<double>(y[i]), g);
    if (ep.z) r = fma(ep.beta, static_cast<double>(static_cast<const V*>(ep.z)[i]), r);
    y[i] = static_cast<V>(r);
  }
}

template <typename V>
bool launch_dense(const SlicedMatrix& m, const void* x, void* y, cudaStream_t s) {
  const long long grid = (m.num_tasks + kWarpsPerBlock - 1) / kWarpsPerBlock;
  if (grid > 0x7fffffffLL) {
    set_error("dense blocks: too many tasks for one launch");
    return false;
  }
  dense_block_kernel<V><<<(unsigned)grid, kWarpsPerBlock * 32, 0, s>>>(
      m.tasks, m.num_tasks, static_cast<const V*>(m.val), m.col, m.rowid, static_cast<const V*>(x), (int)m.n_cols,
      static_cast<V*>(y), static_cast<V*>(m.chunk_sum));
  return VNEC_CUDA(cudaGetLastError());
}

template <typename V>
__global__ void gather_hot(const V* __restrict__ x, const int32_t* __restrict__ hot_cols, int n, V* __restrict__ xh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) xh[i] = __ldg(x + __ldg(hot_cols + i));
}

template <typename V, int U, int H, bool HOT, bool EPI = false>
bool launch_main(const SlicedMatrix& m, const void* x, void* y, cudaStream_t s,
                 const SlicedEpilogue& ep = SlicedEpilogue()) {
  auto kern = sliced_kernel<V, U, H, HOT, EPI>;
  // No shared memory: give the whole unified L1/shared array to L1.
  static std::atomic<unsigned long long> configured{0};  // per instantiation, per device
  if (!once_per_device(configured, [&] {
        return VNEC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 0));
      }))
    return false;
  const long long grid = (m.num_tasks + kWarpsPerBlock - 1) / kWarpsPerBlock;
  if (grid > 0x7fffffffLL) {
    set_error("sliced: too many tasks for one launch");
    return false;
  }
  if (HOT && !m.hot_ready) {
    gather_hot<V><<<(unsigned)((m.hot + 255) / 256), 256, 0, s>>>(static_cast<const V*>(x), m.hot_cols, m.hot,
                                                                  static_cast<V*>(m.xhot));
    if (!VNEC_CUDA(cudaGetLastError())) return false;
  }
  kern<<<(unsigned)grid, kWarpsPerBlock * 32, 0, s>>>(m.tasks, m.num_tasks, static_cast<const V*>(m.val), m.col,
                                                      m.rowid, static_cast<const V*>(x), static_cast<V*>(y),
                                                      static_cast<V*>(m.chunk_sum),
                                                      static_cast<const V*>(m.xhot), (int)m.n_cols, ep, m.col16,
                                                      m.first, m.pf);
  return VNEC_CUDA(cudaGetLastError());
}

template <typename V, int U, bool HOT>
bool launch_hints(const SlicedMatrix& m, const void* x, void* y, cudaStream_t s) {
  switch (m.cache_hints) {
    case 1: return launch_main<V, U, 1, HOT>(m, x, y, s);
    case 2: return launch_main<V, U, 2, HOT>(m, x, y, s);
    case 3: return launch_main<V, U, 3, HOT>(m, x, y, s);
    default: return launch_main<V, U, 0, HOT>(m, x, y, s);
  }
}

template <typename V, bool HOT>
bool launch_unroll(const SlicedMatrix& m, const void* x, void* y, cudaStream_t s) {
  switch (m.unroll) {
    case 4: return launch_hints<V, 4, HOT>(m, x, y, s);
    case 12: return launch_hints<V, 12, HOT>(m, x, y, s);
    case 16: return launch_hints<V, 16, HOT>(m, x, y, s);
    default: return launch_hints<V, 8, HOT>(m, x, y, s);
  }
}

template <typename V, bool HOT>
bool launch_fused(const SlicedMatrix& m, const void* x, void* y, cudaStream_t s, const SlicedEpilogue& ep) {
  switch (m.unroll) {
    case 4: return launch_main<V, 4, 0, HOT, true>(m, x, y, s, ep);
    case 8: return launch_main<V, 8, 0, HOT, true>(m, x, y, s, ep);
    case 16: return launch_main<V, 16, 0, HOT, true>(m, x, y, s, ep);
    default: return launch_main<V, 12, 0, HOT, true>(m, x, y, s, ep);
  }
}

template <typename V>
bool launch_variant(const SlicedMatrix& m, const void* x, void* y, cudaStream_t s) {
  return m.hot > 0 ? launch_unroll<V, true>(m, x, y, s) : launch_unroll<V, false>(m, x, y, s);
}

template <typename V>
bool launch(const SlicedMatrix& m, const void* x, void* y, cudaStream_t s, cudaEvent_t* ev,
            const SlicedEpilogue* epi) {
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[0], s))) return false;
  // The fused epilogue runs at the plan's unroll with default cache hints;
  // dense-block plans apply it as a separate pass.
  const bool fused = epi && m.vpe == 1;
  if (m.num_tasks > 0) {
    bool ok;
    if (m.vpe == 4)
      ok = launch_dense<V>(m, x, y, s);
    else if (fused)
      ok = m.hot > 0 ? launch_fused<V, true>(m, x, y, s, *epi) : launch_fused<V, false>(m, x, y, s, *epi);
    else
      ok = launch_variant<V>(m, x, y, s);
    if (!ok) return false;
  }
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[1], s))) return false;
  if (m.num_long > 0) {
    const int b = 128;
    const FixupGrid g = fixup_grid(m, b);
    if (fused)
      sliced_long_fixup<V, true><<<g.total, b, 0, s>>>(m.long_row, m.long_first, m.long_heavy, m.num_long,
                                                       m.num_heavy, m.heavy_sub, g.light,
                                                       static_cast<const V*>(m.chunk_sum), static_cast<V*>(y), *epi);
    else
      sliced_long_fixup<V><<<g.total, b, 0, s>>>(m.long_row, m.long_first, m.long_heavy, m.num_long, m.num_heavy,
                                                 m.heavy_sub, g.light, static_cast<const V*>(m.chunk_sum),
                                                 static_cast<V*>(y));
    if (!VNEC_CUDA(cudaGetLastError())) return false;
  }
  if (epi && !fused && !apply_epilogue(y, m.n_rows, sizeof(V) == 8, *epi, s)) return false;
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[2], s))) return false;
  return true;
}

}  // namespace

bool sliced_guard_f64(const SlicedMatrix& m, const double* x, double* y, const int* flag, cudaStream_t s) {
  // The guard only runs for DF32 plans, whose FP64 values sit in m.val and
  // whose hot columns (if any) are served from x directly through hot_cols.
  int dev = 0, sms = 0;
  if (!VNEC_CUDA(cudaGetDevice(&dev)) || !VNEC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)))
    return false;
  const long long need = (m.num_tasks + kWarpsPerBlock - 1) / kWarpsPerBlock;
  const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>(need, 8LL * sms));
  if (m.hot > 0) {
    gather_hot<double><<<(unsigned)((m.hot + 255) / 256), 256, 0, s>>>(x, m.hot_cols, m.hot,
                                                                       static_cast<double*>(m.xhot));
    if (!VNEC_CUDA(cudaGetLastError())) return false;
    sliced_guard_kernel<true><<<grid, kWarpsPerBlock * 32, 0, s>>>(
        flag, m.tasks, m.num_tasks, static_cast<const double*>(m.val), m.col, m.rowid, x, y,
        static_cast<double*>(m.chunk_sum), static_cast<const double*>(m.xhot), (int)m.n_cols, m.col16, m.first);
  } else {
    sliced_guard_kernel<false><<<grid, kWarpsPerBlock * 32, 0, s>>>(
        flag, m.tasks, m.num_tasks, static_cast<const double*>(m.val), m.col, m.rowid, x, y,
        static_cast<double*>(m.chunk_sum), nullptr, 0, m.col16, m.first);
  }
  return VNEC_CUDA(cudaGetLastError());
}

bool sliced_spmv(const SlicedMatrix& m, bool fp64, const void* x, void* y, cudaStream_t s, cudaEvent_t* ev,
                 const SlicedEpilogue* epi) {
  return fp64 ? launch<double>(m, x, y, s, ev, epi) : launch<float>(m, x, y, s, ev, epi);
}

bool sliced_gather_hot(const SlicedMatrix& m, bool fp64, const void* x, cudaStream_t s) {
  if (m.hot <= 0) return true;
  const unsigned g = (unsigned)((m.hot + 255) / 256);
  if (fp64)
    gather_hot<double><<<g, 256, 0, s>>>(static_cast<const double*>(x), m.hot_cols, m.hot, static_cast<double*>(m.xhot));
  else
    gather_hot<float><<<g, 256, 0, s>>>(static_cast<const float*>(x), m.hot_cols, m.hot, static_cast<float*>(m.xhot));
  return VNEC_CUDA(cudaGetLastError());
}

bool apply_epilogue(void* y, long long n, bool fp64, const SlicedEpilogue& e, cudaStream_t s) {
  if (n <= 0) return true;
  const int tb = 256;
  const unsigned grid = (unsigned)std::min<long long>((n + tb - 1) / tb, 152LL * 16);
  if (fp64)
    epilogue_kernel<double><<<grid, tb, 0, s>>>(static_cast<double*>(y), n, e);
  else
    epilogue_kernel<float><<<grid, tb, 0, s>>>(static_cast<float*>(y), n, e);
  return VNEC_CUDA(cudaGetLastError());
}

}  // namespace vnec
