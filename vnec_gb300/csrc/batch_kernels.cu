// Batched multi-right-hand-side SpMV kernel (batch.h): one persistent launch
// over the task list of the block-diagonal concatenation of the batch.
//
// Lane l of a warp serves right-hand sides [sub * R, sub * R + R) with
// sub = l % L, R = k / L, and slot l / L of the S = 32 / L (value, column)
// slots the warp reads at every step (lanes of a slot read the same pair, a
// broadcast).  A ROWS task holds G = S / V rows, V = 2^vwl slots per row:
// entry j of row g sits at base + (j / V) * S + g * V + j % V, each lane
// gathers R consecutive values of row `column` of X with 16-byte vector loads
// (so the L lanes of a slot read the whole k-wide X row), and the V slots of a
// row are summed with xor-shuffles.  CHUNK tasks (pieces of rows longer than
// the grouping limit) use all S slots for one row; their sums go to chunk_sum
// and the last chunk of a row to arrive (an arrival counter per long row,
// reset by that chunk) adds the row's chunk sums in chunk order, so no second
// kernel is needed.
//
// Arithmetic forms (codecs):
//   FP64 — FP64 values, X and FMA;
//   FP32 — FP32 values, X rounded to FP32 once per call by a preceding kernel,
//          FP32 products and per-lane accumulation; slot, chunk and long-row
//          sums in FP64;
//   DF32 — values stored as FP32 (hi, lo) truncation-split pairs, X split once
//          per call; Dekker products and TwoSum accumulation on the FP32 pipe
//          (FP64-level accuracy), FP64 slot/chunk sums.  When the split kernel
//          flags an X value outside the split range, the same launch computes
//          in FP64 (value = hi + lo, FP64 X).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "batch.h"
#include "common.h"
#include "df32.cuh"

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
  const void* x;       // X in the codec's element type
  const double* x64;   // DF32: the FP64 X (guard path)
  const int* flag;     // DF32: X outside the split range this call
  double* y;
  int klog2;  // k = 1 << klog2
  int llog2;  // lanes per slot L = 1 << llog2
};

// R consecutive elements of type T at p (16-, 8- or 4-byte vector loads).
template <typename T, int R> __device__ __forceinline__ void load_vec(const T* p, T (&v)[R]) {
  constexpr int bytes = R * (int)sizeof(T);
  if constexpr (bytes >= 16) {
#pragma unroll
    for (int i = 0; i < bytes / 16; ++i) {
      const int4 q = __ldg(reinterpret_cast<const int4*>(p) + i);
      memcpy(reinterpret_cast<char*>(v) + 16 * i, &q, 16);
    }
  } else if constexpr (bytes == 8) {
    const int2 q = __ldg(reinterpret_cast<const int2*>(p));
    memcpy(v, &q, 8);
  } else {
    const int q = __ldg(reinterpret_cast<const int*>(p));
    memcpy(v, &q, 4);
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

struct CodecF64 {
  static constexpr bool kPairReduce = false;
  using V = double;
  using X = double;
  struct A {
    double s;
  };
  __device__ static A zero() { return A{0.0}; }
  __device__ static void mac(A& a, V v, X x) { a.s = fma(v, x, a.s); }
  __device__ static double out(const A& a) { return a.s; }
};

struct CodecF32 {
  static constexpr bool kPairReduce = false;
  using V = float;
  using X = float;
  struct A {
    float s;
  };
  __device__ static A zero() { return A{0.f}; }
  __device__ static void mac(A& a, V v, X x) { a.s = fmaf(v, x, a.s); }
  __device__ static double out(const A& a) { return static_cast<double>(a.s); }
};

// Double-float: value (hi, lo) times x (hi, lo), Dekker product with FMA,
// TwoSum into (s, c).
struct CodecDF32 {
  static constexpr bool kPairReduce = true;
  using V = float2;
  using X = float2;
  struct A {
    float s, c;
  };
  // a += the (s, c) pair of the lane `off` away (TwoSum of the high parts).
  __device__ static void add_shfl(A& a, int off) {
    const float s2 = __shfl_xor_sync(0xffffffffu, a.s, off), c2 = __shfl_xor_sync(0xffffffffu, a.c, off);
    const float t = __fadd_rn(a.s, s2);
    const float bb = __fsub_rn(t, a.s);
    const float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bb)), __fsub_rn(s2, bb));
    a.s = t;
    a.c = __fadd_rn(a.c, __fadd_rn(c2, e));
  }
  __device__ static A zero() { return A{0.f, 0.f}; }
  __device__ static void mac(A& a, V v, X x) {
    const DF r = df_mac(DF{a.s, a.c}, v.x, v.y, x.x, x.y);
    a.s = r.s;
    a.c = r.c;
  }
  __device__ static double out(const A& a) { return df_to_f64(DF{a.s, a.c}); }
};

// FP64 from split values and FP64 X: the guard path of DF32 plans.
struct CodecDF32Guard {
  static constexpr bool kPairReduce = false;
  using V = float2;
  using X = double;
  struct A {
    double s;
  };
  __device__ static A zero() { return A{0.0}; }
  __device__ static void mac(A& a, V v, X x) {
    a.s = fma(static_cast<double>(v.x) + static_cast<double>(v.y), x, a.s);
  }
  __device__ static double out(const A& a) { return a.s; }
};

__device__ __forceinline__ double shfl_val(double v, int src) { return __shfl_sync(kFull, v, src); }
__device__ __forceinline__ float shfl_val(float v, int src) { return __shfl_sync(kFull, v, src); }
__device__ __forceinline__ float2 shfl_val(float2 v, int src) {
  return make_float2(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src));
}

// STAGED: each task's (column, value) entries are read 32 * kStageRounds at a
// time with one coalesced load per lane per 32 entries, and every step's pair
// reaches its slot's lanes by shuffles, so inside the step loop only the X
// gathers wait on memory.  Otherwise every step's pair is loaded by the slot's
// lanes (broadcast), U steps in flight.
constexpr int kStageRounds = 4;

template <class Cd, int R, int U, bool STAGED = false>
__device__ __forceinline__ void run_tasks(const BatchArgs& a, const typename Cd::X* __restrict__ x) {
  using V = typename Cd::V;
  using X = typename Cd::X;
  const int lane = threadIdx.x & 31;
  const int k = 1 << a.klog2;
  const int S = 32 >> a.llog2;  // slots per step
  const int slot = lane >> a.llog2, sub = lane & ((1 << a.llog2) - 1);
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  const V* __restrict__ val = static_cast<const V*>(a.val);
  const X* __restrict__ xs = x + sub * R;
  for (long long t = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < a.num_tasks; t += nw) {
    const int4 raw = __ldg(a.tasks + t);
    const int base = raw.x, row_base = raw.y, steps = raw.z, kind = raw.w & 15, vwl = (raw.w >> 4) & 15,
              nrows = raw.w >> 8;
    if (kind == kSlicedZero) {
      for (int i = lane; i < (nrows << a.klog2); i += 32)
        a.y[((size_t)__ldg(a.rowid + row_base + (i >> a.klog2)) << a.klog2) + (i & (k - 1))] = 0.0;
      continue;
    }
    const V* vp = val + base + slot;
    const int32_t* cp = a.col + base + slot;
    typename Cd::A acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = Cd::zero();
    int s = 0;
    if constexpr (STAGED) {
      const int E = steps * S;  // entries of the task
      const int spr = 32 / S;   // steps per 32 entries (= L)
      const int32_t* cb = a.col + base;
      const V* vb = val + base;
      for (int e0 = 0; e0 < E; e0 += 32 * kStageRounds) {
        int creg[kStageRounds];
        V vreg[kStageRounds];
#pragma unroll
        for (int b = 0; b < kStageRounds; ++b) {
          const int e = e0 + b * 32 + lane;
          creg[b] = e < E ? __ldcs(cb + e) : 0;
          vreg[b] = e < E ? __ldcs(vb + e) : V{};
        }
#pragma unroll
        for (int b = 0; b < kStageRounds; ++b) {
          const int sb = (e0 + b * 32) / S;  // first step held by register round b
          if (sb >= steps) break;
          for (int j = 0; j < spr; j += U) {
            int c[U];
            V v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const int src = (((j + u) * S) & 31) + slot;
              c[u] = __shfl_sync(kFull, creg[b], src);
              v[u] = shfl_val(vreg[b], src);
            }
            X xv[U][R];
#pragma unroll
            for (int u = 0; u < U; ++u)
              if (j + u < spr && sb + j + u < steps) load_vec<X, R>(xs + ((size_t)c[u] << a.klog2), xv[u]);
#pragma unroll
            for (int u = 0; u < U; ++u)
              if (j + u < spr && sb + j + u < steps)
#pragma unroll
                for (int r = 0; r < R; ++r) Cd::mac(acc[r], v[u], xv[u][r]);
          }
        }
      }
      s = steps;
    }
    for (; s + U <= steps; s += U) {
      int c[U];
      V v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        c[u] = __ldcs(cp + (s + u) * S);
        v[u] = __ldcs(vp + (s + u) * S);
      }
      X xv[U][R];
#pragma unroll
      for (int u = 0; u < U; ++u) load_vec<X, R>(xs + ((size_t)c[u] << a.klog2), xv[u]);
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int r = 0; r < R; ++r) Cd::mac(acc[r], v[u], xv[u][r]);
    }
    for (; s < steps; ++s) {
      const int c = __ldcs(cp + s * S);
      const V v = __ldcs(vp + s * S);
      X xv[R];
      load_vec<X, R>(xs + ((size_t)c << a.klog2), xv);
#pragma unroll
      for (int r = 0; r < R; ++r) Cd::mac(acc[r], v, xv[r]);
    }
    // Slots to sum: the whole warp for a chunk, the V slots of a row otherwise.
    const int span = kind == kSlicedChunk ? 32 : 1 << (a.llog2 + vwl);
    double d[R];
    if constexpr (Cd::kPairReduce) {
      // Double-float: sum the slots as (hi, lo) pairs on the FP32 pipe and
      // convert once (each FP64 operation costs 64 FP32 issue slots here).
      for (int off = 1 << a.llog2; off < span; off <<= 1)
#pragma unroll
        for (int r = 0; r < R; ++r) Cd::add_shfl(acc[r], off);
#pragma unroll
      for (int r = 0; r < R; ++r) d[r] = Cd::out(acc[r]);
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) d[r] = Cd::out(acc[r]);
      for (int off = 1 << a.llog2; off < span; off <<= 1)
#pragma unroll
        for (int r = 0; r < R; ++r) d[r] += __shfl_xor_sync(kFull, d[r], off);
    }
    if (kind == kSlicedChunk) {
      if (slot == 0) store_y<R>(a.chunk_sum + ((size_t)row_base << a.klog2) + sub * R, d);
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
    } else {
      const int g = slot >> vwl;
      if ((slot & ((1 << vwl) - 1)) == 0 && g < nrows)
        store_y<R>(a.y + ((size_t)__ldg(a.rowid + row_base + g) << a.klog2) + sub * R, d);
    }
  }
}

template <class Cd, int R, int U, bool STAGED>
__global__ void __launch_bounds__(256) batch_kernel(const BatchArgs a) {
  run_tasks<Cd, R, U, STAGED>(a, static_cast<const typename Cd::X*>(a.x));
}

template <int R, int U, bool STAGED>
__global__ void __launch_bounds__(256) batch_df32_kernel(const BatchArgs a) {
  if (*reinterpret_cast<const volatile int*>(a.flag))
    run_tasks<CodecDF32Guard, R, U, STAGED>(a, a.x64);
  else
    run_tasks<CodecDF32, R, U, STAGED>(a, static_cast<const float2*>(a.x));
}

// Steps in flight per lane: 8 / R (at least 2), doubled in mode 1; mode 2
// stages the entries in registers (STAGED) with the mode-0 step count.
template <int R, int MODE> constexpr int unroll_for() { return (R >= 4 ? 2 : 8 / R) * (MODE == 1 ? 2 : 1); }

template <int R, int MODE> void* kernel_for(int precision) {
  constexpr int U = unroll_for<R, MODE>();
  constexpr bool ST = MODE == 2;
  switch (precision) {
    case kPrecFP32: return reinterpret_cast<void*>(&batch_kernel<CodecF32, R, U, ST>);
    case kPrecDF32: return reinterpret_cast<void*>(&batch_df32_kernel<R, U, ST>);
    default: return reinterpret_cast<void*>(&batch_kernel<CodecF64, R, U, ST>);
  }
}

template <int R> void* kernel_for_mode(int precision, int mode) {
  return mode == 2 ? kernel_for<R, 2>(precision) : mode == 1 ? kernel_for<R, 1>(precision) : kernel_for<R, 0>(precision);
}

void* pick_kernel(int precision, int r, int mode) {
  switch (r) {
    case 1: return kernel_for_mode<1>(precision, mode);
    case 2: return kernel_for_mode<2>(precision, mode);
    case 4: return kernel_for_mode<4>(precision, mode);
    case 8: return kernel_for_mode<8>(precision, mode);
    default: return nullptr;
  }
}

int log2i(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

}  // namespace

int batch_grid(int precision, int rhs_per_lane, int warps_per_block, int mode) {
  void* fn = pick_kernel(precision, rhs_per_lane, mode);
  if (!fn || (warps_per_block != 4 && warps_per_block != 8)) return 0;
  int dev = 0, sms = 0, per_sm = 0;
  if (!VNEC_CUDA(cudaGetDevice(&dev)) ||
      !VNEC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) ||
      !VNEC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, warps_per_block * 32, 0)))
    return 0;
  return sms * std::max(per_sm, 1);
}

bool batch_spmm(const BatchMatrix& m, const double* X, double* Y, cudaStream_t s) {
  return batch_spmm_range(m, X, Y, s, 0, m.num_tasks, 0, m.n_cols, true);
}

bool batch_spmm_range(const BatchMatrix& m, const double* X, double* Y, cudaStream_t s, int64_t t0, int64_t t1,
                      int64_t c0, int64_t c1, bool first) {
  if (!batch_supported(m.k, m.lanes)) {
    set_error("batch: unsupported k / lanes");
    return false;
  }
  const int R = m.k / m.lanes;
  const void* xin = X;
  const long long off = (long long)c0 * m.k, nx = (long long)(c1 - c0) * m.k;
  if (m.precision == kPrecFP32) {
    if (nx > 0 && !round_to_f32(X + off, static_cast<float*>(m.xbuf) + off, nx, s)) return false;
    xin = m.xbuf;
  } else if (m.precision == kPrecDF32) {
    if (first && !VNEC_CUDA(cudaMemsetAsync(m.flag, 0, sizeof(int), s))) return false;
    if (nx > 0 && !split_to_df32(X + off, static_cast<float2*>(m.xbuf) + off, nx, m.flag, s)) return false;
    xin = m.xbuf;
  }
  if (t1 <= t0) return true;
  BatchArgs a;
  a.tasks = reinterpret_cast<const int4*>(m.tasks) + t0;
  a.num_tasks = t1 - t0;
  a.val = m.val;
  a.col = m.col;
  a.rowid = m.rowid;
  a.long_row = m.long_row;
  a.long_first = m.long_first;
  a.chunk_long = m.chunk_long;
  a.chunk_sum = m.chunk_sum;
  a.chunk_count = m.chunk_count;
  a.x = xin;
  a.x64 = X;
  a.flag = m.flag;
  a.y = Y;
  a.klog2 = log2i(m.k);
  a.llog2 = log2i(m.lanes);
  void* fn = pick_kernel(m.precision, R, m.mode);
  // Persistent warps stride the task list; with per_task every warp takes one
  // task and the hardware dispatches the blocks in task order, so the tasks in
  // flight stay a compact window of the list (and of X's rows).
  const long long per_task_grid = (a.num_tasks + m.warps_per_block - 1) / m.warps_per_block;
  if (m.per_task && per_task_grid > 0x7fffffffLL) {
    set_error("batch: too many tasks for one launch with one warp per task");
    return false;
  }
  const int grid = m.per_task ? (int)per_task_grid
                              : (int)std::min<long long>(m.grid, std::max<long long>(1, (a.num_tasks + 7) / 8));
  void* args[] = {&a};
  return VNEC_CUDA(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3((unsigned)(m.warps_per_block * 32)), args, 0, s));
}

}  // namespace vnec
