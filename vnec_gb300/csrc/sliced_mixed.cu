// Precision forms of the sliced row-group SpMV (same warp-task layout as
// sliced_kernels.cu), all producing FP64 y from FP64 x:
//
//   FP32 : values stored as FP32 (4 B), x rounded to FP32 once per call,
//          FP32 products and per-lane FP32 accumulation; the lane partials
//          are converted to FP64 and the VW-lane reduction and the long-row
//          chunk fix-up run in FP64.
//   BF16 : values stored as BF16 (2 B) after scaling each row by a power of
//          two (row exponent stored as int8), FP32 products/accumulation, the
//          scale is applied exactly in FP64 after the FP64 lane reduction.
//   DF32 : values stored as FP64 (8 B), split in-kernel into FP32 (hi, lo)
//          pairs, x split once per call; Dekker products and TwoSum
//          accumulation in FP32 (double-float), FP64 reductions — FP64-level
//          accuracy on the FP32 pipe.  An x outside the split range raises a
//          flag: the DF32 launch then returns at once and a guard launch of
//          the FP64 sliced kernel computes the call.
//
// x conversion kernels: f64 -> f32 with round-to-nearest-even written from
// the IEEE-754 definition in integer arithmetic (no FP64 instructions: the
// FP64 pipe of GB300 converts at about 0.28 G/s per SM group), and the
// truncation split f64 -> (hi, lo) used by DF32.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "common.h"
#include "df32.cuh"
#include "long_rows.cuh"
#include "prefetch.cuh"
#include "sliced.h"
#include "vnec_gb300.h"

namespace vnec {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarps = 8;

// Round-to-nearest-even FP64 -> FP32 from the bit patterns (IEEE 754:
// overflow to infinity, gradual underflow to subnormals, NaN stays NaN):
// every case, in 64-bit integer arithmetic.
__device__ __noinline__ float f64_to_f32_rne_general(double v) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
  const unsigned sign = static_cast<unsigned>(b >> 63) << 31;
  const int e = static_cast<int>((b >> 52) & 0x7ff);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x00400000u : 0u));
  const int E = e - 1023;
  if (E > 127) return __uint_as_float(sign | 0x7f800000u);
  if (e == 0) return __uint_as_float(sign);  // FP64 subnormals are far below FP32's range
  unsigned long long M = m | (1ull << 52);   // 53-bit significand
  int shift;                                 // bits of M dropped
  unsigned expo;
  if (E >= -126) {
    shift = 29;
    expo = static_cast<unsigned>(E + 127);
  } else {
    shift = 29 + (-126 - E);
    expo = 0;
    if (shift > 54) return __uint_as_float(sign);  // below half of the smallest subnormal
  }
  unsigned long long q = M >> shift;
  const unsigned long long rem = M & ((1ull << shift) - 1);
  const unsigned long long half = 1ull << (shift - 1);
  if (rem > half || (rem == half && (q & 1))) ++q;
  unsigned bits;
  if (expo == 0) {
    bits = static_cast<unsigned>(q);  // subnormal; a carry into bit 23 yields the smallest normal
  } else {
    if (q == (1ull << 24)) {  // rounding carried into a new binade
      q >>= 1;
      ++expo;
      if (expo >= 255) return __uint_as_float(sign | 0x7f800000u);
    }
    bits = (expo << 23) | (static_cast<unsigned>(q) & 0x7FFFFFu);
  }
  return __uint_as_float(sign | bits);
}

// The same rounding with a 32-bit fast path for the usual case, an FP64
// exponent inside FP32's normal range (2^-126 <= |v| < 2^128): the high word
// rebiased and shifted gives the sign, exponent and top 20 fraction bits,
// the low word's top 3 bits complete the 23, and adding the round bit (bit
// 28 of the low word) when the bits below it are not all zero or the kept
// lsb is odd rounds to nearest even; a carry out of the fraction moves to
// the next binade, and out of exponent 254 to infinity, as IEEE 754 wants.
__device__ __forceinline__ float f64_to_f32_rne(double v) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
  const unsigned hi = static_cast<unsigned>(b >> 32), lo = static_cast<unsigned>(b);
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e - 897u < 254u) {
    const unsigned bits = (hi & 0x80000000u) | (((hi & 0x7fffffffu) - (896u << 20)) << 3) | (lo >> 29);
    const unsigned up = (lo >> 28) & (((lo & 0x0fffffffu) != 0u) | (lo >> 29)) & 1u;
    return __uint_as_float(bits + up);
  }
  return f64_to_f32_rne_general(v);
}

}  // namespace

namespace {

// x (n values) followed by the values of the `nh` hot columns (a plan with a
// hot-column window reads slot s as column n + s).
__device__ __forceinline__ double x_ext(const double* __restrict__ x, long long n, const int32_t* __restrict__ hot,
                                        long long i) {
  return x[i < n ? i : __ldg(hot + (i - n))];
}

__device__ __forceinline__ bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// x rounded to FP32, then the hot columns' values.  Each thread rounds four
// consecutive values per step (two 16-byte loads, one 16-byte store) when x is
// 16-byte aligned, so enough bytes are in flight to run at HBM rate; the
// remainder and the hot tail take one value per step.
__device__ __forceinline__ void round_x(const double* __restrict__ x, float* __restrict__ x32, long long n,
                                        const int32_t* __restrict__ hot, int nh) {
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x, nt = (long long)gridDim.x * blockDim.x;
  const long long n4 = aligned16(x) && aligned16(x32) ? n / 4 : 0;
  for (long long q = t0; q < n4; q += nt) {
    const double2 a = __ldcs(reinterpret_cast<const double2*>(x) + 2 * q);
    const double2 b = __ldcs(reinterpret_cast<const double2*>(x) + 2 * q + 1);
    reinterpret_cast<float4*>(x32)[q] =
        make_float4(f64_to_f32_rne(a.x), f64_to_f32_rne(a.y), f64_to_f32_rne(b.x), f64_to_f32_rne(b.y));
  }
  for (long long i = 4 * n4 + t0; i < n + nh; i += nt) x32[i] = f64_to_f32_rne(x_ext(x, n, hot, i));
}

}  // namespace

// Outside the anonymous namespace: also launched by SpB_VNEC_f64_to_f32_ext.
__global__ void x_to_f32_kernel(const double* __restrict__ x, float* __restrict__ x32, long long n) {
  round_x(x, x32, n, nullptr, 0);
}
namespace {

__global__ void x_to_f32_ext_kernel(const double* __restrict__ x, float* __restrict__ x32, long long n,
                                    const int32_t* __restrict__ hot, int nh) {
  round_x(x, x32, n, hot, nh);
}

// x split into (hi, lo) pairs, then the hot columns' pairs: two values per
// step (one 16-byte load, one 16-byte store) when x is 16-byte aligned.
__global__ void x_split_kernel(const double* __restrict__ x, float2* __restrict__ xs, long long n, int* flag,
                               const int32_t* __restrict__ hot, int nh) {
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x, nt = (long long)gridDim.x * blockDim.x;
  const long long n2 = aligned16(x) && aligned16(xs) ? n / 2 : 0;
  bool bad = false;
  for (long long q = t0; q < n2; q += nt) {
    const double2 a = __ldcs(reinterpret_cast<const double2*>(x) + q);
    float h0, l0, h1, l1;
    bad |= !df_split(a.x, h0, l0);
    bad |= !df_split(a.y, h1, l1);
    reinterpret_cast<float4*>(xs)[q] = make_float4(h0, l0, h1, l1);
  }
  for (long long i = 2 * n2 + t0; i < n + nh; i += nt) {
    float h, l;
    bad |= !df_split(x_ext(x, n, hot, i), h, l);
    xs[i] = make_float2(h, l);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

struct CodecF32 {
  using Val = float;
  using Acc = float;
  __device__ static Acc zero() { return 0.0f; }
  __device__ static Acc mac(Acc a, Val v, const void* xs, int c) {
    return fmaf(v, __ldg(static_cast<const float*>(xs) + c), a);
  }
  __device__ static double to_f64(Acc a) { return static_cast<double>(a); }
};

struct CodecBF16 {
  using Val = unsigned short;
  using Acc = float;
  __device__ static Acc zero() { return 0.0f; }
  __device__ static Acc mac(Acc a, Val v, const void* xs, int c) {
    return fmaf(__uint_as_float(static_cast<unsigned>(v) << 16), __ldg(static_cast<const float*>(xs) + c), a);
  }
  __device__ static double to_f64(Acc a) { return static_cast<double>(a); }
};

struct CodecDF32 {
  using Val = float2;  // (hi, lo) split at plan build (the range was checked there)
  using Acc = DF;
  __device__ static Acc zero() { return DF{0.0f, 0.0f}; }
  __device__ static Acc mac(Acc acc, Val v, const void* xs, int c) {
    const float2 x = __ldg(static_cast<const float2*>(xs) + c);
    return df_mac(acc, v.x, v.y, x.x, x.y);
  }
  __device__ static double to_f64(Acc a) { return df_to_f64(a); }
};

template <typename T> __device__ __forceinline__ T ld_stream(const T* p) { return __ldcs(p); }
template <> __device__ __forceinline__ unsigned short ld_stream<unsigned short>(const unsigned short* p) {
  return __ldcs(p);
}

// One lane run (SlicedMatrix::lane_run): N consecutive 32-bit words read as
// streaming 8- or 16-byte vectors.
template <int N>
__device__ __forceinline__ void ld_words(const void* p, uint32_t (&w)[N]) {
  static_assert(N == 2 || N % 4 == 0, "runs are 8 bytes or whole 16-byte vectors");
  if constexpr (N == 2) {
    const uint2 r = __ldcs(static_cast<const uint2*>(p));
    w[0] = r.x;
    w[1] = r.y;
  } else {
#pragma unroll
    for (int i = 0; i < N / 4; ++i) {
      const uint4 r = __ldcs(static_cast<const uint4*>(p) + i);
      w[4 * i] = r.x;
      w[4 * i + 1] = r.y;
      w[4 * i + 2] = r.z;
      w[4 * i + 3] = r.w;
    }
  }
}
// Element t of a run of 4-byte (float, int32) or 2-byte (BF16, delta) items.
template <typename T, int N>
__device__ __forceinline__ T run_at(const uint32_t (&w)[N], int t) {
  if constexpr (sizeof(T) == 4) {
    T v;
    memcpy(&v, &w[t], 4);
    return v;
  } else {
    static_assert(sizeof(T) == 2, "2- or 4-byte items");
    return static_cast<T>((w[t >> 1] >> (16 * (t & 1))) & 0xffffu);
  }
}

__device__ __forceinline__ double pow2(int e) {
  return __longlong_as_double(static_cast<long long>(e + 1023) << 52);
}

// P > 0: the arrays hold lane runs of P steps (SlicedMatrix::lane_run);
// 2U / P runs are in flight per lane.  The per-lane sums take the same steps
// in the same order as the stride-32 layout (P = 0), so both give the same y.
// SH: the plan has shared-pattern tasks (kSlicedShared); plans without them
// run the SH = false build, whose registers the shared path does not raise.
template <class C, int U, int P, bool SH>
__global__ void __launch_bounds__(kWarps * 32)
sliced_mixed_kernel(const SlicedTask* __restrict__ tasks, long long num_tasks, const typename C::Val* __restrict__ val,
                    const int32_t* __restrict__ col, const int32_t* __restrict__ rowid, const void* __restrict__ xs,
                    double* __restrict__ y, double* __restrict__ chunk_sum, const signed char* __restrict__ row_scale,
                    const signed char* __restrict__ chunk_scale, const int* __restrict__ flag,
                    const uint16_t* __restrict__ col16, const int32_t* __restrict__ first,
                    const uint16_t* __restrict__ pat16, SlicedPrefetch pf) {
  if (flag && *reinterpret_cast<const volatile int*>(flag)) return;  // DF32: x out of range, guard launch computes
  const long long w = ((long long)blockIdx.x * kWarps) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= num_tasks) return;
  const int4 raw = __ldg(reinterpret_cast<const int4*>(tasks) + w);
  const int base = raw.x, row_base = raw.y, steps = raw.z, meta = raw.w;
  const int kind = meta & 15, vwl = (meta >> 4) & 15, nrows = (meta >> 8) & 0xff;
  // The values (and per-lane column deltas) `pf` entries past this task's,
  // into L2 (prefetch.cuh).
  if (pf.entries > 0) {
    prefetch_l2_task_meta(pf, w, base, row_base, kind != kSlicedChunk, tasks, first, rowid, pat16, lane);
    const long long e0 = base + pf.entries, len = 32LL * steps;
    if (kind != kSlicedZero && e0 + len <= pf.n_entries) {
      prefetch_l2_range(val + e0, len, lane);
      if ((meta & kSlicedDelta) && !(SH && (meta & kSlicedShared))) prefetch_l2_range(col16 + e0, len, lane);
    }
  }
  if (kind == kSlicedZero) {
    if (lane < nrows) y[rowid[row_base + lane]] = 0.0;
    return;
  }
  using Val = typename C::Val;
  // Lane runs: rounds of 2U steps (2U / P runs) per lane, the ragged tail
  // loaded with the first round and summed last.
  constexpr int UB = P > 0 ? 2 * U / P : 1;                  // runs per round
  constexpr int VW = P > 0 ? P * (int)sizeof(Val) / 4 : 1;  // words per value run
  constexpr int TL = P > 1 ? P - 1 : 1;                      // stride-32 steps after the runs
  // BF16 runs (8 steps) instead take U / 4 runs at a time, then single runs,
  // and sum the ragged tail in a final loop: fewer registers, more warps.
  constexpr bool kSerialTail = sizeof(Val) == 2;
  constexpr int UBS = U / 4 > 0 ? U / 4 : 1;
  if (SH && (meta & kSlicedShared)) {
    // Every row of the task has `steps` entries with the same column gaps:
    // lane k loads gap k of the shared pattern, a warp prefix sum turns the
    // gaps into offsets from the first column, and step k's column is the
    // row's first column plus offset k (a shuffle; no load on the x path).
    int off = lane < steps ? __ldg(pat16 + (base >> 5) + lane) : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, off, o);
      if (lane >= o) off += t;
    }
    const int c0 = lane < nrows ? __ldg(first + row_base + lane) : 0;
    typename C::Acc acc = C::zero();
    const Val* vp = val + base + lane;
    if constexpr (P > 0 && kSerialTail) {
      // BF16 runs: UBS runs at a time, then single runs, then the tail one
      // step at a time (fewer registers than a preloaded 7-step tail).
      const int nb = steps / P;
      const Val* vr = val + base + lane * P;
      int b = 0;
      for (; b + UBS <= nb; b += UBS) {
        uint32_t vw[UBS][VW];
#pragma unroll
        for (int u = 0; u < UBS; ++u) ld_words(vr + (b + u) * 32 * P, vw[u]);
#pragma unroll
        for (int u = 0; u < UBS; ++u)
#pragma unroll
          for (int t = 0; t < P; ++t)
            acc = C::mac(acc, run_at<Val>(vw[u], t), xs, c0 + __shfl_sync(0xffffffffu, off, (b + u) * P + t));
      }
      for (; b < nb; ++b) {
        uint32_t vw[VW];
        ld_words(vr + b * 32 * P, vw);
#pragma unroll
        for (int t = 0; t < P; ++t)
          acc = C::mac(acc, run_at<Val>(vw, t), xs, c0 + __shfl_sync(0xffffffffu, off, b * P + t));
      }
      for (int k = nb * P; k < steps; ++k)
        acc = C::mac(acc, ld_stream(vp + k * 32), xs, c0 + __shfl_sync(0xffffffffu, off, k));
    } else if constexpr (P > 0) {
      // Lane runs of P steps, UB runs per round (the last round predicated),
      // then the stride-32 tail, whose values load with the first round.
      const int nb = steps / P, k0 = nb * P;
      Val tv[TL];
#pragma unroll
      for (int t = 0; t < TL; ++t)
        if (k0 + t < steps) tv[t] = ld_stream(vp + (k0 + t) * 32);
      const Val* vr = val + base + lane * P;
      for (int b = 0; b < nb; b += UB) {
        uint32_t vw[UB][VW];
#pragma unroll
        for (int u = 0; u < UB; ++u)
          if (b + u < nb) ld_words(vr + (b + u) * 32 * P, vw[u]);
#pragma unroll
        for (int u = 0; u < UB; ++u)
          if (b + u < nb) {
#pragma unroll
            for (int t = 0; t < P; ++t)
              acc = C::mac(acc, run_at<Val>(vw[u], t), xs, c0 + __shfl_sync(0xffffffffu, off, (b + u) * P + t));
          }
      }
#pragma unroll
      for (int t = 0; t < TL; ++t)
        if (k0 + t < steps) acc = C::mac(acc, tv[t], xs, c0 + __shfl_sync(0xffffffffu, off, k0 + t));
    } else {
      // Chunks of U steps, the last one predicated.
      for (int k = 0; k < steps; k += U) {
        Val v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (k + u < steps) v[u] = ld_stream(vp + (k + u) * 32);
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (k + u < steps) acc = C::mac(acc, v[u], xs, c0 + __shfl_sync(0xffffffffu, off, k + u));
      }
    }
    if (lane < nrows) {
      const double s = C::to_f64(acc);
      y[rowid[row_base + lane]] = row_scale ? s * pow2(row_scale[row_base + lane]) : s;
    }
    return;
  }
  if (meta & kSlicedDelta) {
    // One row per lane, columns as 16-bit deltas from the row's first column.
    const Val* vp = val + base + lane;
    const uint16_t* dp = col16 + base + lane;
    int c = lane < nrows ? __ldg(first + row_base + lane) : 0;
    typename C::Acc acc = C::zero();
    if constexpr (P > 0 && kSerialTail) {
      constexpr int DW = P / 2;
      const int nb = steps / P;
      const Val* vr = val + base + lane * P;
      const uint16_t* dr = col16 + base + lane * P;
      int b = 0;
      for (; b + UBS <= nb; b += UBS) {
        uint32_t vw[UBS][VW], dw[UBS][DW];
#pragma unroll
        for (int u = 0; u < UBS; ++u) {
          ld_words(dr + (b + u) * 32 * P, dw[u]);
          ld_words(vr + (b + u) * 32 * P, vw[u]);
        }
#pragma unroll
        for (int u = 0; u < UBS; ++u)
#pragma unroll
          for (int t = 0; t < P; ++t) {
            c += run_at<uint16_t>(dw[u], t);
            acc = C::mac(acc, run_at<Val>(vw[u], t), xs, c);
          }
      }
      for (; b < nb; ++b) {
        uint32_t vw[VW], dw[DW];
        ld_words(dr + b * 32 * P, dw);
        ld_words(vr + b * 32 * P, vw);
#pragma unroll
        for (int t = 0; t < P; ++t) {
          c += run_at<uint16_t>(dw, t);
          acc = C::mac(acc, run_at<Val>(vw, t), xs, c);
        }
      }
      for (int k = nb * P; k < steps; ++k) {
        c += __ldcs(dp + k * 32);
        acc = C::mac(acc, ld_stream(vp + k * 32), xs, c);
      }
      if (lane < nrows) {
        const double s = C::to_f64(acc);
        y[rowid[row_base + lane]] = row_scale ? s * pow2(row_scale[row_base + lane]) : s;
      }
      return;
    } else if constexpr (P > 0) {
      constexpr int DW = P / 2;  // words per delta run
      const int nb = steps / P, k0 = nb * P;
      const int row = lane < nrows ? __ldg(rowid + row_base + lane) : 0;
      int dd[TL];
      Val tv[TL];
#pragma unroll
      for (int t = 0; t < TL; ++t)
        if (k0 + t < steps) {
          dd[t] = __ldcs(dp + (k0 + t) * 32);
          tv[t] = ld_stream(vp + (k0 + t) * 32);
        }
      const Val* vr = val + base + lane * P;
      const uint16_t* dr = col16 + base + lane * P;
      for (int b = 0; b < nb; b += UB) {
        uint32_t vw[UB][VW], dw[UB][DW];
#pragma unroll
        for (int u = 0; u < UB; ++u)
          if (b + u < nb) {
            ld_words(dr + (b + u) * 32 * P, dw[u]);
            ld_words(vr + (b + u) * 32 * P, vw[u]);
          }
#pragma unroll
        for (int u = 0; u < UB; ++u)
          if (b + u < nb) {
#pragma unroll
            for (int t = 0; t < P; ++t) {
              c += run_at<uint16_t>(dw[u], t);
              acc = C::mac(acc, run_at<Val>(vw[u], t), xs, c);
            }
          }
      }
#pragma unroll
      for (int t = 0; t < TL; ++t)
        if (k0 + t < steps) {
          c += dd[t];
          acc = C::mac(acc, tv[t], xs, c);
        }
      if (lane < nrows) {
        const double s = C::to_f64(acc);
        y[row] = row_scale ? s * pow2(row_scale[row_base + lane]) : s;
      }
      return;
    }
    int k = 0;
    for (; k + U <= steps; k += U) {
      int cc[U];
      typename C::Val v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        cc[u] = __ldcs(dp + (k + u) * 32);
        v[u] = ld_stream(vp + (k + u) * 32);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        c += cc[u];
        acc = C::mac(acc, v[u], xs, c);
      }
    }
    for (; k < steps; ++k) {
      c += __ldcs(dp + k * 32);
      acc = C::mac(acc, ld_stream(vp + k * 32), xs, c);
    }
    if (lane < nrows) {
      const double s = C::to_f64(acc);
      y[rowid[row_base + lane]] = row_scale ? s * pow2(row_scale[row_base + lane]) : s;
    }
    return;
  }
  const Val* vp = val + base + lane;
  const int32_t* cp = col + base + lane;
  typename C::Acc acc = C::zero();
  int k = 0;
  if constexpr (P > 0 && kSerialTail) {
    const int nb = steps / P;
    const Val* vr = val + base + lane * P;
    const int32_t* cr = col + base + lane * P;
    int b = 0;
    for (; b + UBS <= nb; b += UBS) {
      uint32_t vw[UBS][VW], cw[UBS][P];
#pragma unroll
      for (int u = 0; u < UBS; ++u) {
        ld_words(cr + (b + u) * 32 * P, cw[u]);
        ld_words(vr + (b + u) * 32 * P, vw[u]);
      }
#pragma unroll
      for (int u = 0; u < UBS; ++u)
#pragma unroll
        for (int t = 0; t < P; ++t) acc = C::mac(acc, run_at<Val>(vw[u], t), xs, (int)cw[u][t]);
    }
    for (; b < nb; ++b) {
      uint32_t vw[VW], cw[P];
      ld_words(cr + b * 32 * P, cw);
      ld_words(vr + b * 32 * P, vw);
#pragma unroll
      for (int t = 0; t < P; ++t) acc = C::mac(acc, run_at<Val>(vw, t), xs, (int)cw[t]);
    }
    k = nb * P;  // the stride-32 tail runs in the loops below
  } else if constexpr (P > 0) {
    const int nb = steps / P, k0 = nb * P;
    int tc[TL];
    Val tv[TL];
#pragma unroll
    for (int t = 0; t < TL; ++t)
      if (k0 + t < steps) {
        tc[t] = __ldcs(cp + (k0 + t) * 32);
        tv[t] = ld_stream(vp + (k0 + t) * 32);
      }
    const Val* vr = val + base + lane * P;
    const int32_t* cr = col + base + lane * P;
    for (int b = 0; b < nb; b += UB) {
      uint32_t vw[UB][VW], cw[UB][P];
#pragma unroll
      for (int u = 0; u < UB; ++u)
        if (b + u < nb) {
          ld_words(cr + (b + u) * 32 * P, cw[u]);
          ld_words(vr + (b + u) * 32 * P, vw[u]);
        }
#pragma unroll
      for (int u = 0; u < UB; ++u)
        if (b + u < nb) {
#pragma unroll
          for (int t = 0; t < P; ++t) acc = C::mac(acc, run_at<Val>(vw[u], t), xs, (int)cw[u][t]);
        }
    }
#pragma unroll
    for (int t = 0; t < TL; ++t)
      if (k0 + t < steps) acc = C::mac(acc, tv[t], xs, tc[t]);
    k = steps;
  }
  for (; k + U <= steps; k += U) {
    int c[U];
    typename C::Val v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      c[u] = __ldcs(cp + (k + u) * 32);
      v[u] = ld_stream(vp + (k + u) * 32);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) acc = C::mac(acc, v[u], xs, c[u]);
  }
  for (; k < steps; ++k) acc = C::mac(acc, ld_stream(vp + k * 32), xs, __ldcs(cp + k * 32));
  double s = C::to_f64(acc);
  for (int off = (1 << vwl) >> 1; off > 0; off >>= 1) s += __shfl_xor_sync(kFull, s, off);
  if (kind == kSlicedChunk) {
    if (lane == 0) chunk_sum[row_base] = chunk_scale ? s * pow2(chunk_scale[row_base]) : s;
  } else {
    const int g = lane >> vwl;
    if ((lane & ((1 << vwl) - 1)) == 0 && g < nrows)
      y[rowid[row_base + g]] = row_scale ? s * pow2(row_scale[row_base + g]) : s;
  }
}

__global__ void long_fixup_f64(const int32_t* __restrict__ long_row, const int32_t* __restrict__ long_first,
                               const int32_t* __restrict__ long_heavy, long long num_long, long long num_heavy,
                               long long heavy_sub, unsigned light_blocks, const double* __restrict__ chunk_sum,
                               double* __restrict__ y, int* flag) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && flag) *flag = 0;  // consumed: reset for the next call
  long_rows_fixup<double>(long_first, long_heavy, num_long, num_heavy, heavy_sub, light_blocks, chunk_sum,
                          [&](long long i, double s) { y[long_row[i]] = s; });
}

__global__ void reset_flag(int* flag) { *flag = 0; }

template <class C>
bool launch_mixed(const SlicedMatrix& m, const SlicedMixed& mx, const void* xs, double* y, cudaStream_t s,
                  const int* flag) {
  const long long grid = (m.num_tasks + kWarps - 1) / kWarps;
  if (grid > 0x7fffffffLL) {
    set_error("sliced: too many tasks for one launch");
    return false;
  }
  // Lane runs: 16 bytes of values (FP32 form 4 steps, BF16 form 8 steps).
  constexpr int R = std::is_same<typename C::Val, float>::value            ? 4
                    : std::is_same<typename C::Val, unsigned short>::value ? 8
                                                                            : 0;
  if (m.lane_run != 0 && m.lane_run != R) {
    set_error("sliced: lane runs do not match the precision form");
    return false;
  }
  auto pick_u = [&](auto run, auto sh) {
    constexpr int P = decltype(run)::value;
    constexpr bool SH = decltype(sh)::value;
    return m.unroll == 4    ? sliced_mixed_kernel<C, 4, P, SH>
           : m.unroll == 12 ? sliced_mixed_kernel<C, 12, P, SH>
           : m.unroll == 16 ? sliced_mixed_kernel<C, 16, P, SH>
                            : sliced_mixed_kernel<C, 8, P, SH>;
  };
  auto pick = [&](auto run) {
    return m.pat16 ? pick_u(run, std::true_type{}) : pick_u(run, std::false_type{});
  };
  auto kern = (R > 0 && m.lane_run) ? pick(std::integral_constant<int, R>{}) : pick(std::integral_constant<int, 0>{});
  // DF32 reads the pre-split (hi, lo) pairs; the FP64 values stay for the guard launch.
  const void* vals = std::is_same<typename C::Val, float2>::value ? static_cast<const void*>(mx.val_split) : m.val;
  kern<<<(unsigned)grid, kWarps * 32, 0, s>>>(m.tasks, m.num_tasks, static_cast<const typename C::Val*>(vals), m.col,
                                              m.rowid, xs, y, static_cast<double*>(m.chunk_sum), mx.row_scale,
                                              mx.chunk_scale, flag, m.col16, m.first, m.pat16, m.pf);
  return VNEC_CUDA(cudaGetLastError());
}

}  // namespace

bool sliced_mixed_spmv(const SlicedMatrix& m, const SlicedMixed& mx, const double* x, double* y, cudaStream_t s,
                       cudaEvent_t* ev) {
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[0], s))) return false;
  const int tb = 256;
  const long long nx = m.n_cols;
  const int xg = (int)std::min<long long>((nx + m.hot + tb - 1) / tb, 152LL * 16);
  int* flag = nullptr;
  if (nx > 0) {
    if (mx.precision == kPrecDF32) {
      x_split_kernel<<<xg, tb, 0, s>>>(x, static_cast<float2*>(mx.xbuf), nx, mx.flag, m.hot_cols, m.hot);
      flag = mx.flag;
    } else {
      x_to_f32_ext_kernel<<<xg, tb, 0, s>>>(x, static_cast<float*>(mx.xbuf), nx, m.hot_cols, m.hot);
    }
    if (!VNEC_CUDA(cudaGetLastError())) return false;
  }
  if (m.num_tasks > 0) {
    bool ok = false;
    switch (mx.precision) {
      case kPrecFP32: ok = launch_mixed<CodecF32>(m, mx, mx.xbuf, y, s, nullptr); break;
      case kPrecBF16: ok = launch_mixed<CodecBF16>(m, mx, mx.xbuf, y, s, nullptr); break;
      case kPrecDF32: ok = launch_mixed<CodecDF32>(m, mx, mx.xbuf, y, s, flag); break;
      default: set_error("sliced: unknown precision form"); return false;
    }
    if (!ok) return false;
  }
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[1], s))) return false;
  if (mx.precision == kPrecDF32 && m.num_tasks > 0) {
    // Guard: the FP64 sliced kernel, which returns at once unless the flag is set.
    if (!sliced_guard_f64(m, x, y, mx.flag, s)) return false;
  }
  if (m.num_long > 0) {
    const int b = 128;
    const FixupGrid g = fixup_grid(m, b);
    long_fixup_f64<<<g.total, b, 0, s>>>(m.long_row, m.long_first, m.long_heavy, m.num_long, m.num_heavy,
                                         m.heavy_sub, g.light, static_cast<const double*>(m.chunk_sum), y,
                                         mx.precision == kPrecDF32 ? mx.flag : nullptr);
    if (!VNEC_CUDA(cudaGetLastError())) return false;
  } else if (mx.precision == kPrecDF32) {
    reset_flag<<<1, 1, 0, s>>>(mx.flag);
    if (!VNEC_CUDA(cudaGetLastError())) return false;
  }
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[2], s))) return false;
  return true;
}

bool split_to_df32(const double* x, float2* xs, long long n, int* flag, cudaStream_t s) {
  if (n <= 0) return true;
  const int tb = 256;
  const int grid = (int)std::min<long long>((n + tb - 1) / tb, 152LL * 16);
  x_split_kernel<<<grid, tb, 0, s>>>(x, xs, n, flag, nullptr, 0);
  return VNEC_CUDA(cudaGetLastError());
}

bool round_to_f32(const double* x, float* x32, long long n, cudaStream_t s) {
  if (n <= 0) return true;
  const int tb = 256;
  const int grid = (int)std::min<long long>((n + tb - 1) / tb, 152LL * 16);
  x_to_f32_kernel<<<grid, tb, 0, s>>>(x, x32, n);
  return VNEC_CUDA(cudaGetLastError());
}

}  // namespace vnec

extern "C" SpB_Info SpB_VNEC_f64_to_f32_ext(const double* d_in, float* d_out, int64_t n, void* stream) {
  vnec::clear_error();
  if (n < 0 || (n > 0 && (!d_in || !d_out))) {
    vnec::set_error("SpB_VNEC_f64_to_f32_ext: invalid arguments");
    return SpB_FAILURE;
  }
  if (n == 0) return SpB_SUCCESS;
  const int tb = 256;
  const int grid = (int)std::min<long long>((n + tb - 1) / tb, 152LL * 16);
  vnec::x_to_f32_kernel<<<grid, tb, 0, static_cast<cudaStream_t>(stream)>>>(d_in, d_out, n);
  return VNEC_CUDA(cudaGetLastError()) ? SpB_SUCCESS : SpB_FAILURE;
}
