// Pipelined merge-path SpMV for sm_103a (FP64 y = A x, A stored in FP64).
//
// Same work decomposition as mp_kernels.cu (merge-path tiles of TPB*IPT
// items, VNEC-L counterpart, src/operation/src/spmv_vnec_L_for_mxv.c), with a
// GB300-oriented data path:
//
//  * Persistent CTAs walk their tiles (t = blockIdx.x + k*gridDim.x) through an
//    S-stage shared-memory pipeline.  One elected thread moves each tile's
//    values, columns and row ends with 1-D bulk async copies (the TMA bulk
//    engine), completion tracked by a per-stage mbarrier with a transaction
//    count.  Copy ranges are widened to 16-byte boundaries (the device arrays
//    are padded), so every copy is a legal bulk copy.
//  * While tile k is computed, the x values of tile k+1 are gathered with
//    cp.async (8-byte asynchronous copies into shared memory), so the
//    dependent x gather is off the critical path.
//  * Carries between the threads of a tile are combined with warp-level
//    segmented scans (log steps, stopping as soon as no lane needs more) and
//    one scan over the warp totals, instead of per-thread serial walks.  Row
//    results are collected in shared memory and written with coalesced stores.
//
// Two arithmetic modes:
//  * F64  — one FP64 FMA per nonzero (GB300 runs FP64 at 1/64 of FP32, about
//           0.6 T FMA/s, so FP64 instruction count is kept minimal);
//  * DF32 — the same sums in double-float arithmetic on the FP32 pipe: a and
//           x are split into (hi, lo) FP32 pairs with integer operations,
//           products use Dekker's exact product (Dekker 1971) via FMA, sums
//           use Knuth's TwoSum (relative error of a product ~2^-46, of a
//           sum ~2^-47, well inside the 1e-12 row-wise criterion for the
//           <= IPT items a thread accumulates before the FP64 combine).
//           Splitting needs |a|, |x| in [2^-40, 2^41) or zero: the plan checks
//           A once; a call that meets an x outside that range raises a device
//           flag and a guard launch recomputes the call in F64 mode.
// Every mbarrier wait is bounded (Mp2Matrix::wait_polls polls, 2^24 by
// default); on timeout the kernel raises a device error flag, drains its
// outstanding copies (bounded by the full limit) and exits.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "common.h"
#include "df32.cuh"
#include "ptx.cuh"

namespace vnec {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ DF df_add(DF a, DF b) {
  float t = __fadd_rn(a.s, b.s);
  float bb = __fsub_rn(t, a.s);
  float r = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bb)), __fsub_rn(b.s, bb));
  return DF{t, __fadd_rn(__fadd_rn(a.c, b.c), r)};
}

struct ModeF64 {
  using Acc = double;
  static constexpr bool kDF = false;
  __device__ static Acc zero() { return 0.0; }
  __device__ static Acc mac(Acc acc, double a, double x, bool&) { return fma(a, x, acc); }
  __device__ static Acc add(Acc a, Acc b) { return a + b; }
  __device__ static double to_f64(Acc a) { return a; }
  __device__ static Acc shfl_up(Acc v, int d) { return __shfl_up_sync(kFull, v, d); }
};

struct ModeDF32 {
  using Acc = DF;
  static constexpr bool kDF = true;
  __device__ static Acc zero() { return DF{0.0f, 0.0f}; }
  __device__ static Acc mac(Acc acc, double a, double x, bool& bad) {
    float ah, al, xh, xl;
    bool ok = df_split(a, ah, al);
    ok &= df_split(x, xh, xl);
    bad |= !ok;
    return df_mac(acc, ah, al, xh, xl);
  }
  __device__ static Acc add(Acc a, Acc b) { return df_add(a, b); }
  __device__ static double to_f64(Acc a) { return df_to_f64(a); }
  __device__ static Acc shfl_up(Acc v, int d) {
    return DF{__shfl_up_sync(kFull, v.s, d), __shfl_up_sync(kFull, v.c, d)};
  }
};

struct Mp2Args {
  const int* row_end;
  const int32_t* col;
  const double* val;
  const double* x;
  double* y;
  const int* tile_row;
  const int* tile_nz;
  int* carry_row;
  double* carry_val;
  int num_tiles;
  int* flags;  // [0]: x outside the DF32 range this call, [1]: pipeline timeout
  int guard;   // 1: this launch only runs when flags[0] is set (F64 recompute)
  int wait_polls;  // polls of a pipeline wait before it reports a timeout
};

template <int TPB, int IPT>
struct Mp2Layout {
  static constexpr int kIPC = TPB * IPT;
  static constexpr int kCap = kIPC + 8;  // aligned copy ranges add at most 6 elements
  static constexpr size_t kStage = (size_t)kCap * (8 + 4 + 4);
  static constexpr int kWarps = TPB / 32;
};

template <int TPB, int IPT, int S>
constexpr size_t mp2_smem_bytes() {
  using L = Mp2Layout<TPB, IPT>;
  return S * L::kStage + (size_t)2 * L::kCap * 8 + (size_t)L::kCap * 8 + (size_t)L::kWarps * (8 + 8 + 4) + 16 +
         (size_t)S * 8 + 16;
}

template <class M, int TPB, int IPT, int S>
__global__ void __launch_bounds__(TPB) mp2_kernel(const Mp2Args a) {
  using L = Mp2Layout<TPB, IPT>;
  using Acc = typename M::Acc;
  constexpr int kCap = L::kCap, kW = L::kWarps;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* const stage_base = smem;
  double* const xbuf = reinterpret_cast<double*>(smem + S * L::kStage);  // [2][kCap]
  Acc* const srow = reinterpret_cast<Acc*>(xbuf + 2 * kCap);               // [kCap]
  Acc* const wv = srow + kCap;                                             // [kW]
  Acc* const wcin = wv + kW;                                               // [kW]
  int* const wo = reinterpret_cast<int*>(wcin + kW);                       // [kW]
  uint64_t* const bar = reinterpret_cast<uint64_t*>(
      (reinterpret_cast<uintptr_t>(wo + kW) + 15) & ~static_cast<uintptr_t>(15));  // [S]

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (a.guard && *reinterpret_cast<volatile int*>(a.flags) == 0) return;
  const int nk = (a.num_tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  if (nk <= 0) return;

  auto sval = [&](int s) { return reinterpret_cast<double*>(stage_base + s * L::kStage); };
  auto scol = [&](int s) { return reinterpret_cast<int*>(stage_base + s * L::kStage + kCap * 8); };
  auto send = [&](int s) { return reinterpret_cast<int*>(stage_base + s * L::kStage + kCap * 12); };

  auto issue = [&](int k) {  // elected thread: bulk copies of tile k into stage k % S
    const int s = k % S;
    const int t = (int)blockIdx.x + k * (int)gridDim.x;
    const int x0 = a.tile_row[t], y0 = a.tile_nz[t], x1 = a.tile_row[t + 1], y1 = a.tile_nz[t + 1];
    const int y0a = y0 & ~3, y1a = (y1 + 3) & ~3, x0a = x0 & ~3, x1a = (x1 + 3) & ~3;
    const uint32_t bv = (uint32_t)(y1a - y0a) * 8u, bc = (uint32_t)(y1a - y0a) * 4u, be = (uint32_t)(x1a - x0a) * 4u;
    mbar_arrive_expect_tx(&bar[s], bv + bc + be);
    if (bv) {
      bulk_g2s(sval(s), a.val + y0a, bv, &bar[s]);
      bulk_g2s(scol(s), a.col + y0a, bc, &bar[s]);
    }
    if (be) bulk_g2s(send(s), a.row_end + x0a, be, &bar[s]);
  };

  auto gather = [&](int k) {  // all threads: cp.async x[col] of tile k into xbuf[k & 1]
    const int s = k % S;
    const int t = (int)blockIdx.x + k * (int)gridDim.x;
    const int y0 = a.tile_nz[t], y1 = a.tile_nz[t + 1];
    const int off = y0 - (y0 & ~3);
    const int* c = scol(s) + off;
    double* xb = xbuf + (k & 1) * kCap;
    for (int i = tid; i < y1 - y0; i += TPB) cp_async8(xb + i, a.x + c[i]);
    cp_async_commit();
  };

  // Drains the copies this CTA still has in flight before exiting on an error.
  // These waits keep the full kSpinLimit whatever a.wait_polls is, so no CTA
  // leaves while a bulk copy into its shared memory is still running.
  auto drain_and_fail = [&](int k_first_unwaited, int k_end) {
    if (tid == 0) {
      atomicExch(a.flags + 1, 1);
      for (int k = k_first_unwaited; k < k_end; ++k) mbar_wait_bounded(&bar[k % S], (uint32_t)((k / S) & 1), kSpinLimit);
    }
    cp_async_wait_all();
  };

  if (tid == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (tid == 0)
    for (int k = 0; k < S && k < nk; ++k) issue(k);
  {
    const bool ok = mbar_wait_bounded(&bar[0], 0u, a.wait_polls);
    if (__syncthreads_or(!ok)) {
      drain_and_fail(0, nk < S ? nk : S);
      return;
    }
  }
  gather(0);

  bool bad = false;  // DF32: an operand left the split range
  for (int k = 0; k < nk; ++k) {
    const int s = k % S;
    if (k + 1 < nk) {
      const bool ok = mbar_wait_bounded(&bar[(k + 1) % S], (uint32_t)(((k + 1) / S) & 1), a.wait_polls);
      if (__syncthreads_or(!ok)) {
        drain_and_fail(k + 1, (k + S < nk) ? k + S : nk);
        return;
      }
      gather(k + 1);
      cp_async_wait_one_pending();
    } else {
      cp_async_wait_all();
    }
    __syncthreads();

    const int t = (int)blockIdx.x + k * (int)gridDim.x;
    const int x0 = a.tile_row[t], y0 = a.tile_nz[t], x1 = a.tile_row[t + 1], y1 = a.tile_nz[t + 1];
    const int nrows = x1 - x0, nnz = y1 - y0, total = nrows + nnz;
    const double* v = sval(s) + (y0 - (y0 & ~3));
    const int* e = send(s) + (x0 - (x0 & ~3));
    const double* xb = xbuf + (k & 1) * kCap;

    // Per-thread merge path over IPT items.
    const int d = min(tid * IPT, total);
    int lo = max(d - nnz, 0), hi = min(d, nrows);
    while (lo < hi) {
      const int p = (lo + hi) >> 1;
      if (e[p] - y0 <= d - p - 1)
        lo = p + 1;
      else
        hi = p;
    }
    int rr = lo, kk = d - lo;
    const int dend = min(d + IPT, total);
    Acc acc = M::zero(), firstv = M::zero();
    int first = -1;
#pragma unroll
    for (int it = 0; it < IPT; ++it) {
      if (d + it < dend) {
        if (rr < nrows && e[rr] - y0 <= kk) {
          if (first < 0) {
            first = rr;
            firstv = acc;
          } else {
            srow[rr] = acc;
          }
          acc = M::zero();
          ++rr;
        } else {
          acc = M::mac(acc, v[kk], xb[kk], bad);
          ++kk;
        }
      }
    }

    // Warp segmented scan of the tail partials: run sums restart after a
    // thread that emitted a row.
    Acc run = acc;
    int open = first < 0;
    for (int dist = 1; dist < 32; dist <<= 1) {
      if (!__ballot_sync(kFull, open && lane >= dist)) break;
      const Acc up = M::shfl_up(run, dist);
      const int up_open = __shfl_up_sync(kFull, open, dist);
      if (open && lane >= dist) {
        run = M::add(up, run);
        open = up_open;
      }
    }
    if (lane == 31) {
      wv[warp] = run;
      wo[warp] = open;
    }
    __syncthreads();
    if (warp == 0) {
      Acc cv = lane < kW ? wv[lane] : M::zero();
      int co = lane < kW ? wo[lane] : 0;
      for (int dist = 1; dist < kW; dist <<= 1) {
        const Acc up = M::shfl_up(cv, dist);
        const int up_open = __shfl_up_sync(kFull, co, dist);
        if (co && lane >= dist) {
          cv = M::add(up, cv);
          co = up_open;
        }
      }
      const Acc ex = M::shfl_up(cv, 1);
      if (lane < kW) wcin[lane] = lane == 0 ? M::zero() : ex;
    }
    __syncthreads();
    const Acc prev = M::shfl_up(run, 1);
    const int prev_open = __shfl_up_sync(kFull, open, 1);
    if (first >= 0) {
      Acc cin;
      if (lane == 0)
        cin = wcin[warp];
      else
        cin = prev_open ? M::add(prev, wcin[warp]) : prev;
      srow[first] = M::add(firstv, cin);
    }
    if (tid == TPB - 1) {
      const Acc out = open ? M::add(run, wcin[warp]) : run;
      a.carry_row[t] = x1;
      a.carry_val[t] = M::to_f64(out);
    }
    __syncthreads();
    for (int r = tid; r < nrows; r += TPB) a.y[x0 + r] = M::to_f64(srow[r]);
    __syncthreads();
    if (tid == 0 && k + S < nk) {
      fence_proxy_async_shared();
      issue(k + S);
    }
  }
  if (M::kDF && __syncthreads_or(bad) && tid == 0) atomicExch(a.flags, 1);
}

// Cross-tile carries (as in mp_kernels.cu), plus reset of the per-call
// DF32 range flag for the next call.  After a pipeline timeout (flags[1]) the
// skipped tiles' carry slots hold an earlier call's rows (or the zeros of plan
// build): the row check keeps every add inside y, whose values the status
// call then reports as invalid.
__global__ void mp2_fixup_kernel(const int* __restrict__ carry_row, const double* __restrict__ carry_val,
                                 int num_tiles, int n_rows, double* __restrict__ y, int* flags) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) flags[0] = 0;
  if (t >= num_tiles) return;
  const int r = carry_row[t];
  if (r < 0 || r >= n_rows) return;
  if (t > 0 && carry_row[t - 1] == r) return;
  double s = 0.0;
  for (int u = t; u < num_tiles && carry_row[u] == r; ++u) s += carry_val[u];
  y[r] += s;
}

template <class M, int TPB, int IPT, int S>
bool launch_one(const Mp2Args& args, int sms, cudaStream_t st) {
  auto kern = mp2_kernel<M, TPB, IPT, S>;
  constexpr size_t smem = mp2_smem_bytes<TPB, IPT, S>();
  static int per_sm = 0;
  if (per_sm == 0) {
    if (!VNEC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
      return false;
    if (!VNEC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TPB, smem))) return false;
    if (per_sm < 1) {
      set_error("pipelined merge-path kernel does not fit on an SM");
      return false;
    }
  }
  const int grid = std::min<long long>((long long)sms * per_sm, args.num_tiles);
  kern<<<grid, TPB, smem, st>>>(args);
  return VNEC_CUDA(cudaGetLastError());
}

template <int TPB, int IPT, int S>
bool launch_shape(const Mp2Matrix& m, bool df32, const double* x, double* y, cudaStream_t st, cudaEvent_t* ev) {
  Mp2Args args{static_cast<const int*>(m.row_end), m.col, m.val, x, y, static_cast<const int*>(m.tile_row),
               static_cast<const int*>(m.tile_nz), static_cast<int*>(m.carry_row), m.carry_val,
               (int)m.num_tiles, m.flags, 0, m.wait_polls};
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[0], st))) return false;
  if (df32) {
    if (!launch_one<ModeDF32, TPB, IPT, S>(args, m.sms, st)) return false;
    if (ev && !VNEC_CUDA(cudaEventRecord(ev[1], st))) return false;
    args.guard = 1;  // F64 recompute, runs only if the DF32 launch met an x out of range
  }
  if (!launch_one<ModeF64, TPB, IPT, S>(args, m.sms, st)) return false;
  if (!df32 && ev && !VNEC_CUDA(cudaEventRecord(ev[1], st))) return false;
  const int fb = 256;
  const int fg = (int)((m.num_tiles + fb - 1) / fb);
  mp2_fixup_kernel<<<fg, fb, 0, st>>>(static_cast<const int*>(m.carry_row), m.carry_val, (int)m.num_tiles,
                                       (int)m.n_rows, y, m.flags);
  if (!VNEC_CUDA(cudaGetLastError())) return false;
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[2], st))) return false;
  return true;
}

}  // namespace

size_t mp2_smem(int tpb, int ipt, int stages) {
  if (tpb == 256 && ipt == 7 && stages == 2) return mp2_smem_bytes<256, 7, 2>();
  if (tpb == 256 && ipt == 7 && stages == 3) return mp2_smem_bytes<256, 7, 3>();
  if (tpb == 256 && ipt == 12 && stages == 2) return mp2_smem_bytes<256, 12, 2>();
  if (tpb == 128 && ipt == 12 && stages == 3) return mp2_smem_bytes<128, 12, 3>();
  if (tpb == 512 && ipt == 5 && stages == 2) return mp2_smem_bytes<512, 5, 2>();
  return 0;
}

bool mp2_spmv(const Mp2Matrix& m, bool df32, const double* x, double* y, cudaStream_t s, cudaEvent_t* ev) {
  if (m.n_rows == 0) return true;
  const int tpb = m.shape.tpb, ipt = m.shape.ipt, st = m.stages;
#define VNEC_MP2_CASE(T, I, S) \
  if (tpb == T && ipt == I && st == S) return launch_shape<T, I, S>(m, df32, x, y, s, ev);
  VNEC_MP2_CASE(256, 7, 2)
  VNEC_MP2_CASE(256, 7, 3)
  VNEC_MP2_CASE(256, 12, 2)
  VNEC_MP2_CASE(128, 12, 3)
  VNEC_MP2_CASE(512, 5, 2)
#undef VNEC_MP2_CASE
  set_error("pipelined merge-path: unsupported tile shape / stage count");
  return false;
}

}  // namespace vnec
