// Matrix features for the learned kernel selection (tuner.h), computed on the
// GPU: one warp per row (lanes stride over the row's entries) accumulates row
// length, column span, aligned 4-column blocks and per-column counts; a
// second pass over the column counts measures the hot-column share.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"
#include "host.h"
#include "tuner.h"

namespace vnec {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarps = 8;

struct FeatAcc {
  unsigned long long hist[6];
  unsigned long long blocks;      // aligned 4-column blocks
  unsigned long long dense_rows;  // non-empty rows with nnz >= 2 * blocks
  unsigned long long nonempty;
  unsigned long long max_len;
  unsigned long long hot_nnz;
  double sum_len2;
  double span;  // sum over non-empty rows of span / n_cols
};

__device__ __forceinline__ int len_bin(long long len) {
  return len == 0 ? 0 : len < 4 ? 1 : len < 16 ? 2 : len < 64 ? 3 : len < 1024 ? 4 : 5;
}

__global__ void __launch_bounds__(kWarps * 32)
row_features_kernel(long long n_rows, long long n_cols, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                    unsigned* __restrict__ col_count, FeatAcc* __restrict__ acc) {
  __shared__ unsigned long long s_u[kWarps][11];
  __shared__ double s_d[kWarps][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long u[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // hist[6], blocks, dense, nonempty, max, unused
  double len2 = 0.0, span = 0.0;
  const long long nw = (long long)gridDim.x * kWarps;
  for (long long r = (long long)blockIdx.x * kWarps + warp; r < n_rows; r += nw) {
    const long long b = rp[r], e = rp[r + 1], len = e - b;
    int mn = 0x7fffffff, mx = -1;
    unsigned nb = 0;
    for (long long q = b + lane; q < e; q += 32) {
      const int c = col[q];
      mn = min(mn, c);
      mx = max(mx, c);
      if (q == b || (col[q - 1] >> 2) != (c >> 2)) ++nb;
      atomicAdd(col_count + c, 1u);
    }
    for (int off = 16; off > 0; off >>= 1) {
      mn = min(mn, __shfl_xor_sync(kFull, mn, off));
      mx = max(mx, __shfl_xor_sync(kFull, mx, off));
      nb += __shfl_xor_sync(kFull, nb, off);
    }
    if (lane == 0) {
      ++u[len_bin(len)];
      len2 += (double)len * (double)len;
      if (len > 0) {
        u[6] += nb;
        if (len >= 2 * (long long)nb) ++u[7];
        ++u[8];
        u[9] = max(u[9], (unsigned long long)len);
        span += (double)(mx - mn + 1) / (double)n_cols;
      }
    }
  }
  if (lane == 0) {
    for (int i = 0; i < 11; ++i) s_u[warp][i] = u[i];
    s_d[warp][0] = len2;
    s_d[warp][1] = span;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kWarps; ++w) {
      for (int i = 0; i < 9; ++i) s_u[0][i] += s_u[w][i];
      s_u[0][9] = max(s_u[0][9], s_u[w][9]);
      s_d[0][0] += s_d[w][0];
      s_d[0][1] += s_d[w][1];
    }
    for (int i = 0; i < 6; ++i) atomicAdd(&acc->hist[i], s_u[0][i]);
    atomicAdd(&acc->blocks, s_u[0][6]);
    atomicAdd(&acc->dense_rows, s_u[0][7]);
    atomicAdd(&acc->nonempty, s_u[0][8]);
    atomicMax(&acc->max_len, s_u[0][9]);
    atomicAdd(&acc->sum_len2, s_d[0][0]);
    atomicAdd(&acc->span, s_d[0][1]);
  }
}

__global__ void hot_share_kernel(long long n_cols, const unsigned* __restrict__ col_count, unsigned threshold,
                                 FeatAcc* __restrict__ acc) {
  unsigned long long s = 0;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n_cols; c += (long long)gridDim.x * blockDim.x)
    if (col_count[c] >= threshold) s += col_count[c];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(kFull, s, off);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(&acc->hot_nnz, s);
}

inline float clamp01(double v) { return (float)std::min(1.0, std::max(0.0, v)); }

}  // namespace

bool matrix_features_device(int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t* d_row_ptr,
                            const int32_t* d_col, float* out, cudaStream_t s) {
  DeviceBuffer accb, cnt;
  if (!accb.alloc(sizeof(FeatAcc)) || !cnt.alloc(sizeof(unsigned) * (size_t)std::max<int64_t>(n_cols, 1)) ||
      !VNEC_CUDA(cudaMemsetAsync(accb.ptr, 0, sizeof(FeatAcc), s)) ||
      !VNEC_CUDA(cudaMemsetAsync(cnt.ptr, 0, sizeof(unsigned) * (size_t)std::max<int64_t>(n_cols, 1), s)))
    return false;
  FeatAcc* acc = accb.as<FeatAcc>();
  if (n_rows > 0 && n_cols > 0) {
    const long long grid = std::min<long long>((n_rows + kWarps - 1) / kWarps, 152LL * 16);
    row_features_kernel<<<(unsigned)grid, kWarps * 32, 0, s>>>(n_rows, n_cols, d_row_ptr, d_col, cnt.as<unsigned>(),
                                                               acc);
    if (!VNEC_CUDA(cudaGetLastError())) return false;
    const double mean = (double)nnz / (double)n_cols;
    const unsigned thr = (unsigned)std::max(1.0, std::ceil(8.0 * mean));
    hot_share_kernel<<<(unsigned)std::min<long long>((n_cols + 255) / 256, 152LL * 8), 256, 0, s>>>(
        n_cols, cnt.as<unsigned>(), thr, acc);
    if (!VNEC_CUDA(cudaGetLastError())) return false;
  }
  FeatAcc h;
  if (!VNEC_CUDA(cudaMemcpyAsync(&h, acc, sizeof(h), cudaMemcpyDeviceToHost, s)) ||
      !VNEC_CUDA(cudaStreamSynchronize(s)))
    return false;
  const double nr = (double)std::max<int64_t>(n_rows, 1);
  const double mean_len = (double)nnz / nr;
  const double var = std::max(0.0, h.sum_len2 / nr - mean_len * mean_len);
  const double cv = mean_len > 0 ? std::sqrt(var) / mean_len : 0.0;
  const double ne = (double)std::max<unsigned long long>(h.nonempty, 1);
  out[0] = (float)(std::log2((double)n_rows + 1.0) / 24.0);
  out[1] = (float)(std::log2((double)n_cols + 1.0) / 24.0);
  out[2] = (float)(std::log2((double)nnz + 1.0) / 32.0);
  out[3] = (float)(std::log2(mean_len + 1.0) / 12.0);
  out[4] = (float)(std::min(cv, 8.0) / 8.0);
  out[5] = (float)(std::log2((double)h.max_len + 1.0) / 16.0);
  for (int i = 0; i < 6; ++i) out[6 + i] = (float)((double)h.hist[i] / nr);
  out[12] = clamp01(h.span / ne);
  out[13] = h.blocks ? clamp01((double)nnz / (4.0 * (double)h.blocks)) : 0.f;
  out[14] = clamp01((double)h.dense_rows / ne);
  out[15] = nnz ? clamp01((double)h.hot_nnz / (double)nnz) : 0.f;
  return true;
}

bool matrix_features(const CsrView& v, float* out) {
  std::vector<int64_t> rp((size_t)v.n_rows + 1);
  for (int64_t r = 0; r <= v.n_rows; ++r) rp[(size_t)r] = v.row_begin(r);
  DeviceBuffer drp, dcol;
  if (!drp.alloc(sizeof(int64_t) * rp.size()) || !dcol.alloc(sizeof(int32_t) * (size_t)std::max<int64_t>(v.nnz, 1)))
    return false;
  if (!VNEC_CUDA(cudaMemcpy(drp.ptr, rp.data(), sizeof(int64_t) * rp.size(), cudaMemcpyHostToDevice))) return false;
  if (v.nnz > 0) {
    if (v.idx) {
      if (!VNEC_CUDA(cudaMemcpy(dcol.ptr, v.idx, sizeof(int32_t) * (size_t)v.nnz, cudaMemcpyHostToDevice))) return false;
    } else {
      std::vector<int32_t> c((size_t)v.nnz);
      convert_cols(v, c.data());
      if (!VNEC_CUDA(cudaMemcpy(dcol.ptr, c.data(), sizeof(int32_t) * c.size(), cudaMemcpyHostToDevice))) return false;
    }
  }
  return matrix_features_device(v.n_rows, v.n_cols, v.nnz, drp.as<int64_t>(), dcol.as<int32_t>(), out, nullptr);
}

}  // namespace vnec
