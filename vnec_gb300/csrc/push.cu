// Push-side sparse-matrix x sparse-vector product (SpMSpV, the operation the
// reference declares as SpB_vxm, OpenSparseBLAS.h:1940, without a body):
// y = A x for a sparse x given as (index, value) pairs, touching only the
// columns of A that x selects.  A is held as its CSC (the CSR of A^T); one
// warp per nonzero of x streams that column and adds value * x_j into y with
// FP64 (FP32) atomics, so the order of the additions into one y entry varies
// from run to run (results agree to rounding, not bit for bit).  An index
// outside [0, n_cols) is skipped and recorded in a device status word.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "common.h"
#include "push.h"

namespace vnec {
namespace {

constexpr int kWarps = 8;

template <typename V>
__global__ void __launch_bounds__(kWarps * 32)
push_kernel(long long nx, const int32_t* __restrict__ idx, const V* __restrict__ xval, const int64_t* __restrict__ cp,
            const int32_t* __restrict__ row, const V* __restrict__ val, long long n_cols, V* __restrict__ y,
            int* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * kWarps;
  for (long long w = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5); w < nx; w += nw) {
    const long long j = idx ? (long long)__ldg(idx + w) : w;
    if (j < 0 || j >= n_cols) {
      if (lane == 0) atomicExch(status, 1);
      continue;
    }
    const V xj = __ldg(xval + w);
    if (xj == V(0)) continue;
    const long long b = __ldg(cp + j), e = __ldg(cp + j + 1);
    for (long long p = b + lane; p < e; p += 32) atomicAdd(y + __ldg(row + p), __ldcs(val + p) * xj);
  }
}

template <typename V>
bool launch(const PushMatrix& m, long long nx, const int32_t* idx, const void* xval, void* y, cudaStream_t s) {
  if (m.n_rows > 0 && !VNEC_CUDA(cudaMemsetAsync(y, 0, sizeof(V) * (size_t)m.n_rows, s))) return false;
  if (nx <= 0) return true;
  const long long grid = std::min<long long>((nx + kWarps - 1) / kWarps, 152LL * 32);
  push_kernel<V><<<(unsigned)grid, kWarps * 32, 0, s>>>(nx, idx, static_cast<const V*>(xval), m.col_ptr, m.row,
                                                       static_cast<const V*>(m.val), m.n_cols, static_cast<V*>(y),
                                                       m.status);
  return VNEC_CUDA(cudaGetLastError());
}

}  // namespace

bool push_spmspv(const PushMatrix& m, bool fp64, long long nx, const int32_t* idx, const void* xval, void* y,
                 cudaStream_t s) {
  return fp64 ? launch<double>(m, nx, idx, xval, y, s) : launch<float>(m, nx, idx, xval, y, s);
}

}  // namespace vnec
