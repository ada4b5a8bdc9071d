// Device reductions for chains of SpMV calls that stay on the GPU (power
// iterations: a dangling-mass dot product, an L1 convergence distance).  Two
// launches with a fixed summation order, so the result has the same bits on
// every run: SPB_VNEC_DOT_BLOCKS blocks write partial sums, one block adds
// them in block order.

#include <cuda_runtime.h>

#include <cstdint>

#include "common.h"
#include "vnec_gb300.h"

namespace vnec {
namespace {

constexpr int kDotTpb = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
  return s;
}

__global__ void __launch_bounds__(kDotTpb)
dot_partial_kernel(long long n, const double* __restrict__ a, const double* __restrict__ b, int mode,
                   double* __restrict__ partial) {
  __shared__ double sh[kDotTpb / 32];
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * kDotTpb + threadIdx.x; i < n; i += (long long)gridDim.x * kDotTpb)
    acc = mode == 0 ? fma(a[i], b[i], acc) : acc + fabs(a[i] - b[i]);
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kDotTpb)
dot_final_kernel(const double* __restrict__ partial, int n, double* __restrict__ out) {
  __shared__ double sh[kDotTpb / 32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += kDotTpb) acc += partial[i];
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) out[0] = s;
}

}  // namespace
}  // namespace vnec

extern "C" SpB_Info SpB_VNEC_dot_ext(int64_t n, const double* d_a, const double* d_b, int mode, double* d_partial,
                                     double* d_out, void* stream) {
  using namespace vnec;
  clear_error();
  if (n < 0 || (mode != 0 && mode != 1) || !d_partial || !d_out || (n > 0 && (!d_a || !d_b))) {
    set_error("SpB_VNEC_dot_ext: invalid arguments");
    return SpB_FAILURE;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  dot_partial_kernel<<<SPB_VNEC_DOT_BLOCKS, kDotTpb, 0, s>>>(n, d_a, d_b, mode, d_partial);
  if (!VNEC_CUDA(cudaGetLastError())) return SpB_FAILURE;
  dot_final_kernel<<<1, kDotTpb, 0, s>>>(d_partial, SPB_VNEC_DOT_BLOCKS, d_out);
  return VNEC_CUDA(cudaGetLastError()) ? SpB_SUCCESS : SpB_FAILURE;
}
