// Measurement kernel: the memory traffic of one CSR nonzero without the row
// structure.  For i in [0, n): one coalesced 8-byte value and 4-byte column
// read, one 8-byte gather x[col[i]], one FP64 FMA into a per-thread sum; each
// block writes its partial sum.  bench.py times it on a matrix's own column
// stream and on uniform random columns over windows of several sizes: the rate
// it reaches is the device's ceiling for a kernel that gathers x once per
// nonzero, which no SpMV layout of the same matrix can exceed by more than its
// cache reuse.  Not used by any SpMV path.

#include <cuda_runtime.h>

#include <cstdint>

#include "common.h"
#include "vnec_gb300.h"

namespace vnec {
namespace {

constexpr int kCeilTpb = 256;
constexpr int kCeilU = 16;  // independent loads in flight per thread

__global__ void __launch_bounds__(kCeilTpb)
stream_gather_kernel(const double* __restrict__ x, const int32_t* __restrict__ col, const double* __restrict__ val,
                     long long n, double* __restrict__ out) {
  const long long tid = (long long)blockIdx.x * kCeilTpb + threadIdx.x;
  const long long stride = (long long)gridDim.x * kCeilTpb;
  double acc = 0.0;
  for (long long base = tid; base < n; base += kCeilU * stride) {
    int c[kCeilU];
    double v[kCeilU], xv[kCeilU];
#pragma unroll
    for (int u = 0; u < kCeilU; ++u) {
      const long long i = base + u * stride;
      c[u] = i < n ? __ldcs(col + i) : 0;
      v[u] = i < n ? __ldcs(val + i) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kCeilU; ++u) xv[u] = base + u * stride < n ? __ldg(x + c[u]) : 0.0;
#pragma unroll
    for (int u = 0; u < kCeilU; ++u) acc = fma(v[u], xv[u], acc);
  }
  __shared__ double part[kCeilTpb / 32];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kCeilTpb / 32; ++w) s += part[w];
    out[blockIdx.x] = s;
  }
}

}  // namespace
}  // namespace vnec

extern "C" SpB_Info SpB_VNEC_stream_gather_ext(const double* d_x, int64_t n_x, const int32_t* d_col,
                                               const double* d_val, int64_t n, double* d_out, void* stream) {
  using namespace vnec;
  clear_error();
  if (n < 0 || n_x < 0 || (n > 0 && (!d_x || !d_col || !d_val || !d_out))) {
    set_error("SpB_VNEC_stream_gather_ext: invalid arguments");
    return SpB_FAILURE;
  }
  if (n == 0) return SpB_SUCCESS;
  (void)n_x;  // columns must lie in [0, n_x): the caller's guarantee, as for every SpMV entry point
  stream_gather_kernel<<<SPB_VNEC_STREAM_GATHER_BLOCKS, kCeilTpb, 0, static_cast<cudaStream_t>(stream)>>>(
      d_x, d_col, d_val, n, d_out);
  return VNEC_CUDA(cudaGetLastError()) ? SpB_SUCCESS : SpB_FAILURE;
}
