// Internal declarations shared by the host plan code and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <string>

namespace vnec {

// ---------------------------------------------------------------------------
// Errors: every C-ABI entry point reports failures through SpB_Info and a
// thread-local message (the reference prints and exit()s instead,
// src/core/src/SpB_Error.c:4-8).
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
void clear_error();
const char* last_error();

bool cuda_ok(cudaError_t e, const char* what);
#define VNEC_CUDA(call) ::vnec::cuda_ok((call), #call)

// Owning device allocation.
// Runs `set` (a per-function CUDA attribute setting) once per device for one
// call site: `mask` holds a bit per device ordinal already configured.
template <class F>
bool once_per_device(std::atomic<unsigned long long>& mask, F set) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    set_error("cudaGetDevice failed");
    return false;
  }
  const unsigned long long bit = 1ull << (dev & 63);
  if (mask.load(std::memory_order_acquire) & bit) return true;
  if (!set()) return false;
  mask.fetch_or(bit, std::memory_order_acq_rel);
  return true;
}

// Truncation split of an FP64 value into FP32 hi (sign, exponent, top 23
// mantissa bits) and lo (the remaining 29 bits, normalised and truncated to
// 24): the host twin of the device split used for X, so that values and X of
// the DF32 form are split the same way.  Needs a zero or |v| in [2^-40, 2^41).
inline void split_df_host(double v, float* hi, float* lo) {
  uint64_t b;
  std::memcpy(&b, &v, 8);
  const uint32_t sign = (uint32_t)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7ff);
  const uint64_t m = b & 0xFFFFFFFFFFFFFull;
  if (e == 0 && m == 0) {
    *hi = 0.f;
    *lo = 0.f;
    return;
  }
  const int E = e - 1023;
  const uint32_t hb = sign | ((uint32_t)(E + 127) << 23) | (uint32_t)(m >> 29);
  const uint32_t rem = (uint32_t)(m & 0x1FFFFFFFull);
  const int msb = 31 - __builtin_clz(rem | 1u);
  const uint32_t mant = msb > 23 ? (rem >> (msb - 23)) : (rem << (23 - msb));
  const uint32_t lb = rem ? (sign | ((uint32_t)(E - 52 + msb + 127) << 23) | (mant & 0x7FFFFFu)) : 0u;
  std::memcpy(hi, &hb, 4);
  std::memcpy(lo, &lb, 4);
}

// A non-blocking stream and two timing events, released on every exit path
// (the timing loops of the autotuners).
struct TimingStream {
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  TimingStream() = default;
  TimingStream(const TimingStream&) = delete;
  TimingStream& operator=(const TimingStream&) = delete;
  ~TimingStream() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
  }
  bool create() {
    return cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess && cudaEventCreate(&e0) == cudaSuccess &&
           cudaEventCreate(&e1) == cudaSuccess;
  }
};

struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  ~DeviceBuffer() { release(); }
  bool alloc(size_t n);
  void release();
  template <typename T> T* as() const { return static_cast<T*>(ptr); }
};

// ---------------------------------------------------------------------------
// Merge-path CSR kernels (the GPU counterpart of VNEC-L,
// src/operation/src/spmv_vnec_L_for_mxv.c).
// ---------------------------------------------------------------------------

// Tile shape of the merge-path kernels: threads per CTA x merge items per thread.
struct MpShape {
  int tpb = 256;
  int ipt = 7;
  int64_t items_per_tile() const { return (int64_t)tpb * ipt; }
};

// Value/accumulation forms of the merge-path kernel.
enum class MpForm : int {
  kF64 = 0,     // FP64 values and x, FP64 accumulation (plain form)
  kF32 = 1,     // FP32 values and x, FP32 accumulation (the reference's FP32 twin)
};

// Device arrays describing a CSR matrix prepared for the merge-path kernels.
// Offsets are int32 when n_rows + nnz < 2^31, else int64 (`wide`).
struct MpMatrix {
  int64_t n_rows = 0, n_cols = 0, nnz = 0;
  bool wide = false;
  const void* row_end = nullptr;   // n_rows offsets: row_ptr[1..n_rows]
  const int32_t* col = nullptr;    // nnz column indices
  const void* val = nullptr;       // nnz values (double or float)
  const void* tile_row = nullptr;  // num_tiles + 1 merge coordinates (row)
  const void* tile_nz = nullptr;   // num_tiles + 1 merge coordinates (nonzero)
  void* carry_row = nullptr;       // num_tiles scratch
  void* carry_val = nullptr;       // num_tiles scratch
  int64_t num_tiles = 0;
  MpShape shape;
};

// Fills tile_row / tile_nz (device) for the given shape.
bool mp_partition(const MpMatrix& m, cudaStream_t s);
// y = A x; x and y are device pointers of the form's value type.  When
// `events` is non-null, events[0..2] are recorded before the tile kernel,
// between the tile and fix-up kernels, and after the fix-up kernel.
bool mp_spmv(const MpMatrix& m, MpForm form, const void* x, void* y, cudaStream_t s,
             cudaEvent_t* events = nullptr);
// Dynamic shared memory bytes of one tile for a shape and value size.
size_t mp_smem_bytes(const MpShape& sh, size_t value_bytes);
// Kernel launches per mp_spmv call.
constexpr int kMpLaunchesPerCall = 2;

// Pipelined merge-path kernels (mp2_kernels.cu): FP64 values, int32 offsets.
// Default poll limit of the pipelined kernel's waits (seconds of wall time).
constexpr int kMp2DefaultWaitPolls = 1 << 24;
struct Mp2Matrix {
  int64_t n_rows = 0, n_cols = 0, nnz = 0;
  const int* row_end = nullptr;  // padded by >= 4 elements
  const int32_t* col = nullptr;  // padded by >= 4 elements
  const double* val = nullptr;   // padded by >= 4 elements
  const int* tile_row = nullptr;
  const int* tile_nz = nullptr;
  int* carry_row = nullptr;
  double* carry_val = nullptr;
  int* flags = nullptr;  // device [2]: DF32 range flag, pipeline timeout flag
  int64_t num_tiles = 0;
  MpShape shape;
  int stages = 2;
  int sms = 0;
  int wait_polls = kMp2DefaultWaitPolls;  // polls of a pipeline wait before a timeout is reported
};
// y = A x.  df32: double-float arithmetic on the FP32 pipe with an F64 guard
// launch for out-of-range x.  Events as for mp_spmv.
bool mp2_spmv(const Mp2Matrix& m, bool df32, const double* x, double* y, cudaStream_t s,
              cudaEvent_t* events = nullptr);
// Shared memory of a supported (threads, items, stages) combination, 0 if unsupported.
size_t mp2_smem(int tpb, int ipt, int stages);
// Kernel launches per mp2_spmv call.
inline int mp2_launches(bool df32) { return df32 ? 3 : 2; }

}  // namespace vnec
