// Merge-path CSR SpMV for sm_103a — the GPU counterpart of VNEC-L
// (src/operation/src/spmv_vnec_L_for_mxv.c:124-165) and of its partitioner
// MergePathDivide (src/operation/src/spmv_vnec_common.c:3-33).
//
// Work decomposition.  The merge of the row-end list (row_ptr[1..n]) and the
// nonzero counting list (0..nnz-1) has n_rows + nnz items.  It is cut into
// tiles of TPB*IPT items, one CTA per tile; the tile boundaries are found once
// per matrix (plan time) by mp_partition_kernel.  Inside a tile:
//   1. stage: the tile's values, the gathered x[col] and its row ends are
//      copied to shared memory with coalesced loads (values and columns are
//      read once, so they are loaded with the streaming cache hint; x is
//      gathered through the read-only path so it stays resident in L2);
//   2. consume: each thread runs the merge path over IPT consecutive items of
//      the tile — one FMA per nonzero, a row result at each row end — exactly
//      the per-thread loop of the reference's OpenMP threads, at warp lane
//      granularity;
//   3. carry: a thread whose segment starts inside a row adds the partial sums
//      of the preceding threads that stopped in the same row, found by a
//      segmented scan over the threads (warp shuffles plus one scan over the
//      warp totals, log steps), then writes that row; the tile's own
//      carry-out (partial of its last row) goes to a per-tile scratch slot;
//   4. fix-up (second, tiny launch): rows spanning tiles receive the ordered
//      sum of the carries of the tiles that stopped inside them — the
//      counterpart of the reference's serial carry loop (:159-164).
// The FP64 form performs exactly one FP64 FMA per nonzero plus at most
// log2(32) + log2(warps) adds per thread for the carries: on GB300 the FP64
// pipe (about 0.6 T FMA/s) is close to the HBM rate for SpMV, so no other
// FP64 work is done in the loop.  (A walk back over the preceding threads'
// partials costs one add per thread a row spans, quadratic in the rows that
// cover a whole tile: on R-MAT 2^24 it kept the FP64 pipe 70% busy.)

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "common.h"
#include "vnec_gb300.h"

namespace vnec {
namespace {

template <typename T> __device__ __forceinline__ T ld_stream(const T* p) { return __ldcs(p); }
__device__ __forceinline__ long long ld_stream(const long long* p) { return __ldcs(p); }

template <typename V> __device__ __forceinline__ V fma_v(V a, V b, V c);
template <> __device__ __forceinline__ double fma_v<double>(double a, double b, double c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fma_v<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Diagonal search of one merge-path boundary (MergePathDivide semantics:
// move right while row_end[pivot] <= diag - pivot - 1).
template <typename Off>
__device__ __forceinline__ Off merge_search(const Off* row_end, Off diag, Off n_rows, Off nnz) {
  Off lo = diag - nnz > 0 ? diag - nnz : 0;
  Off hi = diag < n_rows ? diag : n_rows;
  while (lo < hi) {
    Off p = (lo + hi) >> 1;
    if (row_end[p] <= diag - p - 1)
      lo = p + 1;
    else
      hi = p;
  }
  return lo;
}

template <typename Off>
__global__ void mp_partition_kernel(const Off* __restrict__ row_end, Off n_rows, Off nnz, long long ipc,
                                    long long num_tiles, Off* __restrict__ tile_row, Off* __restrict__ tile_nz) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t > num_tiles) return;
  Off total = n_rows + nnz;
  long long d64 = t * ipc;
  Off diag = d64 < (long long)total ? (Off)d64 : total;
  Off r = merge_search<Off>(row_end, diag, n_rows, nnz);
  tile_row[t] = r;
  tile_nz[t] = diag - r;
}

// One CTA per tile.  Shared memory: s_val[IPC], s_x[IPC] (V), s_end[IPC]
// (int, row ends relative to the tile's first nonzero), per-warp carry
// totals, open flags and carry-ins (TPB / 32 each).
template <typename V, typename Off, int TPB, int IPT>
__global__ void __launch_bounds__(TPB)
mp_spmv_kernel(const Off* __restrict__ row_end, const int32_t* __restrict__ col, const V* __restrict__ val,
               const V* __restrict__ x, V* __restrict__ y, const Off* __restrict__ tile_row,
               const Off* __restrict__ tile_nz, Off* __restrict__ carry_row, V* __restrict__ carry_val) {
  constexpr int IPC = TPB * IPT;
  constexpr int kW = TPB / 32;
  constexpr unsigned kFull = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* s_val = reinterpret_cast<V*>(smem_raw);
  V* s_x = s_val + IPC;
  V* w_run = s_x + IPC;  // [kW] warp totals of the open run
  V* w_cin = w_run + kW;  // [kW] carry into each warp
  int* s_end = reinterpret_cast<int*>(w_cin + kW);
  int* w_open = s_end + IPC;  // [kW]

  const int tile = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const Off x0 = tile_row[tile], y0 = tile_nz[tile];
  const Off x1 = tile_row[tile + 1], y1 = tile_nz[tile + 1];
  const int nrows = (int)(x1 - x0);
  const int nnz = (int)(y1 - y0);

  // 1. stage values, gathered x and row ends.
  {
    const int32_t* c_t = col + y0;
    const V* v_t = val + y0;
#pragma unroll 4
    for (int i = tid; i < nnz; i += TPB) {
      int c = ld_stream(c_t + i);
      s_val[i] = ld_stream(v_t + i);
      s_x[i] = __ldg(x + c);
    }
    const Off* e_t = row_end + x0;
    for (int i = tid; i < nrows; i += TPB) s_end[i] = (int)(ld_stream(e_t + i) - y0);
  }
  __syncthreads();

  // 2. per-thread merge path over IPT items.
  const int total = nrows + nnz;
  const int d = min(tid * IPT, total);
  int rr = merge_search<int>(s_end, d, nrows, nnz);
  int kk = d - rr;
  const int dend = min(d + IPT, total);
  V acc = V(0);
  V first_val = V(0);
  int first = -1;
#pragma unroll
  for (int it = 0; it < IPT; ++it) {
    if (d + it < dend) {
      if (rr < nrows && s_end[rr] <= kk) {
        if (first < 0) {
          first = rr;
          first_val = acc;
        } else {
          y[x0 + rr] = acc;
        }
        acc = V(0);
        ++rr;
      } else {
        acc = fma_v<V>(s_val[kk], s_x[kk], acc);
        ++kk;
      }
    }
  }

  // 3. in-tile carries.  A thread that emitted a row starts a new run with its
  // tail partial; a thread that did not is still inside the row of the
  // threads before it.  A segmented inclusive scan over the threads (warp
  // shuffles, then one scan over the warp totals) gives every thread the sum
  // of the open run before it in log steps, however many threads a row spans.
  V run = acc;
  int open = first < 0;
  for (int dist = 1; dist < 32; dist <<= 1) {
    if (!__ballot_sync(kFull, open && lane >= dist)) break;
    const V up = __shfl_up_sync(kFull, run, dist);
    const int up_open = __shfl_up_sync(kFull, open, dist);
    if (open && lane >= dist) {
      run += up;
      open = up_open;
    }
  }
  if (lane == 31) {
    w_run[warp] = run;
    w_open[warp] = open;
  }
  __syncthreads();
  if (warp == 0) {
    V cv = lane < kW ? w_run[lane] : V(0);
    int co = lane < kW ? w_open[lane] : 0;
    for (int dist = 1; dist < kW; dist <<= 1) {
      const V up = __shfl_up_sync(kFull, cv, dist);
      const int up_open = __shfl_up_sync(kFull, co, dist);
      if (co && lane >= dist) {
        cv += up;
        co = up_open;
      }
    }
    const V ex = __shfl_up_sync(kFull, cv, 1);
    if (lane < kW) w_cin[lane] = lane == 0 ? V(0) : ex;
  }
  __syncthreads();
  const V prev = __shfl_up_sync(kFull, run, 1);
  const int prev_open = __shfl_up_sync(kFull, open, 1);
  if (first >= 0) {
    V cin;
    if (lane == 0)
      cin = w_cin[warp];
    else
      cin = prev_open ? prev + w_cin[warp] : prev;
    y[x0 + first] = first_val + cin;
  }
  if (tid == TPB - 1) {
    carry_row[tile] = x1;
    carry_val[tile] = open ? run + w_cin[warp] : run;
  }
}

// 4. cross-tile carries: the first tile of each run of tiles that stopped in
// the same row adds the run's carries, in tile order, to that row.
template <typename V, typename Off>
__global__ void mp_fixup_kernel(const Off* __restrict__ carry_row, const V* __restrict__ carry_val,
                                long long num_tiles, Off n_rows, V* __restrict__ y) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= num_tiles) return;
  Off r = carry_row[t];
  if (r >= n_rows) return;
  if (t > 0 && carry_row[t - 1] == r) return;
  V s = V(0);
  for (long long u = t; u < num_tiles && carry_row[u] == r; ++u) s += carry_val[u];
  y[r] += s;
}

template <typename V, typename Off, int TPB, int IPT>
bool launch_mp(const MpMatrix& m, const void* x, void* y, cudaStream_t s, cudaEvent_t* ev) {
  auto kern = mp_spmv_kernel<V, Off, TPB, IPT>;
  MpShape sh;
  sh.tpb = TPB;
  sh.ipt = IPT;
  size_t smem = mp_smem_bytes(sh, sizeof(V));
  static std::atomic<unsigned long long> configured{0};  // per instantiation, per device
  if (!once_per_device(configured, [&] {
        return VNEC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      }))
    return false;
  if (m.num_tiles > 0x7fffffffLL) {
    set_error("merge-path: tile count exceeds the grid limit");
    return false;
  }
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[0], s))) return false;
  kern<<<(unsigned)m.num_tiles, TPB, smem, s>>>(
      static_cast<const Off*>(m.row_end), m.col, static_cast<const V*>(m.val), static_cast<const V*>(x),
      static_cast<V*>(y), static_cast<const Off*>(m.tile_row), static_cast<const Off*>(m.tile_nz),
      static_cast<Off*>(m.carry_row), static_cast<V*>(m.carry_val));
  if (!VNEC_CUDA(cudaGetLastError())) return false;
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[1], s))) return false;
  const int fb = 256;
  long long fg = (m.num_tiles + fb - 1) / fb;
  mp_fixup_kernel<V, Off><<<(unsigned)fg, fb, 0, s>>>(static_cast<const Off*>(m.carry_row),
                                                      static_cast<const V*>(m.carry_val), m.num_tiles,
                                                      (Off)m.n_rows, static_cast<V*>(y));
  if (!VNEC_CUDA(cudaGetLastError())) return false;
  if (ev && !VNEC_CUDA(cudaEventRecord(ev[2], s))) return false;
  return true;
}

template <typename V, typename Off>
bool dispatch_shape(const MpMatrix& m, const void* x, void* y, cudaStream_t s, cudaEvent_t* ev) {
  const int tpb = m.shape.tpb, ipt = m.shape.ipt;
#define VNEC_MP_CASE(T, I) \
  if (tpb == T && ipt == I) return launch_mp<V, Off, T, I>(m, x, y, s, ev);
  VNEC_MP_CASE(128, 4)
  VNEC_MP_CASE(128, 7)
  VNEC_MP_CASE(128, 10)
  VNEC_MP_CASE(256, 4)
  VNEC_MP_CASE(256, 7)
  VNEC_MP_CASE(256, 10)
#undef VNEC_MP_CASE
  set_error("merge-path: unsupported tile shape");
  return false;
}

}  // namespace

size_t mp_smem_bytes(const MpShape& sh, size_t value_bytes) {
  const size_t ipc = (size_t)sh.tpb * sh.ipt, warps = (size_t)sh.tpb / 32;
  return 2 * ipc * value_bytes + 2 * warps * value_bytes + ipc * sizeof(int) + warps * sizeof(int);
}

bool mp_partition(const MpMatrix& m, cudaStream_t s) {
  long long ipc = m.shape.items_per_tile();
  const int b = 256;
  long long g = (m.num_tiles + 1 + b - 1) / b;
  if (m.wide) {
    mp_partition_kernel<long long><<<(unsigned)g, b, 0, s>>>(
        static_cast<const long long*>(m.row_end), (long long)m.n_rows, (long long)m.nnz, ipc, m.num_tiles,
        static_cast<long long*>(const_cast<void*>(m.tile_row)), static_cast<long long*>(const_cast<void*>(m.tile_nz)));
  } else {
    mp_partition_kernel<int><<<(unsigned)g, b, 0, s>>>(
        static_cast<const int*>(m.row_end), (int)m.n_rows, (int)m.nnz, ipc, m.num_tiles,
        static_cast<int*>(const_cast<void*>(m.tile_row)), static_cast<int*>(const_cast<void*>(m.tile_nz)));
  }
  return VNEC_CUDA(cudaGetLastError());
}

bool mp_spmv(const MpMatrix& m, MpForm form, const void* x, void* y, cudaStream_t s, cudaEvent_t* ev) {
  if (m.n_rows == 0) return true;
  switch (form) {
    case MpForm::kF64:
      return m.wide ? dispatch_shape<double, long long>(m, x, y, s, ev) : dispatch_shape<double, int>(m, x, y, s, ev);
    case MpForm::kF32:
      return m.wide ? dispatch_shape<float, long long>(m, x, y, s, ev) : dispatch_shape<float, int>(m, x, y, s, ev);
  }
  set_error("merge-path: unknown value form");
  return false;
}

}  // namespace vnec

// ---------------------------------------------------------------------------
// Allocation-free entry point: SpB_mxv_csr_noalloc_ext.
//
// Some callers cannot let a library allocate device memory on their behalf:
// hosts whose device memory is handed out entirely by their own pool
// allocator (the library could not obtain more), and latency-critical loops
// in which a cudaMalloc/cudaFree and the device synchronisation it implies
// are not acceptable.  For them this entry point runs the FP64 merge-path
// kernel (256 threads x 7 merge items per tile) on CSR arrays the caller
// already holds in device memory, and keeps its scratch — the merge
// coordinates of each tile and each tile's carry-out — in the fixed array
// below, which every device that loads this library holds until the process
// exits.
// ---------------------------------------------------------------------------
namespace vnec {
namespace {

constexpr int kNaTpb = 256, kNaIpt = 7;
// Scratch capacity: 2^18 tiles of 1,792 merge items, i.e. n_rows + nnz <=
// 469,762,048; 5,242,888 bytes.
constexpr long long kNaMaxTiles = 1LL << 18;
constexpr long long kNaMaxItems = kNaMaxTiles * kNaTpb * kNaIpt;  // 469,762,048
constexpr size_t kNaTileRowOff = 0;
constexpr size_t kNaTileNzOff = kNaTileRowOff + 4 * (kNaMaxTiles + 1);
constexpr size_t kNaCarryRowOff = kNaTileNzOff + 4 * (kNaMaxTiles + 1);
constexpr size_t kNaCarryValOff = kNaCarryRowOff + 4 * kNaMaxTiles;
constexpr size_t kNaBytes = kNaCarryValOff + 8 * kNaMaxTiles;
static_assert(kNaCarryValOff % 8 == 0, "carry values must be 8-byte aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

// Identity of the calling thread's current CUDA context: its driver-assigned
// id, unique for the life of the process (cuCtxGetId), reached through the
// runtime's driver entry points so the library needs no link against the
// driver library.  False when the driver lacks these calls or no context is
// current yet.
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);
bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  if (!get_current || !get_id) return false;
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || !ctx) return false;
  return get_id(ctx, id) == 0;
}

// Device address of g_noalloc_scratch in the current context.  In host code
// the symbol is only a host-side stand-in, so the address is looked up with
// cudaGetSymbolAddress the first time a context calls and cached under that
// context's id: a device reset or a caller's own driver context gets a new id
// and therefore its own lookup, never a stale address.  Where the context id
// cannot be read, the address is looked up on every call.
bool noalloc_scratch(unsigned char** out) {
  struct Entry {
    unsigned long long ctx;
    unsigned char* addr;
  };
  static std::mutex mu;
  static Entry cache[64] = {};
  static int next = 0;
  unsigned long long id = 0;
  bool have_id = current_context_id(&id);
  if (have_id) {
    std::lock_guard<std::mutex> g(mu);
    for (const Entry& e : cache)
      if (e.addr && e.ctx == id) {
        *out = e.addr;
        return true;
      }
  }
  void* p = nullptr;
  if (!VNEC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch))) return false;
  if (!p) {
    set_error("SpB_mxv_csr_noalloc_ext: no device address for the fixed scratch array");
    return false;
  }
  if (!have_id) have_id = current_context_id(&id);  // the lookup made the primary context current
  if (have_id) {
    std::lock_guard<std::mutex> g(mu);
    cache[next] = Entry{id, static_cast<unsigned char*>(p)};
    next = (next + 1) % 64;
  }
  *out = static_cast<unsigned char*>(p);
  return true;
}

}  // namespace
}  // namespace vnec

extern "C" SpB_Info SpB_mxv_csr_noalloc_ext(int64_t n_rows, int64_t n_cols, int64_t nnz, const int32_t* d_row_ptr,
                                            const int32_t* d_col, const double* d_val, const double* d_x,
                                            double* d_y, void* stream) {
  using namespace vnec;
  clear_error();
  if (n_rows < 0 || n_cols < 0 || nnz < 0) {
    set_error("SpB_mxv_csr_noalloc_ext: negative size");
    return SpB_FAILURE;
  }
  const long long ipc = (long long)kNaTpb * kNaIpt;
  // Each size is checked on its own before the sum is formed, so huge
  // arguments cannot overflow it.
  if (n_rows > kNaMaxItems || nnz > kNaMaxItems || n_rows + nnz > kNaMaxItems) {
    set_error("SpB_mxv_csr_noalloc_ext: n_rows + nnz exceeds the allocation-free limit of 469,762,048 "
              "(its fixed scratch holds 262,144 tiles); use a plan (SpB_VNEC_plan_ext) instead");
    return SpB_FAILURE;
  }
  if (n_cols > INT32_MAX) {
    set_error("SpB_mxv_csr_noalloc_ext: n_cols exceeds the int32 column range");
    return SpB_FAILURE;
  }
  const long long tiles = (n_rows + nnz + ipc - 1) / ipc;
  if (n_rows == 0) return SpB_SUCCESS;
  if (!d_row_ptr || !d_y || (nnz > 0 && (!d_col || !d_val || !d_x))) {
    set_error("SpB_mxv_csr_noalloc_ext: NULL device array");
    return SpB_FAILURE;
  }
  unsigned char* scratch = nullptr;
  if (!noalloc_scratch(&scratch)) return SpB_FAILURE;
  MpMatrix m;
  m.n_rows = n_rows;
  m.n_cols = n_cols;
  m.nnz = nnz;
  m.wide = false;
  m.row_end = d_row_ptr + 1;
  m.col = d_col;
  m.val = d_val;
  m.tile_row = scratch + kNaTileRowOff;
  m.tile_nz = scratch + kNaTileNzOff;
  m.carry_row = scratch + kNaCarryRowOff;
  m.carry_val = scratch + kNaCarryValOff;
  m.num_tiles = tiles;
  m.shape.tpb = kNaTpb;
  m.shape.ipt = kNaIpt;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Every scratch word a launch reads is written earlier in the same call
  // (coordinates by the partition kernel, carries by the tile kernel), so
  // nothing needs clearing between calls.
  if (!mp_partition(m, s)) return SpB_FAILURE;
  return mp_spmv(m, MpForm::kF64, d_x, d_y, s) ? SpB_SUCCESS : SpB_FAILURE;
}
