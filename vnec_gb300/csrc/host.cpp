// Host-side plan machinery: CSR ingestion and validation, the plan registry,
// the merge-path plan and the IRD selector restated from the reference.

#include "host.h"

#include <omp.h>

#include <algorithm>
#include <cstring>
#include <unordered_map>

namespace vnec {

// ---------------------------------------------------------------------------
// Errors and device buffers
// ---------------------------------------------------------------------------
namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
const char* last_error() { return g_last_error.c_str(); }

bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

bool DeviceBuffer::alloc(size_t n) {
  release();
  if (n == 0) n = 16;
  if (!VNEC_CUDA(cudaMalloc(&ptr, n))) {
    ptr = nullptr;
    return false;
  }
  bytes = n;
  return true;
}

void DeviceBuffer::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

// ---------------------------------------------------------------------------
// CSR ingestion
// ---------------------------------------------------------------------------
bool view_from_matrix(const SpB_Matrix A, CsrView* v) {
  if (!A) {
    set_error("matrix is NULL");
    return false;
  }
  auto* m = reinterpret_cast<const SpB_Matrix_CSC_or_CSR*>(A);
  if (A->format_type != SpB_CSR) {
    set_error("matrix is not in CSR format (the VNEC path reads CSR, SpB_Global_Option_set_ext)");
    return false;
  }
  if (A->element_type != SpB_FP64 && A->element_type != SpB_FP32) {
    set_error("matrix element type must be SpB_FP64 or SpB_FP32");
    return false;
  }
  if (m->ptr_len != A->row + 1) {
    set_error("CSR ptr_len != rows + 1");
    return false;
  }
  v->type = A->element_type;
  v->n_rows = (int64_t)A->row;
  v->n_cols = (int64_t)A->col;
  v->nnz = (int64_t)m->nnz;
  v->ptr64 = m->ptr;
  v->idx64 = m->indices;
  v->ptr = nullptr;
  v->idx = nullptr;
  v->val = m->val;
  if (v->n_rows > 0 && !v->ptr64) {
    set_error("CSR ptr is NULL");
    return false;
  }
  if (v->nnz > 0 && (!v->idx64 || !v->val)) {
    set_error("CSR indices or values are NULL");
    return false;
  }
  return true;
}

bool view_from_arrays(SpB_Type type, int64_t n_rows, int64_t n_cols, const int64_t* row_ptr, const int32_t* col,
                      const void* val, CsrView* v) {
  if (type != SpB_FP64 && type != SpB_FP32) {
    set_error("value type must be SpB_FP64 or SpB_FP32");
    return false;
  }
  if (n_rows < 0 || n_cols < 0 || !row_ptr) {
    set_error("invalid CSR shape or NULL row_ptr");
    return false;
  }
  v->type = type;
  v->n_rows = n_rows;
  v->n_cols = n_cols;
  v->nnz = row_ptr[n_rows];
  v->ptr = row_ptr;
  v->idx = col;
  v->ptr64 = nullptr;
  v->idx64 = nullptr;
  v->val = val;
  if (v->nnz > 0 && (!col || !val)) {
    set_error("CSR col or val is NULL");
    return false;
  }
  return true;
}

bool validate_csr(const CsrView& v, bool need_sorted) {
  if (v.n_cols > 0x7fffffffLL) {
    set_error("n_cols must fit in int32");
    return false;
  }
  if (v.row_begin(0) != 0 || v.row_begin(v.n_rows) != v.nnz || v.nnz < 0) {
    set_error("CSR offsets must start at 0 and end at nnz");
    return false;
  }
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t r = 0; r < v.n_rows; ++r) {
    int64_t b = v.row_begin(r), e = v.row_begin(r + 1);
    if (e < b || e > v.nnz) {
      bad |= 1;
      continue;
    }
    int64_t prev = -1;
    for (int64_t p = b; p < e; ++p) {
      int64_t c = v.col_at(p);
      if (c < 0 || c >= v.n_cols) bad |= 2;
      if (need_sorted && c <= prev) bad |= 4;
      prev = c;
    }
  }
  if (bad & 1) {
    set_error("CSR offsets are not monotone");
    return false;
  }
  if (bad & 2) {
    set_error("CSR column index out of range");
    return false;
  }
  if (bad & 4) {
    set_error("CSR columns are not strictly increasing within a row");
    return false;
  }
  return true;
}

void convert_row_end(const CsrView& v, bool wide, void* out) {
  if (wide) {
    auto* o = static_cast<int64_t*>(out);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < v.n_rows; ++r) o[r] = v.row_begin(r + 1);
  } else {
    auto* o = static_cast<int32_t*>(out);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < v.n_rows; ++r) o[r] = (int32_t)v.row_begin(r + 1);
  }
}

void convert_cols(const CsrView& v, int32_t* out) {
  if (v.idx) {
    std::memcpy(out, v.idx, sizeof(int32_t) * (size_t)v.nnz);
    return;
  }
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < v.nnz; ++p) out[p] = (int32_t)v.idx64[p];
}

bool transpose_csr(const CsrView& v, CsrTranspose* t) {
  if (v.n_rows >= ((int64_t)1 << 31)) {
    set_error("transpose: more than 2^31 rows");
    return false;
  }
  const size_t vb = v.value_bytes();
  t->row_ptr.assign((size_t)v.n_cols + 1, 0);
  t->col.resize((size_t)std::max<int64_t>(v.nnz, 1));
  t->val.resize((size_t)std::max<int64_t>(v.nnz, 1) * vb);
  std::vector<int64_t> cursor((size_t)v.n_cols + 1, 0);
  // Column counts, then positions reserved atomically; each transposed row is
  // then sorted by original row so the result does not depend on thread timing.
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < v.nnz; ++p) __atomic_fetch_add(&cursor[(size_t)v.col_at(p) + 1], 1, __ATOMIC_RELAXED);
  for (int64_t c = 0; c < v.n_cols; ++c) cursor[(size_t)c + 1] += cursor[(size_t)c];
  std::copy(cursor.begin(), cursor.end(), t->row_ptr.begin());
  const unsigned char* src = static_cast<const unsigned char*>(v.val);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t r = 0; r < v.n_rows; ++r)
    for (int64_t p = v.row_begin(r); p < v.row_begin(r + 1); ++p) {
      const int64_t q = __atomic_fetch_add(&cursor[(size_t)v.col_at(p)], 1, __ATOMIC_RELAXED);
      t->col[(size_t)q] = (int32_t)r;
      std::memcpy(&t->val[(size_t)q * vb], src + (size_t)p * vb, vb);
    }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t c = 0; c < v.n_cols; ++c) {
    const int64_t b = t->row_ptr[(size_t)c], e = t->row_ptr[(size_t)c + 1];
    if (e - b < 2) continue;
    std::vector<std::pair<int32_t, int64_t>> order((size_t)(e - b));
    for (int64_t q = b; q < e; ++q) order[(size_t)(q - b)] = {t->col[(size_t)q], q};
    std::sort(order.begin(), order.end());
    std::vector<unsigned char> vals((size_t)(e - b) * vb);
    for (int64_t i = 0; i < e - b; ++i) std::memcpy(&vals[(size_t)i * vb], &t->val[(size_t)order[(size_t)i].second * vb], vb);
    for (int64_t i = 0; i < e - b; ++i) t->col[(size_t)(b + i)] = order[(size_t)i].first;
    std::memcpy(&t->val[(size_t)b * vb], vals.data(), vals.size());
  }
  t->view.type = v.type;
  t->view.n_rows = v.n_cols;
  t->view.n_cols = v.n_rows;
  t->view.nnz = v.nnz;
  t->view.ptr = t->row_ptr.data();
  t->view.idx = t->col.data();
  t->view.ptr64 = nullptr;
  t->view.idx64 = nullptr;
  t->view.val = t->val.data();
  return true;
}

// ---------------------------------------------------------------------------
// Plans and registry
// ---------------------------------------------------------------------------
Plan::~Plan() {
  if (own_stream) cudaStreamDestroy(own_stream);
  for (cudaEvent_t& e : events)
    if (e) cudaEventDestroy(e);
}

bool Plan::ensure_events() {
  for (cudaEvent_t& e : events)
    if (!e && !VNEC_CUDA(cudaEventCreate(&e))) return false;
  return true;
}

bool Plan::run_epilogue(const void* d_x, void* d_y, const SlicedEpilogue& e, cudaStream_t s) {
  SlicedEpilogue ee = e;
  const size_t vb = type == SpB_FP64 ? 8 : 4;
  const size_t ny = (size_t)n_rows * rhs;
  if (e.z && e.z == d_y && e.beta != 0.0 && ny > 0) {
    if (epi_scratch.bytes < vb * ny && !(epi_scratch.release(), epi_scratch.alloc(vb * ny))) return false;
    if (!VNEC_CUDA(cudaMemcpyAsync(epi_scratch.ptr, d_y, vb * ny, cudaMemcpyDeviceToDevice, s))) return false;
    ee.z = epi_scratch.ptr;
  }
  if (!run(d_x, d_y, s)) return false;
  return apply_epilogue(d_y, (long long)ny, type == SpB_FP64, ee, s);
}

bool Plan::run_host(const void* h_x, void* h_y) {
  std::lock_guard<std::mutex> g(host_mu);
  if (!drain_pipe()) return false;
  const size_t vb = type == SpB_FP64 ? 8 : 4;
  if (!own_stream && !VNEC_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking))) return false;
  const size_t nx = (size_t)n_cols * rhs, ny = (size_t)n_rows * rhs;
  if (!dx.ptr && !dx.alloc(vb * std::max<size_t>(nx, 1))) return false;
  if (!dy.ptr && !dy.alloc(vb * std::max<size_t>(ny, 1))) return false;
  if (nx > 0 && !VNEC_CUDA(cudaMemcpyAsync(dx.ptr, h_x, vb * nx, cudaMemcpyHostToDevice, own_stream))) return false;
  if (!run(dx.ptr, dy.ptr, own_stream)) return false;
  if (ny > 0 && !VNEC_CUDA(cudaMemcpyAsync(h_y, dy.ptr, vb * ny, cudaMemcpyDeviceToHost, own_stream))) return false;
  return device_status(own_stream);
}

Plan::HostPipe::~HostPipe() {
  for (cudaStream_t q : {in, comp, out})
    if (q) cudaStreamSynchronize(q);
  for (int i = 0; i < 2; ++i)
    for (cudaEvent_t e : {x_ready[i], comp_done[i], out_done[i]})
      if (e) cudaEventDestroy(e);
  for (cudaStream_t q : {in, comp, out})
    if (q) cudaStreamDestroy(q);
}

bool Plan::HostPipe::init(size_t xb, size_t yb) {
  for (cudaStream_t* q : {&in, &comp, &out})
    if (!VNEC_CUDA(cudaStreamCreateWithFlags(q, cudaStreamNonBlocking))) return false;
  for (int i = 0; i < 2; ++i) {
    for (cudaEvent_t* e : {&x_ready[i], &comp_done[i], &out_done[i]})
      if (!VNEC_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming))) return false;
    if (!x[i].alloc(xb) || !y[i].alloc(yb)) return false;
  }
  return true;
}

bool Plan::run_host_async(const void* h_x, void* h_y) {
  std::lock_guard<std::mutex> g(host_mu);
  const size_t vb = type == SpB_FP64 ? 8 : 4;
  const size_t nx = (size_t)n_cols * rhs, ny = (size_t)n_rows * rhs;
  if (!pipe) {
    auto p = std::make_unique<HostPipe>();
    if (!p->init(vb * std::max<size_t>(nx, 1), vb * std::max<size_t>(ny, 1))) return false;
    pipe = std::move(p);
  }
  HostPipe& q = *pipe;
  const int s = (int)(q.calls & 1);
  // Slot s was last used two calls ago: its x is free once that SpMV is done,
  // its y once that copy-out is done.
  if (q.used[s] && !VNEC_CUDA(cudaStreamWaitEvent(q.in, q.comp_done[s], 0))) return false;
  if (nx > 0 && !VNEC_CUDA(cudaMemcpyAsync(q.x[s].ptr, h_x, vb * nx, cudaMemcpyHostToDevice, q.in))) return false;
  if (!VNEC_CUDA(cudaEventRecord(q.x_ready[s], q.in)) || !VNEC_CUDA(cudaStreamWaitEvent(q.comp, q.x_ready[s], 0)))
    return false;
  if (q.used[s] && !VNEC_CUDA(cudaStreamWaitEvent(q.comp, q.out_done[s], 0))) return false;
  if (!run_slot(s, q.x[s].ptr, q.y[s].ptr, q.comp) || !VNEC_CUDA(cudaEventRecord(q.comp_done[s], q.comp)) ||
      !VNEC_CUDA(cudaStreamWaitEvent(q.out, q.comp_done[s], 0)))
    return false;
  if (ny > 0 && !VNEC_CUDA(cudaMemcpyAsync(h_y, q.y[s].ptr, vb * ny, cudaMemcpyDeviceToHost, q.out))) return false;
  if (!VNEC_CUDA(cudaEventRecord(q.out_done[s], q.out))) return false;
  q.used[s] = true;
  ++q.calls;
  return true;
}

bool Plan::host_wait() {
  std::lock_guard<std::mutex> g(host_mu);
  if (!pipe) return true;
  if (!VNEC_CUDA(cudaStreamSynchronize(pipe->out)) || !VNEC_CUDA(cudaStreamSynchronize(pipe->in))) return false;
  return device_status(pipe->comp);
}

namespace {
std::mutex g_reg_mu;
std::unordered_map<const void*, std::unique_ptr<Plan>>& registry() {
  static auto* r = new std::unordered_map<const void*, std::unique_ptr<Plan>>();
  return *r;
}
}  // namespace

void register_plan(const void* handle, std::unique_ptr<Plan> plan) {
  std::lock_guard<std::mutex> g(g_reg_mu);
  registry()[handle] = std::move(plan);
}

Plan* find_plan(const void* handle) {
  std::lock_guard<std::mutex> g(g_reg_mu);
  auto it = registry().find(handle);
  return it == registry().end() ? nullptr : it->second.get();
}

std::unique_ptr<Plan> take_plan(const void* handle) {
  std::lock_guard<std::mutex> g(g_reg_mu);
  auto it = registry().find(handle);
  if (it == registry().end()) return nullptr;
  std::unique_ptr<Plan> p = std::move(it->second);
  registry().erase(it);
  // Pipelined host calls still in flight read the plan's device arrays.
  if (p && p->pipe) {
    for (cudaStream_t q : {p->pipe->in, p->pipe->comp, p->pipe->out}) cudaStreamSynchronize(q);
  }
  return p;
}

// ---------------------------------------------------------------------------
// Merge-path plan (VNEC-L counterpart)
// ---------------------------------------------------------------------------
namespace {

struct MergePathPlan final : Plan {
  MpMatrix m;     // unpipelined kernel (any value type / offset width)
  Mp2Matrix m2;   // pipelined kernel (FP64, int32 offsets)
  bool pipelined = false;
  bool df32 = false;
  DeviceBuffer row_end, col, val, tile_row, tile_nz, carry_row, carry_val, flags;
  MergePathPlan() : Plan(PlanKind::kMergePath) {}
  bool run(const void* d_x, void* d_y, cudaStream_t s) override {
    if (profiling && !ensure_events()) return false;
    cudaEvent_t* ev = profiling ? events : nullptr;
    if (pipelined)
      return mp2_spmv(m2, df32, static_cast<const double*>(d_x), static_cast<double*>(d_y), s, ev);
    return mp_spmv(m, type == SpB_FP64 ? MpForm::kF64 : MpForm::kF32, d_x, d_y, s, ev);
  }
  int kernel_ms(float* ms, int cap) const override {
    if (!profiling || !events[0] || cap < 2) return 0;
    if (cudaEventSynchronize(events[2]) != cudaSuccess) return 0;
    cudaEventElapsedTime(&ms[0], events[0], events[1]);
    cudaEventElapsedTime(&ms[1], events[1], events[2]);
    return 2;
  }
  int launches_per_call() const override {
    if (n_rows == 0) return 0;
    return pipelined ? mp2_launches(df32) : kMpLaunchesPerCall;
  }
  int64_t device_bytes() const override {
    return (int64_t)(row_end.bytes + col.bytes + val.bytes + tile_row.bytes + tile_nz.bytes + carry_row.bytes +
                     carry_val.bytes + flags.bytes + dx.bytes + dy.bytes);
  }
  int64_t algorithmic_bytes() const override {
    const int64_t vb = type == SpB_FP64 ? 8 : 4, ob = m.wide ? 8 : 4;
    return nnz * (vb + 4) + (n_rows + 1) * ob + n_cols * vb + n_rows * vb;
  }
  void describe(SpB_VNEC_info_ext* info) const override {
    info->kernel = SpB_VNEC_KERNEL_L;
    info->threads_per_block = m.shape.tpb;
    info->items_per_thread = m.shape.ipt;
    info->num_tiles = m.num_tiles;
    info->pipeline_stages = pipelined ? m2.stages : 0;
    info->arithmetic = type == SpB_FP64 ? (df32 ? SpB_VNEC_ARITH_DF32 : SpB_VNEC_ARITH_FP64) : 0;
  }
  void set_wait_polls(int64_t polls) override {
    m2.wait_polls = polls < 0 ? kMp2DefaultWaitPolls : (int)std::min<int64_t>(polls, INT32_MAX);
  }
  bool device_status(cudaStream_t s) override {
    if (!pipelined) return VNEC_CUDA(cudaStreamSynchronize(s));
    int h[2] = {0, 0};
    if (!VNEC_CUDA(cudaMemcpyAsync(h, flags.ptr, sizeof(h), cudaMemcpyDeviceToHost, s))) return false;
    if (!VNEC_CUDA(cudaStreamSynchronize(s))) return false;
    if (h[1]) {
      cudaMemsetAsync(flags.as<int>() + 1, 0, sizeof(int), s);
      cudaStreamSynchronize(s);
      set_error("merge-path pipeline: a bounded wait timed out (results of the affected call are invalid)");
      return false;
    }
    return true;
  }
};

bool shape_supported(int tpb, int ipt) {
  return (tpb == 128 || tpb == 256) && (ipt == 4 || ipt == 7 || ipt == 10);
}

// DF32 splits every value into two floats; that needs |a| in [2^-40, 2^41)
// (or a == 0) so that both halves and their products stay normal floats.
bool values_df32_safe(const CsrView& v) {
  if (v.type != SpB_FP64) return false;
  const double* a = static_cast<const double*>(v.val);
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t p = 0; p < v.nnz; ++p) {
    uint64_t b;
    std::memcpy(&b, a + p, 8);
    const int e = (int)((b >> 52) & 0x7ff);
    const bool zero = (b & 0x7FFFFFFFFFFFFFFFull) == 0;
    if (!zero && (e - 1023 < -40 || e - 1023 > 40)) bad = 1;
  }
  return !bad;
}

}  // namespace

std::unique_ptr<Plan> build_merge_path(const CsrView& v, const SpB_VNEC_options_ext* opts) {
  if (!validate_csr(v, false)) return nullptr;
  if (opts && opts->precision != 0) {
    set_error("precision forms apply to sliced plans (kernel S, or LEARNED / SEARCH / AUTO)");
    return nullptr;
  }
  auto p = std::make_unique<MergePathPlan>();
  p->type = v.type;
  p->n_rows = v.n_rows;
  p->n_cols = v.n_cols;
  p->nnz = v.nnz;
  cudaGetDevice(&p->device);
  const bool wide = (v.n_rows + v.nnz) >= ((int64_t)1 << 31) - 1 || (opts && opts->offsets64 > 0);
  const int req_stages = opts ? opts->pipeline_stages : 0;
  const int req_arith = opts ? opts->arithmetic : SpB_VNEC_ARITH_AUTO;
  // The pipelined kernel serves FP64 matrices with int32 merge coordinates.
  // By default large matrices (>= 2^26 nonzeros) take the unpipelined kernel
  // with 256 x 4 tiles: on GB300 timings of matrices that size it is 1.5x
  // faster (more resident warps than the shared-memory pipeline allows).
  constexpr int64_t kPipelineMaxNnz = (int64_t)1 << 26;
  const bool large = req_stages == 0 && v.nnz >= kPipelineMaxNnz;
  p->pipelined = v.type == SpB_FP64 && !wide && req_stages != 1 && !large;
  MpShape sh;
  if (p->pipelined) {
    sh.tpb = 256;
    sh.ipt = 7;
  } else if (large) {
    sh.ipt = 4;
  }
  if (opts && opts->threads_per_block) sh.tpb = opts->threads_per_block;
  if (opts && opts->items_per_thread) sh.ipt = opts->items_per_thread;
  const int stages = req_stages >= 2 ? req_stages : 2;
  if (p->pipelined ? mp2_smem(sh.tpb, sh.ipt, stages) == 0 : !shape_supported(sh.tpb, sh.ipt)) {
    set_error(p->pipelined ? "unsupported pipelined tile shape (256x7 s2/s3, 256x12 s2, 128x12 s3, 512x5 s2)"
                           : "unsupported merge-path tile shape (threads 128/256, items 4/7/10)");
    return nullptr;
  }
  if (p->pipelined) {
    if (req_arith == SpB_VNEC_ARITH_DF32 && !values_df32_safe(v)) {
      set_error("DF32 arithmetic requested but a matrix value lies outside [2^-40, 2^41)");
      return nullptr;
    }
    p->df32 = req_arith == SpB_VNEC_ARITH_DF32 || (req_arith == SpB_VNEC_ARITH_AUTO && values_df32_safe(v));
  }
  MpMatrix& m = p->m;
  m.n_rows = v.n_rows;
  m.n_cols = v.n_cols;
  m.nnz = v.nnz;
  m.shape = sh;
  m.wide = wide;
  const size_t ob = m.wide ? 8 : 4;
  const size_t vb = v.value_bytes();
  const int64_t ipc = sh.items_per_tile();
  m.num_tiles = (v.n_rows + v.nnz + ipc - 1) / ipc;
  // Device arrays are padded by 16 elements so that widened bulk copies and
  // vector loads near the end stay inside the allocation.
  const size_t pad = 16;
  if (!p->row_end.alloc(ob * (v.n_rows + pad)) || !p->col.alloc(4 * (v.nnz + pad)) ||
      !p->val.alloc(vb * (v.nnz + pad)) || !p->tile_row.alloc(ob * (m.num_tiles + 1)) ||
      !p->tile_nz.alloc(ob * (m.num_tiles + 1)) || !p->carry_row.alloc(ob * (m.num_tiles + 1)) ||
      !p->carry_val.alloc(8 * (m.num_tiles + 1)) || !p->flags.alloc(64))
    return nullptr;
  {
    std::vector<unsigned char> host_end(ob * (size_t)std::max<int64_t>(v.n_rows, 1));
    convert_row_end(v, m.wide, host_end.data());
    if (v.n_rows && !VNEC_CUDA(cudaMemcpy(p->row_end.ptr, host_end.data(), ob * v.n_rows, cudaMemcpyHostToDevice)))
      return nullptr;
  }
  if (v.nnz) {
    if (v.idx) {
      if (!VNEC_CUDA(cudaMemcpy(p->col.ptr, v.idx, 4 * v.nnz, cudaMemcpyHostToDevice))) return nullptr;
    } else {
      std::vector<int32_t> host_col((size_t)v.nnz);
      convert_cols(v, host_col.data());
      if (!VNEC_CUDA(cudaMemcpy(p->col.ptr, host_col.data(), 4 * v.nnz, cudaMemcpyHostToDevice))) return nullptr;
    }
    if (!VNEC_CUDA(cudaMemcpy(p->val.ptr, v.val, vb * v.nnz, cudaMemcpyHostToDevice))) return nullptr;
  }
  // Zero the padding so no uninitialised value is ever read.
  if (!VNEC_CUDA(cudaMemset(p->col.as<char>() + 4 * v.nnz, 0, 4 * pad)) ||
      !VNEC_CUDA(cudaMemset(p->val.as<char>() + vb * v.nnz, 0, vb * pad)) ||
      !VNEC_CUDA(cudaMemset(p->row_end.as<char>() + ob * v.n_rows, 0, ob * pad)) ||
      !VNEC_CUDA(cudaMemset(p->flags.ptr, 0, 64)) ||
      !VNEC_CUDA(cudaMemset(p->carry_row.ptr, 0, p->carry_row.bytes)))
    return nullptr;
  m.row_end = p->row_end.ptr;
  m.col = p->col.as<int32_t>();
  m.val = p->val.ptr;
  m.tile_row = p->tile_row.ptr;
  m.tile_nz = p->tile_nz.ptr;
  m.carry_row = p->carry_row.ptr;
  m.carry_val = p->carry_val.ptr;
  if (p->pipelined) {
    Mp2Matrix& q = p->m2;
    q.n_rows = v.n_rows;
    q.n_cols = v.n_cols;
    q.nnz = v.nnz;
    q.row_end = p->row_end.as<int>();
    q.col = p->col.as<int32_t>();
    q.val = p->val.as<double>();
    q.tile_row = p->tile_row.as<int>();
    q.tile_nz = p->tile_nz.as<int>();
    q.carry_row = p->carry_row.as<int>();
    q.carry_val = p->carry_val.as<double>();
    q.flags = p->flags.as<int>();
    q.num_tiles = m.num_tiles;
    q.shape = sh;
    q.stages = stages;
    if (!VNEC_CUDA(cudaDeviceGetAttribute(&q.sms, cudaDevAttrMultiProcessorCount, p->device))) return nullptr;
  }
  if (v.n_rows > 0) {
    if (!mp_partition(m, nullptr)) return nullptr;
    if (!VNEC_CUDA(cudaDeviceSynchronize())) return nullptr;
  }
  return p;
}

// ---------------------------------------------------------------------------
// IRD selector (ird_calc.c:2-122), restated for a host CSR view.
// ---------------------------------------------------------------------------
IrdParams ird_params(SpB_Type type) {
  // Constants of the reference's X86_SIMD build (SpB_mxv.h:25-32).
  if (type == SpB_FP32) return IrdParams{36, 16, 0.437f};
  return IrdParams{36, 8, 0.477f};
}

namespace {
// MergePathDivide (spmv_vnec_common.c:3-33) on a host view.
void merge_divide(const CsrView& v, int64_t diag, int64_t* x, int64_t* y) {
  int64_t lo = std::max<int64_t>(diag - v.nnz, 0), hi = std::min<int64_t>(diag, v.n_rows);
  while (lo < hi) {
    int64_t p = (lo + hi) >> 1;
    if (v.row_begin(p + 1) <= diag - p - 1)
      lo = p + 1;
    else
      hi = p;
  }
  *x = std::min<int64_t>(lo, v.n_rows);
  *y = diag - lo;
}
}  // namespace

float ird_ratio(const CsrView& v, const IrdParams& prm) {
  const int P = prm.nparts;
  std::vector<int64_t> sx(P), sy(P), ex(P), ey(P);
  const int64_t items = v.nnz + v.n_rows, per = (items + P - 1) / P;
  for (int t = 0; t < P; ++t) {
    int64_t d0 = std::min(per * t, items), d1 = std::min(d0 + per, items);
    merge_divide(v, d0, &sx[t], &sy[t]);
    merge_divide(v, d1, &ex[t], &ey[t]);
  }
  const int64_t words = (v.n_cols + 63) / 64;
  int64_t blocks_total = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : blocks_total)
  for (int t = 0; t < P; ++t) {
    // ECR ranks: rank of a column among the distinct columns of the partition.
    std::vector<uint64_t> bits((size_t)words, 0);
    for (int64_t p = sy[t]; p < ey[t]; ++p) {
      int64_t c = v.col_at(p);
      bits[c >> 6] |= 1ull << (c & 63);
    }
    std::vector<int32_t> base((size_t)words + 1, 0);
    for (int64_t w = 0; w < words; ++w) base[w + 1] = base[w] + __builtin_popcountll(bits[w]);
    auto rank = [&](int64_t c) -> int64_t {
      uint64_t below = bits[c >> 6] & ((1ull << (c & 63)) - 1);
      return base[c >> 6] + __builtin_popcountll(below);
    };
    // Block grouping of the complete rows (ird_calc.c:72-101).
    int64_t g = 0;
    for (int64_t i = sx[t]; i < ex[t]; ++i) {
      int64_t p0 = std::max(v.row_begin(i), sy[t]);
      int64_t len = v.row_begin(i + 1) - p0;
      if (len <= 0) continue;
      int64_t cs = rank(v.col_at(p0));
      for (int64_t j = 1; j < len; ++j) {
        int64_t r = rank(v.col_at(p0 + j));
        if (r - cs >= prm.nlanes) {
          ++g;
          cs = r;
        }
      }
      ++g;
    }
    blocks_total += g;
  }
  // 32-bit, as the reference's `int _nnz_` (ird_calc.c:103): past 2^31 - 1 it
  // wraps the way the reference's does, so the decision stays the reference's.
  const int denom = (int)(uint32_t)(blocks_total * prm.nlanes);
  return (float)v.nnz / (float)denom;
}

}  // namespace vnec
