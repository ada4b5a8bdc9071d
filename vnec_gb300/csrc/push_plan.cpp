// Push plans (SpMSpV): A transposed to CSC at plan time and uploaded; calls
// with a sparse x (SpB_VNEC_spmspv_ext) or a dense x (SpB_mxv_device_ext).

#include <algorithm>
#include <cstring>
#include <vector>

#include "host.h"
#include "push.h"

namespace vnec {
namespace {

struct PushPlan final : Plan {
  PushMatrix m;
  DeviceBuffer col_ptr, row, val, status, sx_idx, sx_val;
  PushPlan() : Plan(PlanKind::kPush) {}
  bool run(const void* d_x, void* d_y, cudaStream_t s) override {
    return push_spmspv(m, type == SpB_FP64, n_cols, nullptr, d_x, d_y, s);
  }
  bool run_sparse(long long nx, const int32_t* d_idx, const void* d_val, void* d_y, cudaStream_t s) {
    return push_spmspv(m, type == SpB_FP64, nx, d_idx, d_val, d_y, s);
  }
  int kernel_ms(float*, int) const override { return 0; }
  int launches_per_call() const override { return n_cols > 0 ? 1 : 0; }
  int64_t device_bytes() const override {
    return (int64_t)(col_ptr.bytes + row.bytes + val.bytes + status.bytes + dx.bytes + dy.bytes + sx_idx.bytes +
                     sx_val.bytes);
  }
  int64_t algorithmic_bytes() const override {
    const int64_t vb = type == SpB_FP64 ? 8 : 4;
    return nnz * (vb + 4) + (n_cols + 1) * 8 + n_cols * vb + n_rows * vb;
  }
  void describe(SpB_VNEC_info_ext* info) const override {
    info->kernel = SpB_VNEC_KERNEL_PUSH;
    info->threads_per_block = 256;
  }
  bool device_status(cudaStream_t s) override {
    int h = 0;
    if (!VNEC_CUDA(cudaMemcpyAsync(&h, m.status, sizeof(h), cudaMemcpyDeviceToHost, s)) ||
        !VNEC_CUDA(cudaStreamSynchronize(s)))
      return false;
    if (h) {
      cudaMemsetAsync(m.status, 0, sizeof(int), s);
      cudaStreamSynchronize(s);
      set_error("SpMSpV: an index of x lies outside [0, n_cols) (that entry was skipped)");
      return false;
    }
    return true;
  }
};

}  // namespace

std::unique_ptr<Plan> build_push(const CsrView& v, const SpB_VNEC_options_ext*) {
  if (!validate_csr(v, false)) return nullptr;
  CsrTranspose t;
  if (!transpose_csr(v, &t)) return nullptr;
  auto p = std::make_unique<PushPlan>();
  p->type = v.type;
  p->n_rows = v.n_rows;
  p->n_cols = v.n_cols;
  p->nnz = v.nnz;
  cudaGetDevice(&p->device);
  const size_t vb = v.value_bytes();
  auto up = [](DeviceBuffer& b, const void* src, size_t bytes) {
    if (!b.alloc(bytes + 64)) return false;
    return bytes == 0 || VNEC_CUDA(cudaMemcpy(b.ptr, src, bytes, cudaMemcpyHostToDevice));
  };
  if (!up(p->col_ptr, t.row_ptr.data(), sizeof(int64_t) * t.row_ptr.size()) ||
      !up(p->row, t.col.data(), sizeof(int32_t) * (size_t)v.nnz) || !up(p->val, t.val.data(), vb * (size_t)v.nnz) ||
      !p->status.alloc(16) || !VNEC_CUDA(cudaMemset(p->status.ptr, 0, 16)))
    return nullptr;
  p->m.n_rows = v.n_rows;
  p->m.n_cols = v.n_cols;
  p->m.nnz = v.nnz;
  p->m.col_ptr = p->col_ptr.as<int64_t>();
  p->m.row = p->row.as<int32_t>();
  p->m.val = p->val.ptr;
  p->m.status = p->status.as<int>();
  return p;
}

bool push_run_sparse(Plan* p, long long nx, const int32_t* d_idx, const void* d_val, void* d_y, cudaStream_t s) {
  if (!p || p->kind != PlanKind::kPush) {
    set_error("SpMSpV needs a plan built with kernel SpB_VNEC_KERNEL_PUSH");
    return false;
  }
  return static_cast<PushPlan*>(p)->run_sparse(nx, d_idx, d_val, d_y, s);
}

bool push_run_sparse_host(Plan* p, long long nx, const int32_t* idx, const void* val, void* y) {
  if (!p || p->kind != PlanKind::kPush) {
    set_error("SpMSpV needs a plan built with kernel SpB_VNEC_KERNEL_PUSH");
    return false;
  }
  auto* q = static_cast<PushPlan*>(p);
  std::lock_guard<std::mutex> g(q->host_mu);
  if (!q->drain_pipe()) return false;
  const size_t vb = q->type == SpB_FP64 ? 8 : 4;
  if (!q->own_stream && !VNEC_CUDA(cudaStreamCreateWithFlags(&q->own_stream, cudaStreamNonBlocking))) return false;
  if (q->sx_idx.bytes < sizeof(int32_t) * (size_t)std::max<long long>(nx, 1)) {
    q->sx_idx.release();
    q->sx_val.release();
    if (!q->sx_idx.alloc(sizeof(int32_t) * (size_t)std::max<long long>(nx, 1)) ||
        !q->sx_val.alloc(vb * (size_t)std::max<long long>(nx, 1)))
      return false;
  }
  if (!q->dy.ptr && !q->dy.alloc(vb * (size_t)std::max<int64_t>(q->n_rows, 1))) return false;
  cudaStream_t s = q->own_stream;
  if (nx > 0 && (!VNEC_CUDA(cudaMemcpyAsync(q->sx_idx.ptr, idx, sizeof(int32_t) * nx, cudaMemcpyHostToDevice, s)) ||
                 !VNEC_CUDA(cudaMemcpyAsync(q->sx_val.ptr, val, vb * nx, cudaMemcpyHostToDevice, s))))
    return false;
  if (!q->run_sparse(nx, q->sx_idx.as<int32_t>(), q->sx_val.ptr, q->dy.ptr, s)) return false;
  if (q->n_rows > 0 && !VNEC_CUDA(cudaMemcpyAsync(y, q->dy.ptr, vb * q->n_rows, cudaMemcpyDeviceToHost, s)))
    return false;
  return q->device_status(s);
}

}  // namespace vnec
