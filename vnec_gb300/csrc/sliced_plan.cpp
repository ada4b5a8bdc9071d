// Plan wrapper of the sliced row-group format (VNEC-S counterpart).

#include <algorithm>
#include <cstring>

#include "host.h"
#include "sliced.h"

namespace vnec {
namespace {

struct SlicedPlan final : Plan {
  SlicedMatrix m;
  DeviceBuffer tasks, val, col, rowid, long_row, long_first, chunk_sum;
  SlicedParams prm;
  SlicedPlan() : Plan(PlanKind::kWindowSliced) {}
  bool run(const void* d_x, void* d_y, cudaStream_t s) override {
    if (profiling && !ensure_events()) return false;
    return sliced_spmv(m, type == SpB_FP64, d_x, d_y, s, profiling ? events : nullptr);
  }
  int kernel_ms(float* ms, int cap) const override {
    if (!profiling || !events[0] || cap < 2) return 0;
    if (cudaEventSynchronize(events[2]) != cudaSuccess) return 0;
    cudaEventElapsedTime(&ms[0], events[0], events[1]);
    cudaEventElapsedTime(&ms[1], events[1], events[2]);
    return 2;
  }
  int launches_per_call() const override { return n_rows > 0 ? sliced_launches(m) : 0; }
  int64_t device_bytes() const override {
    return (int64_t)(tasks.bytes + val.bytes + col.bytes + rowid.bytes + long_row.bytes + long_first.bytes +
                     chunk_sum.bytes + dx.bytes + dy.bytes);
  }
  int64_t algorithmic_bytes() const override {
    const int64_t vb = type == SpB_FP64 ? 8 : 4;
    return nnz * (vb + 4) + (n_rows + 1) * 4 + n_cols * vb + n_rows * vb;
  }
  void describe(SpB_VNEC_info_ext* info) const override {
    info->kernel = SpB_VNEC_KERNEL_S;
    info->threads_per_block = 256;
    info->items_per_thread = prm.max_steps;
    info->num_tiles = m.num_tasks;
  }
};

}  // namespace

std::unique_ptr<Plan> build_sliced(const CsrView& v, const SpB_VNEC_options_ext* opts) {
  if (!validate_csr(v, false)) return nullptr;
  auto p = std::make_unique<SlicedPlan>();
  p->type = v.type;
  p->n_rows = v.n_rows;
  p->n_cols = v.n_cols;
  p->nnz = v.nnz;
  cudaGetDevice(&p->device);
  SlicedParams& prm = p->prm;
  if (opts && opts->window_rows > 0) prm.window_rows = opts->window_rows;
  if (opts && opts->long_row_len > 0) prm.long_len = opts->long_row_len;
  if (opts && opts->max_steps > 0) prm.max_steps = std::min(opts->max_steps, 1 << 20);
  prm.chunk = std::max(32, (prm.long_len + 31) / 32 * 32);
  const int vb = (int)v.value_bytes();
  SlicedHost* h = sliced_build(v.n_rows, v.n_cols, v.ptr, v.ptr64, v.idx, v.idx64, v.val, vb, prm);
  if (!h) {
    set_error("sliced format: more than 2^31 entries or row slots");
    return nullptr;
  }
  std::unique_ptr<SlicedHost, void (*)(SlicedHost*)> guard(h, sliced_free);
  SlicedHostView hv = sliced_view(h);
  const size_t pad = 64;
  auto up = [](DeviceBuffer& b, const void* src, size_t bytes, size_t alloc) {
    if (!b.alloc(std::max(alloc, bytes))) return false;
    return bytes == 0 || VNEC_CUDA(cudaMemcpy(b.ptr, src, bytes, cudaMemcpyHostToDevice));
  };
  if (!up(p->tasks, hv.tasks, sizeof(SlicedTask) * hv.num_tasks, sizeof(SlicedTask) * hv.num_tasks) ||
      !up(p->val, hv.val, (size_t)vb * (hv.entries + pad), 0) ||
      !up(p->col, hv.col, 4 * (size_t)(hv.entries + pad), 0) ||
      !up(p->rowid, hv.rowid, 4 * (size_t)hv.n_rowid, 4 * (size_t)hv.n_rowid + 64) ||
      !up(p->long_row, hv.long_row, 4 * (size_t)hv.num_long, 4 * (size_t)hv.num_long + 64) ||
      !up(p->long_first, hv.long_first, 4 * (size_t)(hv.num_long + 1), 0) ||
      !p->chunk_sum.alloc((size_t)vb * (hv.num_chunks + 1)))
    return nullptr;
  SlicedMatrix& m = p->m;
  m.n_rows = v.n_rows;
  m.n_cols = v.n_cols;
  m.nnz = v.nnz;
  m.entries = hv.entries;
  m.num_tasks = hv.num_tasks;
  m.num_long = hv.num_long;
  m.num_chunks = hv.num_chunks;
  m.tasks = p->tasks.as<SlicedTask>();
  m.val = p->val.ptr;
  m.col = p->col.as<int32_t>();
  m.rowid = p->rowid.as<int32_t>();
  m.long_row = p->long_row.as<int32_t>();
  m.long_first = p->long_first.as<int32_t>();
  m.chunk_sum = p->chunk_sum.ptr;
  m.cache_hints = (opts && opts->cache_hints == 2) ? 1 : 0;
  return p;
}

}  // namespace vnec
