// Plan wrappers of the sliced row-group format (VNEC-S counterpart) and of the
// dense-block format built on the same warp-task layout (VNEC-D counterpart).

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
  int64_t blocks = 0;  // dense-block plans: number of blocks of 4
  explicit SlicedPlan(PlanKind k) : Plan(k) {}
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
    info->kernel = kind == PlanKind::kWindowDense ? SpB_VNEC_KERNEL_D : SpB_VNEC_KERNEL_S;
    info->threads_per_block = 256;
    info->items_per_thread = prm.max_steps;
    info->num_tiles = m.num_tasks;
    info->blocks = blocks;
  }
};

SlicedParams params_from(const SpB_VNEC_options_ext* opts) {
  SlicedParams prm;
  if (opts && opts->window_rows > 0) prm.window_rows = opts->window_rows;
  if (opts && opts->long_row_len > 0) prm.long_len = opts->long_row_len;
  if (opts && opts->max_steps > 0) prm.max_steps = std::min(opts->max_steps, 1 << 20);
  prm.chunk = std::max(32, (prm.long_len + 31) / 32 * 32);
  return prm;
}

// Uploads a built host layout into a plan.
std::unique_ptr<Plan> upload(std::unique_ptr<SlicedPlan> p, SlicedHost* h, int vb, const SpB_VNEC_options_ext* opts) {
  std::unique_ptr<SlicedHost, void (*)(SlicedHost*)> guard(h, sliced_free);
  SlicedHostView hv = sliced_view(h);
  const size_t eb = (size_t)vb * hv.vpe;
  const size_t pad = 64;
  auto up = [](DeviceBuffer& b, const void* src, size_t bytes, size_t alloc) {
    if (!b.alloc(std::max(alloc, bytes))) return false;
    return bytes == 0 || VNEC_CUDA(cudaMemcpy(b.ptr, src, bytes, cudaMemcpyHostToDevice));
  };
  if (!up(p->tasks, hv.tasks, sizeof(SlicedTask) * hv.num_tasks, sizeof(SlicedTask) * hv.num_tasks) ||
      !up(p->val, hv.val, eb * (hv.entries + pad), 0) ||
      !up(p->col, hv.col, 4 * (size_t)(hv.entries + pad), 0) ||
      !up(p->rowid, hv.rowid, 4 * (size_t)hv.n_rowid, 4 * (size_t)hv.n_rowid + 64) ||
      !up(p->long_row, hv.long_row, 4 * (size_t)hv.num_long, 4 * (size_t)hv.num_long + 64) ||
      !up(p->long_first, hv.long_first, 4 * (size_t)(hv.num_long + 1), 0) ||
      !p->chunk_sum.alloc((size_t)vb * (hv.num_chunks + 1)))
    return nullptr;
  SlicedMatrix& m = p->m;
  m.n_rows = p->n_rows;
  m.n_cols = p->n_cols;
  m.nnz = p->nnz;
  m.vpe = hv.vpe;
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

}  // namespace

std::unique_ptr<Plan> build_sliced(const CsrView& v, const SpB_VNEC_options_ext* opts) {
  if (!validate_csr(v, false)) return nullptr;
  auto p = std::make_unique<SlicedPlan>(PlanKind::kWindowSliced);
  p->type = v.type;
  p->n_rows = v.n_rows;
  p->n_cols = v.n_cols;
  p->nnz = v.nnz;
  cudaGetDevice(&p->device);
  p->prm = params_from(opts);
  const int vb = (int)v.value_bytes();
  SlicedHost* h = sliced_build(v.n_rows, v.n_cols, v.ptr, v.ptr64, v.idx, v.idx64, v.val, vb, p->prm);
  if (!h) {
    set_error("sliced format: more than 2^31 entries or row slots");
    return nullptr;
  }
  return upload(std::move(p), h, vb, opts);
}

// Dense-block format (VNEC-D counterpart, spmv_vnec_D_for_mxv.c:242-398):
// each row is cut into blocks of 4 consecutive columns — the first nonzero
// opens a block at its column, a later nonzero whose distance to the open
// block's start is below 4 takes that slot, any other opens a new block
// (the reference's grouping rule, :370-384, applied to global instead of
// partition-compressed columns) — and the blocks are laid out as entries of
// the sliced warp-task format.
std::unique_ptr<Plan> build_dense(const CsrView& v, const SpB_VNEC_options_ext* opts) {
  if (!validate_csr(v, true)) return nullptr;
  constexpr int W = 4;
  auto p = std::make_unique<SlicedPlan>(PlanKind::kWindowDense);
  p->type = v.type;
  p->n_rows = v.n_rows;
  p->n_cols = v.n_cols;
  p->nnz = v.nnz;
  cudaGetDevice(&p->device);
  p->prm = params_from(opts);
  const int vb = (int)v.value_bytes();
  std::vector<int64_t> bptr((size_t)v.n_rows + 1, 0);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < v.n_rows; ++r) {
    int64_t nb = 0, cs = 0;
    for (int64_t q = v.row_begin(r); q < v.row_begin(r + 1); ++q) {
      const int64_t c = v.col_at(q);
      if (nb == 0 || c - cs >= W) {
        ++nb;
        cs = c;
      }
    }
    bptr[(size_t)r + 1] = nb;
  }
  for (int64_t r = 0; r < v.n_rows; ++r) bptr[(size_t)r + 1] += bptr[(size_t)r];
  const int64_t nblocks = bptr[(size_t)v.n_rows];
  std::vector<int32_t> bcol((size_t)std::max<int64_t>(nblocks, 1));
  std::vector<unsigned char> bval((size_t)std::max<int64_t>(nblocks, 1) * W * vb, 0);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < v.n_rows; ++r) {
    int64_t b = bptr[(size_t)r] - 1, cs = 0;
    for (int64_t q = v.row_begin(r); q < v.row_begin(r + 1); ++q) {
      const int64_t c = v.col_at(q);
      if (b < bptr[(size_t)r] || c - cs >= W) {
        ++b;
        cs = c;
        bcol[(size_t)b] = (int32_t)c;
      }
      std::memcpy(&bval[((size_t)b * W + (size_t)(c - cs)) * vb], static_cast<const unsigned char*>(v.val) + q * vb,
                  (size_t)vb);
    }
  }
  p->blocks = nblocks;
  SlicedHost* h = sliced_build(v.n_rows, v.n_cols, bptr.data(), nullptr, bcol.data(), nullptr, bval.data(), vb,
                               p->prm, W);
  if (!h) {
    set_error("dense-block format: more than 2^31 blocks or row slots");
    return nullptr;
  }
  return upload(std::move(p), h, vb, opts);
}

}  // namespace vnec
