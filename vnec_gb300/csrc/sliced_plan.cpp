// Plan wrappers of the sliced row-group format (VNEC-S counterpart) and of the
// dense-block format built on the same warp-task layout (VNEC-D counterpart).

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <limits>

#include "host.h"
#include "sliced.h"

namespace vnec {
namespace {

struct SlicedPlan final : Plan {
  SlicedMatrix m;
  SlicedMixed mx;  // precision form (FP64 = plain)
  DeviceBuffer tasks, val, col, rowid, long_row, long_first, chunk_sum, xbuf, flag, row_scale, chunk_scale;
  DeviceBuffer hot_cols, xhot, col16, first, val_split, pat16, long_heavy;
  std::vector<int32_t> hot_host;  // hot-column window: original column of each slot
  SlicedParams prm;
  int64_t blocks = 0;  // dense-block plans: number of blocks of 4
  int64_t delta_nnz = 0, delta_rows = 0;  // stored with 16-bit column deltas (+ a first column per row)
  int64_t shared_nnz = 0, shared_steps = 0;  // of those, in shared-pattern tasks (one delta per step)
  // Host-vector calls are split into parts (consecutive row windows) so that
  // the copy of one part's y rows to the host overlaps the next part's SpMV.
  struct Part {
    int64_t t0, t1, l0, l1, r0, r1;  // task, long-row and row ranges
    int64_t h0, h1;                  // heavy long rows (SlicedMatrix::long_heavy) of the part
  };
  std::vector<Part> parts;
  // Each part runs on its own stream, with stream priorities falling from the
  // first part to the last: all parts are launched together once x is on the
  // device, the block scheduler serves earlier parts first, so parts finish in
  // order while later parts fill the SMs that earlier parts' tails leave idle;
  // copy_stream carries each part's y copy as soon as that part is done.
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaStream_t> part_streams;
  cudaEvent_t x_ready = nullptr;
  std::vector<cudaEvent_t> part_done;
  explicit SlicedPlan(PlanKind k) : Plan(k) {}
  ~SlicedPlan() override {
    for (cudaEvent_t e : part_done)
      if (e) cudaEventDestroy(e);
    if (x_ready) cudaEventDestroy(x_ready);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    for (cudaStream_t q : part_streams)
      if (q) cudaStreamDestroy(q);
  }
  // Picks the unroll (4, 8, 12 or 16 load steps in flight) by timing each on
  // this matrix: median of 3 calls after one warm-up, x filled with a constant.
  bool tune_unroll() {
    const size_t vb = type == SpB_FP64 ? 8 : 4;
    DeviceBuffer tx, ty;
    TimingStream ts;
    bool ok = tx.alloc(vb * (size_t)std::max<int64_t>(n_cols, 1)) && ty.alloc(vb * (size_t)std::max<int64_t>(n_rows, 1)) &&
              VNEC_CUDA(cudaMemset(tx.ptr, 0x3f, tx.bytes)) && ts.create();
    cudaStream_t s = ts.s;
    cudaEvent_t e0 = ts.e0, e1 = ts.e1;
    float best = 0.f;
    int best_u = 12;
    for (int u : {4, 8, 12, 16}) {
      if (!ok) break;
      m.unroll = u;
      std::vector<float> t;
      for (int rep = 0; rep < 4 && ok; ++rep) {
        ok = VNEC_CUDA(cudaEventRecord(e0, s)) && run(tx.ptr, ty.ptr, s) && VNEC_CUDA(cudaEventRecord(e1, s)) &&
             VNEC_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        if (ok && rep > 0 && VNEC_CUDA(cudaEventElapsedTime(&ms, e0, e1))) t.push_back(ms);
      }
      if (!ok) break;
      std::sort(t.begin(), t.end());
      if (best == 0.f || t[1] < best) {
        best = t[1];
        best_u = u;
      }
    }
    m.unroll = best_u;
    if (!ok && last_error()[0] == '\0') set_error("sliced: unroll timing failed");
    return ok;
  }
  bool ensure_part_streams() {
    if (part_streams.size() == parts.size()) return true;
    int least = 0, greatest = 0;
    if (!VNEC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest))) return false;
    const int levels = least - greatest + 1;  // greatest is the numerically lowest
    for (size_t i = part_streams.size(); i < parts.size(); ++i) {
      const int prio = greatest + (int)((int64_t)i * levels / (int64_t)parts.size());
      cudaStream_t q = nullptr;
      if (!VNEC_CUDA(cudaStreamCreateWithPriority(&q, cudaStreamNonBlocking, std::min(prio, least)))) return false;
      part_streams.push_back(q);
    }
    return true;
  }
  bool run_host(const void* h_x, void* h_y) override {
    if (mx.precision != kPrecFP64 || m.vpe != 1 || parts.size() < 2 || profiling) return Plan::run_host(h_x, h_y);
    std::lock_guard<std::mutex> g(host_mu);
    if (!drain_pipe()) return false;
    const size_t vb = type == SpB_FP64 ? 8 : 4;
    if (!own_stream && !VNEC_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking))) return false;
    if (!copy_stream && !VNEC_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking))) return false;
    if (!ensure_part_streams()) return false;
    if (!x_ready && !VNEC_CUDA(cudaEventCreateWithFlags(&x_ready, cudaEventDisableTiming))) return false;
    while (part_done.size() < parts.size()) {
      cudaEvent_t e = nullptr;
      if (!VNEC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming))) return false;
      part_done.push_back(e);
    }
    if (!dx.ptr && !dx.alloc(vb * (size_t)std::max<int64_t>(n_cols, 1))) return false;
    if (!dy.ptr && !dy.alloc(vb * (size_t)std::max<int64_t>(n_rows, 1))) return false;
    if (n_cols > 0 && !VNEC_CUDA(cudaMemcpyAsync(dx.ptr, h_x, vb * n_cols, cudaMemcpyHostToDevice, own_stream)))
      return false;
    if (!sliced_gather_hot(m, type == SpB_FP64, dx.ptr, own_stream) || !VNEC_CUDA(cudaEventRecord(x_ready, own_stream)))
      return false;
    for (size_t i = 0; i < parts.size(); ++i) {
      const Part& q = parts[i];
      cudaStream_t cs = part_streams[i];
      if (!VNEC_CUDA(cudaStreamWaitEvent(cs, x_ready, 0))) return false;
      SlicedMatrix mp = m;
      mp.tasks = m.tasks + q.t0;
      mp.num_tasks = q.t1 - q.t0;
      mp.long_row = m.long_row + q.l0;
      mp.long_first = m.long_first + q.l0;
      mp.num_long = q.l1 - q.l0;
      mp.long_heavy = m.long_heavy + q.h0;
      mp.num_heavy = q.h1 - q.h0;
      mp.heavy_sub = q.l0;
      mp.pf.n_tasks = m.pf.n_tasks - q.t0;  // task indices of a part count from its first task
      mp.hot_ready = true;  // gathered above
      if (!sliced_spmv(mp, type == SpB_FP64, dx.ptr, dy.ptr, cs) || !VNEC_CUDA(cudaEventRecord(part_done[i], cs)) ||
          !VNEC_CUDA(cudaStreamWaitEvent(copy_stream, part_done[i], 0)))
        return false;
      if (q.r1 > q.r0 &&
          !VNEC_CUDA(cudaMemcpyAsync(static_cast<char*>(h_y) + vb * q.r0, static_cast<char*>(dy.ptr) + vb * q.r0,
                                     vb * (q.r1 - q.r0), cudaMemcpyDeviceToHost, copy_stream)))
        return false;
    }
    if (!VNEC_CUDA(cudaStreamSynchronize(copy_stream))) return false;
    for (cudaStream_t q : part_streams)
      if (!VNEC_CUDA(cudaStreamSynchronize(q))) return false;
    return device_status(own_stream);
  }
  bool run(const void* d_x, void* d_y, cudaStream_t s) override {
    if (profiling && !ensure_events()) return false;
    if (mx.precision != kPrecFP64)
      return sliced_mixed_spmv(m, mx, static_cast<const double*>(d_x), static_cast<double*>(d_y), s,
                               profiling ? events : nullptr);
    return sliced_spmv(m, type == SpB_FP64, d_x, d_y, s, profiling ? events : nullptr);
  }
  int kernel_ms(float* ms, int cap) const override {
    if (!profiling || !events[0] || cap < 2) return 0;
    if (cudaEventSynchronize(events[2]) != cudaSuccess) return 0;
    cudaEventElapsedTime(&ms[0], events[0], events[1]);
    cudaEventElapsedTime(&ms[1], events[1], events[2]);
    return 2;
  }
  bool run_epilogue(const void* d_x, void* d_y, const SlicedEpilogue& e, cudaStream_t s) override {
    // Fused into the sliced kernel's (and long-row fix-up's) stores for the
    // plain form; other forms use the elementwise pass.
    if (mx.precision != kPrecFP64 || m.vpe != 1) return Plan::run_epilogue(d_x, d_y, e, s);
    if (profiling && !ensure_events()) return false;
    return sliced_spmv(m, type == SpB_FP64, d_x, d_y, s, profiling ? events : nullptr, &e);
  }
  int launches_per_call() const override {
    if (n_rows == 0) return 0;
    return mx.precision != kPrecFP64 ? sliced_mixed_launches(m, mx.precision) : sliced_launches(m);
  }
  int64_t device_bytes() const override {
    return (int64_t)(tasks.bytes + val.bytes + col.bytes + rowid.bytes + long_row.bytes + long_first.bytes +
                     chunk_sum.bytes + xbuf.bytes + flag.bytes + row_scale.bytes + chunk_scale.bytes + dx.bytes +
                     dy.bytes + hot_cols.bytes + xhot.bytes + col16.bytes + first.bytes + val_split.bytes +
                     pat16.bytes);
  }
  int64_t algorithmic_bytes() const override {
    // Stored value size of the form; x and y stay in the matrix's type.
    const int64_t io = type == SpB_FP64 ? 8 : 4;
    const int64_t sv = mx.precision == kPrecFP32 ? 4 : mx.precision == kPrecBF16 ? 2 : io;
    const int64_t scale = mx.precision == kPrecBF16 ? n_rows : 0;
    // Dense-block plans move whole blocks: 4 values and one start column each.
    if (kind == PlanKind::kWindowDense)
      return blocks * (4 * sv + 4) + (n_rows + 1) * 4 + n_cols * io + n_rows * io;
    // Columns: 4 bytes, or 2 bytes per delta-coded nonzero plus its row's first
    // column; shared-pattern tasks read 2 bytes per step for all their rows.
    const int64_t cols =
        4 * (nnz - delta_nnz) + 2 * (delta_nnz - shared_nnz) + 2 * shared_steps + 4 * delta_rows;
    return nnz * sv + cols + (n_rows + 1) * 4 + scale + n_cols * io + n_rows * io;
  }
  void describe(SpB_VNEC_info_ext* info) const override {
    info->kernel = kind == PlanKind::kWindowDense ? SpB_VNEC_KERNEL_D : SpB_VNEC_KERNEL_S;
    info->threads_per_block = 256;
    info->items_per_thread = m.unroll;
    info->num_tiles = m.num_tasks;
    info->blocks = blocks;
    info->precision = mx.precision;
    info->long_row_len = prm.long_len;
  }
};

// Hot-column window (SlicedMatrix::hot): the `want` most used columns that
// occur at least twice, hottest first.  `mapped` receives the layout's column
// array with each hot column c replaced by n_cols + slot.
// With `min_cover` > 0 the window is only built when its columns carry at
// least that fraction of the nonzeros.
bool choose_hot(const CsrView& v, int64_t want, double min_cover, std::vector<int32_t>* hot,
                std::vector<int32_t>* mapped) {
  if (want <= 0 || v.nnz == 0 || v.n_cols + want >= ((int64_t)1 << 31)) return false;
  std::vector<uint32_t> cnt((size_t)v.n_cols, 0);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < v.nnz; ++q) __atomic_fetch_add(&cnt[(size_t)v.col_at(q)], 1u, __ATOMIC_RELAXED);
  std::vector<int32_t> cand;
  for (int64_t c = 0; c < v.n_cols; ++c)
    if (cnt[(size_t)c] >= 2) cand.push_back((int32_t)c);
  auto hotter = [&](int32_t a, int32_t b) { return cnt[(size_t)a] != cnt[(size_t)b] ? cnt[(size_t)a] > cnt[(size_t)b] : a < b; };
  if ((int64_t)cand.size() > want) {
    std::nth_element(cand.begin(), cand.begin() + want, cand.end(), hotter);
    cand.resize((size_t)want);
  }
  std::sort(cand.begin(), cand.end(), hotter);
  if (cand.empty()) return false;
  int64_t covered = 0;
  for (int32_t c : cand) covered += cnt[(size_t)c];
  if ((double)covered < min_cover * (double)v.nnz) return false;
  // The default window also needs skew: its columns must carry at least 4x
  // their share of the nonzeros (uniform column use gains nothing from a
  // window but pays its gather launch).
  if (min_cover > 0.0 && (double)covered * (double)v.n_cols < 4.0 * (double)cand.size() * (double)v.nnz)
    return false;
  std::vector<int32_t> slot((size_t)v.n_cols, -1);
  for (size_t s = 0; s < cand.size(); ++s) slot[(size_t)cand[s]] = (int32_t)s;
  mapped->resize((size_t)v.nnz);
  const int32_t nc = (int32_t)v.n_cols;
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < v.nnz; ++q) {
    const int32_t c = (int32_t)v.col_at(q);
    const int32_t sl = slot[(size_t)c];
    (*mapped)[(size_t)q] = sl >= 0 ? nc + sl : c;
  }
  *hot = std::move(cand);
  return true;
}

// Hot-first entry order: within each row, the entries of hot-window columns
// come first, hottest slot first, then the other entries in CSR order; `col`
// (the relabelled columns) and the values are permuted in place of a copy.
// row_key[r] is the slot of row r's first entry (n_cols + slot > n_cols for a
// hot column, INT32_MAX otherwise): rows of equal length sorted by it put
// rows sharing their hottest column side by side, so the lanes of one gather
// step read the same few x lines.
void hot_first_order(const CsrView& v, int32_t n_cols, const void* val, int vb, std::vector<int32_t>* col,
                     std::vector<unsigned char>* out_val, std::vector<int32_t>* row_key) {
  out_val->resize((size_t)std::max<int64_t>(v.nnz, 1) * vb);
  row_key->assign((size_t)std::max<int64_t>(v.n_rows, 1), INT32_MAX);
  const unsigned char* src = static_cast<const unsigned char*>(val);
#pragma omp parallel
  {
    std::vector<int64_t> idx;
    std::vector<int32_t> c;
#pragma omp for schedule(dynamic, 4096)
    for (int64_t r = 0; r < v.n_rows; ++r) {
      const int64_t b = v.row_begin(r), e = v.row_begin(r + 1);
      if (e == b) continue;
      idx.resize((size_t)(e - b));
      for (int64_t q = b; q < e; ++q) idx[(size_t)(q - b)] = q;
      // Hot entries (relabelled >= n_cols) by slot, then the rest in CSR order.
      std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t bq) {
        const int32_t ca = (*col)[(size_t)a], cb = (*col)[(size_t)bq];
        const bool ha = ca >= n_cols, hb = cb >= n_cols;
        if (ha != hb) return ha;
        return ha && ca < cb;
      });
      c.resize(idx.size());
      for (size_t k = 0; k < idx.size(); ++k) {
        c[k] = (*col)[(size_t)idx[k]];
        std::memcpy(out_val->data() + (size_t)(b + (int64_t)k) * vb, src + (size_t)idx[k] * vb, (size_t)vb);
      }
      std::copy(c.begin(), c.end(), col->begin() + b);
      if (c[0] >= n_cols) (*row_key)[(size_t)r] = c[0];
    }
  }
}

// Window size asked for by the options (0: none) and the coverage it needs.
// Default: 32,768 columns (the best of 4K-4M on R-MAT 2^24 with FP64 x), built
// when they carry at least 5 % of the nonzeros and at least 4x their share of
// them.  The FP32 and BF16 forms gather 4-byte x, so the same L1 holds twice
// the slots: they first try 524,288 (R-MAT 2^24: FP32 0.828 -> 0.808 ms, BF16
// 0.823 -> 0.807 ms) and keep 32,768 where the larger window fails the test.
constexpr int64_t kHotDefault = 32768;
constexpr int64_t kHotDefaultX32 = 524288;
constexpr double kHotMinCover = 0.05;
int64_t hot_window(const SpB_VNEC_options_ext* opts, double* min_cover) {
  *min_cover = 0.0;
  if (opts && opts->hot_columns < 0) return 0;
  if (opts && opts->hot_columns > 0) return std::min<int64_t>(opts->hot_columns, 1 << 22);
  *min_cover = kHotMinCover;
  return kHotDefault;
}

// Default max_steps: 32, lowered for small matrices so that the grid still
// holds about 8,192 warp tasks (a GB300 runs ~9,700 warps at once): rows then
// spread over more lanes with fewer steps each (65,536 rows x 16 nonzeros:
// 4 steps, 21 -> 16 us per call).
SlicedParams params_from(const SpB_VNEC_options_ext* opts, int64_t nnz) {
  SlicedParams prm;
  if (opts && opts->window_rows > 0) prm.window_rows = opts->window_rows;
  if (opts && opts->long_row_len > 0) prm.long_len = opts->long_row_len;
  if (opts && opts->max_steps > 0) {
    prm.max_steps = std::min(opts->max_steps, 1 << 20);
  } else {
    while (prm.max_steps > 1 && nnz < (int64_t)prm.max_steps * 32 * 8192) prm.max_steps >>= 1;
  }
  prm.chunk = std::max(32, (prm.long_len + 31) / 32 * 32);
  return prm;
}

// FP64 -> BF16: round to nearest even applied to the FP32 rounding of the
// value.  This double rounding can differ from a direct FP64 -> BF16 rounding
// by one BF16 unit in rare ties; the stored value stays within 2^-8 relative.
uint16_t to_bf16(double v) {
  const float f = static_cast<float>(v);
  uint32_t b;
  std::memcpy(&b, &f, 4);
  if ((b & 0x7f800000u) == 0x7f800000u) return static_cast<uint16_t>((b >> 16) | ((b & 0xffff) ? 0x40 : 0));
  b += 0x7fffu + ((b >> 16) & 1u);
  return static_cast<uint16_t>(b >> 16);
}

// Rewrites a stride-32 entry array into lane runs of P steps (the layout of
// SlicedMatrix::lane_run): inside each task, every full block of P steps x 32
// lanes is transposed so that each lane's P entries are adjacent.
template <typename T>
void to_lane_runs(const SlicedHostView& hv, int P, T* a) {
#pragma omp parallel
  {
    std::vector<T> tmp((size_t)32 * P);
#pragma omp for schedule(dynamic, 4096)
    for (int64_t t = 0; t < hv.num_tasks; ++t) {
      const SlicedTask& k = hv.tasks[t];
      if ((k.meta & 15) == kSlicedZero) continue;
      for (int b = 0; b < k.steps / P; ++b) {
        T* blk = a + k.base + (int64_t)b * 32 * P;
        for (int st = 0; st < P; ++st)
          for (int l = 0; l < 32; ++l) tmp[(size_t)(l * P + st)] = blk[st * 32 + l];
        std::copy(tmp.begin(), tmp.end(), blk);
      }
    }
  }
}

// Uploads a built host layout into a plan.  `row_exp` (BF16 form): the
// power-of-two exponent each row was scaled by.
std::unique_ptr<Plan> upload(std::unique_ptr<SlicedPlan> p, SlicedHost* h, int vb, const SpB_VNEC_options_ext* opts,
                             const std::vector<signed char>* row_exp = nullptr, bool keep_mask = false) {
  std::unique_ptr<SlicedHost, void (*)(SlicedHost*)> guard(h, sliced_free);
  SlicedHostView hv = sliced_view(h);
  const size_t pad = 64;
  const int prec = p->mx.precision;
  // Stored values: FP64/FP32 as built, or converted for the FP32 / BF16 forms.
  std::vector<unsigned char> conv;
  const void* vals = hv.val;
  size_t evb = (size_t)vb;
  if (prec == kPrecFP32 || prec == kPrecBF16) {
    const double* src = static_cast<const double*>(hv.val);
    const int64_t ne = hv.entries + (int64_t)pad;
    evb = prec == kPrecFP32 ? 4 : 2;
    conv.resize((size_t)ne * evb);
    if (prec == kPrecFP32) {
      float* d = reinterpret_cast<float*>(conv.data());
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < ne; ++i) d[i] = static_cast<float>(src[i]);
    } else {
      uint16_t* d = reinterpret_cast<uint16_t*>(conv.data());
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < ne; ++i) d[i] = to_bf16(src[i]);
    }
    vals = conv.data();
  }
  const size_t eb = evb * hv.vpe;
  // FP32 / BF16 forms: lane runs of 16 bytes of values (4 / 8 steps).  By
  // default where most entries sit in 16-bit-delta tasks (local columns,
  // stream-bound: the 256^3 stencil runs 11% / 7% faster); gather-bound
  // layouts keep stride 32.  The FP32 form also keeps stride 32 where most
  // entries sit in shared-pattern tasks: there its kernel needs 32 registers
  // against 48 for lane runs, and the extra resident warps hide more latency
  // than the 16-byte loads save (256^3 stencil, unroll 4: 0.560 -> 0.551 ms).
  std::vector<int32_t> col_runs;
  std::vector<uint16_t> col16_runs;
  const int32_t* cols = hv.col;
  const uint16_t* col16 = hv.col16;
  int run = 0;
  const int lv = opts ? opts->lane_vectors : 0;
  if ((prec == kPrecFP32 || prec == kPrecBF16) && hv.vpe == 1 && lv >= 0) {
    int64_t delta_entries = 0, shared_entries = 0;
    bool aligned = true;
    for (int64_t t = 0; t < hv.num_tasks; ++t) {
      const SlicedTask& k = hv.tasks[t];
      if ((k.meta & 15) == kSlicedZero) continue;
      if (k.meta & kSlicedDelta) delta_entries += (int64_t)k.steps * 32;
      if (k.meta & kSlicedShared) shared_entries += (int64_t)k.steps * 32;
      if (k.base % 32 != 0) aligned = false;  // vector loads need bases aligned to 32 entries
    }
    const bool fp32_shared = prec == kPrecFP32 && 2 * shared_entries >= hv.entries;
    if (aligned && (lv > 0 || (2 * delta_entries >= hv.entries && !fp32_shared))) run = prec == kPrecFP32 ? 4 : 8;
  }
  if (run) {
    const size_t ne = (size_t)(hv.entries + pad);
    if (prec == kPrecFP32)
      to_lane_runs(hv, run, reinterpret_cast<float*>(conv.data()));
    else
      to_lane_runs(hv, run, reinterpret_cast<uint16_t*>(conv.data()));
    col_runs.assign(hv.col, hv.col + ne);
    to_lane_runs(hv, run, col_runs.data());
    cols = col_runs.data();
    if (hv.col16) {
      col16_runs.assign(hv.col16, hv.col16 + ne);
      to_lane_runs(hv, run, col16_runs.data());
      col16 = col16_runs.data();
    }
  }
  // Long rows whose chunk sums one warp adds up in the fix-up launch.
  std::vector<int32_t> heavy;
  for (int64_t i = 0; i < hv.num_long; ++i)
    if (hv.long_first[i + 1] - hv.long_first[i] > kHeavyChunks) heavy.push_back((int32_t)i);
  auto up = [](DeviceBuffer& b, const void* src, size_t bytes, size_t alloc) {
    if (!b.alloc(std::max(alloc, bytes))) return false;
    return bytes == 0 || VNEC_CUDA(cudaMemcpy(b.ptr, src, bytes, cudaMemcpyHostToDevice));
  };
  if (!up(p->tasks, hv.tasks, sizeof(SlicedTask) * hv.num_tasks, sizeof(SlicedTask) * hv.num_tasks) ||
      !up(p->val, vals, eb * (hv.entries + pad), 0) ||
      !up(p->col, cols, 4 * (size_t)(hv.entries + pad), 0) ||
      !up(p->rowid, hv.rowid, 4 * (size_t)hv.n_rowid, 4 * (size_t)hv.n_rowid + 64) ||
      !up(p->long_row, hv.long_row, 4 * (size_t)hv.num_long, 4 * (size_t)hv.num_long + 64) ||
      !up(p->long_first, hv.long_first, 4 * (size_t)(hv.num_long + 1), 0) ||
      !up(p->long_heavy, heavy.data(), 4 * heavy.size(), 4 * heavy.size() + 64) ||
      !p->chunk_sum.alloc((size_t)vb * (hv.num_chunks + 1)))
    return nullptr;
  const int64_t nhot = (int64_t)p->hot_host.size();
  if (nhot > 0) {
    if (!up(p->hot_cols, p->hot_host.data(), 4 * (size_t)nhot, 0) || !p->xhot.alloc((size_t)vb * nhot + 16)) return nullptr;
    p->m.hot = (int)nhot;
    p->m.hot_cols = p->hot_cols.as<int32_t>();
    p->m.xhot = p->xhot.ptr;
  }
  if (prec != kPrecFP64) {
    if (!p->xbuf.alloc((size_t)std::max<int64_t>(p->n_cols + nhot, 1) * (prec == kPrecDF32 ? 8 : 4)) ||
        !p->flag.alloc(16) ||
        !VNEC_CUDA(cudaMemset(p->flag.ptr, 0, 16)))
      return nullptr;
    p->mx.xbuf = p->xbuf.ptr;
    p->mx.flag = p->flag.as<int>();
  }
  if (prec == kPrecBF16) {
    std::vector<signed char> rs((size_t)std::max<int64_t>(hv.n_rowid, 1)), cs((size_t)std::max<int64_t>(hv.num_chunks, 1));
    for (int64_t k = 0; k < hv.n_rowid; ++k) rs[(size_t)k] = (*row_exp)[(size_t)hv.rowid[k]];
    for (int64_t i = 0; i < hv.num_long; ++i)
      for (int32_t c = hv.long_first[i]; c < hv.long_first[i + 1]; ++c) cs[(size_t)c] = (*row_exp)[(size_t)hv.long_row[i]];
    if (!up(p->row_scale, rs.data(), rs.size(), 0) || !up(p->chunk_scale, cs.data(), cs.size(), 0)) return nullptr;
    p->mx.row_scale = p->row_scale.as<signed char>();
    p->mx.chunk_scale = p->chunk_scale.as<signed char>();
  }
  if (prec == kPrecDF32) {
    // (hi, lo) pairs of the FP64 entries for the double-float kernel.
    const double* src = static_cast<const double*>(hv.val);
    const int64_t ne = hv.entries + (int64_t)pad;
    std::vector<float> split((size_t)ne * 2);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < ne; ++i) split_df_host(src[i], &split[2 * (size_t)i], &split[2 * (size_t)i + 1]);
    if (!up(p->val_split, split.data(), sizeof(float) * split.size(), 0)) return nullptr;
    p->mx.val_split = p->val_split.as<float2>();
  }
  if (hv.col16) {
    if (!up(p->col16, col16, sizeof(uint16_t) * (size_t)(hv.entries + pad), 0) ||
        !up(p->first, hv.first, sizeof(int32_t) * (size_t)std::max<int64_t>(hv.n_rowid, 1), 0))
      return nullptr;
    p->m.col16 = p->col16.as<uint16_t>();
    p->m.first = p->first.as<int32_t>();
  }
  if (hv.col16 && hv.pat16 && hv.shared_steps > 0) {
    if (!up(p->pat16, hv.pat16, sizeof(uint16_t) * (size_t)(hv.entries / 32 + pad), 0)) return nullptr;
    p->m.pat16 = p->pat16.as<uint16_t>();
    p->shared_nnz = hv.shared_nnz;
    p->shared_steps = hv.shared_steps;
  }
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
  m.long_heavy = p->long_heavy.as<int32_t>();
  m.num_heavy = (int64_t)heavy.size();
  m.chunk_sum = p->chunk_sum.ptr;
  m.lane_run = run;
  p->delta_nnz = hv.col16 ? hv.delta_nnz : 0;
  p->delta_rows = hv.col16 ? hv.delta_rows : 0;
  // Options: cache_hints 2 explicit L1/L2 policies, 3 no L1 allocation for the
  // streamed arrays, 4 the same with L1 evict-last x gathers; items_per_thread
  // selects the unroll (4, 8, 12, 16), and by default (0 or -1) the plan times
  // the four on the matrix: no one value suits every layout (R-MAT 2^24 runs
  // fastest at 12, the 256^3 stencil's shared-pattern tasks at 4, where 12 is
  // 1.4x slower in FP64).  The unroll changes how many loads are in flight,
  // not the order of any row's sums: y is the same at every value.
  m.cache_hints = (opts && opts->cache_hints >= 2 && opts->cache_hints <= 4) ? opts->cache_hints - 1 : 0;
  // L2 prefetch ahead of the running tasks (prefetch.cuh): by default 262,144
  // entries ahead where most nonzeros sit in 16-bit-delta row groups (local
  // columns: the tasks' chains wait on HBM; 256^3 stencil FP64 0.859 -> 0.777
  // ms, FP32 form 0.539 -> 0.470, BF16 0.447 -> 0.416, DF32 0.732 -> 0.666),
  // off for gather-bound layouts, where it only adds requests (R-MAT 2^24
  // FP64 0.908 -> 1.035 ms).
  {
    const int lp = opts ? opts->l2_prefetch : 0;
    const bool local = hv.col16 && 2 * hv.delta_nnz >= p->nnz;
    const int64_t d = m.vpe != 1 || lp < 0 ? 0 : lp > 0 ? (int64_t)(lp / 32) * 32 : (local ? 262144 : 0);
    if (d > 0 && hv.entries > 0) {
      m.pf.entries = d;
      m.pf.tasks = (long long)((double)d * (double)hv.num_tasks / (double)hv.entries);
      m.pf.rows = (long long)((double)d * (double)hv.n_rowid / (double)hv.entries);
      m.pf.n_entries = hv.entries;
      m.pf.n_tasks = hv.num_tasks;
      m.pf.n_rows = hv.n_rowid;
    }
  }
  const int ipt = opts ? opts->items_per_thread : 0;
  m.unroll = (ipt == 4 || ipt == 8 || ipt == 12 || ipt == 16) ? ipt : 12;
  if ((ipt == 0 || ipt == -1) && m.vpe == 1 && !p->tune_unroll()) return nullptr;
  // Parts for host-vector calls: about 8 groups of whole windows with equal
  // entries (only plans that compute every row: no keep mask).
  const int kParts = (opts && opts->host_parts > 0) ? std::min(opts->host_parts, 1024) : 8;
  if (hv.num_windows > 1 && !keep_mask && kParts > 1) {
    const int64_t W = p->prm.window_rows;
    int64_t w0 = 0;
    for (int i = 1; i <= kParts && w0 < hv.num_windows; ++i) {
      const int64_t target = hv.entries * i / kParts;
      int64_t w1 = w0 + 1;
      while (w1 < hv.num_windows && hv.win_entry[w1] < target) ++w1;
      if (i == kParts) w1 = hv.num_windows;
      const int64_t l0 = hv.win_long[w0], l1 = hv.win_long[w1];
      const int64_t h0 = std::lower_bound(heavy.begin(), heavy.end(), (int32_t)l0) - heavy.begin();
      const int64_t h1 = std::lower_bound(heavy.begin(), heavy.end(), (int32_t)l1) - heavy.begin();
      p->parts.push_back(SlicedPlan::Part{hv.win_task[w0], hv.win_task[w1], l0, l1,
                                          w0 * W, std::min<int64_t>(p->n_rows, w1 * W), h0, h1});
      w0 = w1;
    }
  }
  return p;
}

}  // namespace

std::unique_ptr<Plan> build_sliced(const CsrView& v, const SpB_VNEC_options_ext* opts, const uint8_t* keep) {
  if (!validate_csr(v, false)) return nullptr;
  auto p = std::make_unique<SlicedPlan>(PlanKind::kWindowSliced);
  p->type = v.type;
  p->n_rows = v.n_rows;
  p->n_cols = v.n_cols;
  p->nnz = v.nnz;
  cudaGetDevice(&p->device);
  p->prm = params_from(opts, v.nnz);
  const int prec = opts ? opts->precision : kPrecFP64;
  if (prec < kPrecFP64 || prec > kPrecDF32) {
    set_error("unknown precision form");
    return nullptr;
  }
  if (prec != kPrecFP64 && v.type != SpB_FP64) {
    set_error("precision forms apply to FP64 matrices");
    return nullptr;
  }
  p->mx.precision = prec;
  const int vb = (int)v.value_bytes();
  const double* a = static_cast<const double*>(v.val);
  int bad = 0;
  std::vector<signed char> row_exp;
  std::vector<double> scaled;
  const void* src_val = v.val;
  if (prec == kPrecFP32) {
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t q = 0; q < v.nnz; ++q)
      if (!(std::fabs(a[q]) <= (double)std::numeric_limits<float>::max())) bad = 1;
    if (bad) {
      set_error("FP32 form: a matrix value is not finite in FP32");
      return nullptr;
    }
  } else if (prec == kPrecDF32) {
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t q = 0; q < v.nnz; ++q) {
      int e = 0;
      if (a[q] != 0.0 && (!std::isfinite(a[q]) || (std::frexp(a[q], &e), e - 1 < -40 || e - 1 > 40))) bad = 1;
    }
    if (bad) {
      set_error("DF32 form: a matrix value lies outside [2^-40, 2^41)");
      return nullptr;
    }
  } else if (prec == kPrecBF16) {
    // Row scale 2^-e with e the exponent of the row's largest |value| (so the
    // scaled values lie in (-1, 1)), stored as int8.
    row_exp.assign((size_t)v.n_rows, 0);
    scaled.assign((size_t)std::max<int64_t>(v.nnz, 1), 0.0);
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t r = 0; r < v.n_rows; ++r) {
      double mx = 0.0;
      for (int64_t q = v.row_begin(r); q < v.row_begin(r + 1); ++q) mx = std::max(mx, std::fabs(a[q]));
      int e = 0;
      if (mx > 0.0) std::frexp(mx, &e);
      if (!std::isfinite(mx) || e < -120 || e > 120) bad = 1;
      row_exp[(size_t)r] = (signed char)std::max(-120, std::min(120, e));
      for (int64_t q = v.row_begin(r); q < v.row_begin(r + 1); ++q) scaled[(size_t)q] = std::ldexp(a[q], -e);
    }
    if (bad) {
      set_error("BF16 form: a row's magnitude is outside 2^[-120, 120] or not finite");
      return nullptr;
    }
    src_val = scaled.data();
  }
  std::vector<int32_t> mapped, row_key;
  std::vector<unsigned char> ordered_val;
  const int32_t* cols = v.idx;
  const uint64_t* cols64 = v.idx64;
  double min_cover = 0.0;
  const int64_t want_hot = hot_window(opts, &min_cover);
  const bool x32 = prec == kPrecFP32 || prec == kPrecBF16;
  const bool default_window = min_cover > 0.0;  // no explicit hot_columns option
  bool have_hot = false;
  if (default_window && x32) have_hot = choose_hot(v, kHotDefaultX32, min_cover, &p->hot_host, &mapped);
  if (!have_hot) have_hot = choose_hot(v, want_hot, min_cover, &p->hot_host, &mapped);
  if (have_hot) {
    cols = mapped.data();
    cols64 = nullptr;
    p->prm.hot = (int)p->hot_host.size();
    if (!(opts && opts->hot_order < 0)) {
      hot_first_order(v, (int32_t)v.n_cols, src_val, vb, &mapped, &ordered_val, &row_key);
      src_val = ordered_val.data();
      p->prm.row_key = row_key.data();
    }
  }
  // 16-bit column deltas where rows allow them (not with a hot window, whose
  // relabelled columns break the increasing order).
  p->prm.delta16 = p->prm.hot == 0 && !(opts && opts->column_deltas < 0);
  // Shared-pattern tasks: read by the precision forms' kernel (the FP64
  // kernel walks the per-lane deltas, which stay stored).
  p->prm.shared = p->prm.delta16 && prec != kPrecFP64 && !(opts && opts->shared_patterns < 0);
  SlicedHost* h = sliced_build(v.n_rows, v.n_cols, v.ptr, v.ptr64, cols, cols64, src_val, vb, p->prm, 1, keep);
  if (!h) {
    set_error("sliced format: more than 2^31 entries or row slots");
    return nullptr;
  }
  return upload(std::move(p), h, vb, opts, prec == kPrecBF16 ? &row_exp : nullptr, keep != nullptr);
}

// Dense-block format (VNEC-D counterpart, spmv_vnec_D_for_mxv.c:242-398):
// each row is cut into blocks of 4 consecutive columns — the first nonzero
// opens a block at its column, a later nonzero whose distance to the open
// block's start is below 4 takes that slot, any other opens a new block
// (the reference's grouping rule, :370-384, applied to global instead of
// partition-compressed columns) — and the blocks are laid out as entries of
// the sliced warp-task format.
std::unique_ptr<Plan> build_dense(const CsrView& v, const SpB_VNEC_options_ext* opts, const uint8_t* keep) {
  if (!validate_csr(v, true)) return nullptr;
  if (opts && opts->precision != 0) {
    set_error("precision forms apply to sliced plans (kernel S, or LEARNED / SEARCH / AUTO)");
    return nullptr;
  }
  constexpr int W = 4;
  auto p = std::make_unique<SlicedPlan>(PlanKind::kWindowDense);
  p->type = v.type;
  p->n_rows = v.n_rows;
  p->n_cols = v.n_cols;
  p->nnz = v.nnz;
  cudaGetDevice(&p->device);
  p->prm = params_from(opts, v.nnz);
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
                               p->prm, W, keep);
  if (!h) {
    set_error("dense-block format: more than 2^31 blocks or row slots");
    return nullptr;
  }
  return upload(std::move(p), h, vb, opts, nullptr, keep != nullptr);
}

namespace {

// Row-level dense/sparse split: rows whose dense-block fill (nonzeros / (4 x
// blocks), blocks formed by the dense-block grouping rule) reaches the
// threshold run in the dense-block format, the others in the sliced format.
// It generalises the reference's matrix-level choice between VNEC-D and
// VNEC-S (IRD against a fixed threshold, ird_calc.c:2-122 and
// SpB_mxv.h:17-32) to single rows; threshold 0 gives the pure dense-block
// plan, a threshold above 1 the pure sliced plan.
struct HybridPlan final : Plan {
  std::unique_ptr<Plan> dense, sparse;
  int fill_permille = 500;
  int64_t dense_rows = 0;
  HybridPlan() : Plan(PlanKind::kHybrid) {}
  bool run(const void* d_x, void* d_y, cudaStream_t s) override {
    for (Plan* q : {dense.get(), sparse.get()}) {
      if (!q) continue;
      q->profiling = profiling;
      if (!q->run(d_x, d_y, s)) return false;
    }
    return true;
  }
  int kernel_ms(float* ms, int cap) const override {
    if (!profiling || cap < 2) return 0;
    ms[0] = ms[1] = 0.f;
    for (const Plan* q : {dense.get(), sparse.get()}) {
      float part[8] = {0.f};
      if (!q) continue;
      const int n = q->kernel_ms(part, 8);
      for (int i = 0; i < n && i < 2; ++i) ms[i] += part[i];
    }
    return 2;
  }
  int launches_per_call() const override {
    return (dense ? dense->launches_per_call() : 0) + (sparse ? sparse->launches_per_call() : 0);
  }
  int64_t device_bytes() const override {
    return (dense ? dense->device_bytes() : 0) + (sparse ? sparse->device_bytes() : 0);
  }
  int64_t algorithmic_bytes() const override {
    const int64_t vb = type == SpB_FP64 ? 8 : 4;
    return nnz * (vb + 4) + (n_rows + 1) * 4 + n_cols * vb + n_rows * vb;
  }
  void describe(SpB_VNEC_info_ext* info) const override {
    if (sparse) sparse->describe(info);
    else if (dense) dense->describe(info);
    info->kernel = SpB_VNEC_KERNEL_HYBRID;
    info->blocks = dense_rows;
  }
};

}  // namespace

std::unique_ptr<Plan> build_hybrid(const CsrView& v, const SpB_VNEC_options_ext* opts) {
  if (!validate_csr(v, true)) return nullptr;
  if (opts && opts->precision != 0) {
    set_error("precision forms apply to sliced plans (kernel S, or LEARNED / SEARCH / AUTO)");
    return nullptr;
  }
  constexpr int W = 4;
  auto p = std::make_unique<HybridPlan>();
  p->type = v.type;
  p->n_rows = v.n_rows;
  p->n_cols = v.n_cols;
  p->nnz = v.nnz;
  cudaGetDevice(&p->device);
  p->fill_permille = (opts && opts->dense_fill_permille > 0) ? opts->dense_fill_permille : 500;
  // Row r goes dense when len_r * 1000 >= permille * 4 * blocks_r.
  std::vector<uint8_t> is_dense((size_t)std::max<int64_t>(v.n_rows, 1), 0);
  int64_t nd = 0;
#pragma omp parallel for schedule(static) reduction(+ : nd)
  for (int64_t r = 0; r < v.n_rows; ++r) {
    int64_t nb = 0, cs = 0;
    for (int64_t q = v.row_begin(r); q < v.row_begin(r + 1); ++q) {
      const int64_t c = v.col_at(q);
      if (nb == 0 || c - cs >= W) {
        ++nb;
        cs = c;
      }
    }
    const int64_t len = v.row_begin(r + 1) - v.row_begin(r);
    if (nb > 0 && len * 1000 >= (int64_t)p->fill_permille * W * nb) {
      is_dense[(size_t)r] = 1;
      ++nd;
    }
  }
  p->dense_rows = nd;
  SpB_VNEC_options_ext o;
  std::memset(&o, 0, sizeof(o));
  if (opts) o = *opts;
  if (nd > 0) {
    p->dense = build_dense(v, &o, nd == v.n_rows ? nullptr : is_dense.data());
    if (!p->dense) return nullptr;
  }
  if (nd < v.n_rows) {
    for (auto& f : is_dense) f = !f;
    p->sparse = build_sliced(v, &o, nd == 0 ? nullptr : is_dense.data());
    if (!p->sparse) return nullptr;
  }
  return p;
}

}  // namespace vnec
