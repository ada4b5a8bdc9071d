// Batch plans: the batched multi-right-hand-side layout (batch.h) in device
// memory, the CUDA graph each call replays, and the autotuner that picks the
// layout (lanes per row, long-row limit) and block size by timing candidates
// on a sample of the batch.

#include <omp.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "batch.h"
#include "host.h"

namespace vnec {
namespace {

struct BatchDev {
  DeviceBuffer tasks, val, col, rowid, long_row, long_first, chunk_long, chunk_sum, chunk_count, xbuf, flag;
  BatchMatrix m;
  int64_t bytes() const {
    return (int64_t)(tasks.bytes + val.bytes + col.bytes + rowid.bytes + long_row.bytes + long_first.bytes +
                     chunk_long.bytes + chunk_sum.bytes + chunk_count.bytes + xbuf.bytes + flag.bytes);
  }
};

bool df32_range_ok(double v) {
  if (v == 0.0) return true;
  if (!std::isfinite(v)) return false;
  int e = 0;
  std::frexp(v, &e);
  return e - 1 >= -40 && e - 1 <= 40;
}

bool up(DeviceBuffer& b, const void* src, size_t bytes, size_t extra = 64) {
  if (!b.alloc(bytes + extra)) return false;
  return bytes == 0 || VNEC_CUDA(cudaMemcpy(b.ptr, src, bytes, cudaMemcpyHostToDevice));
}

bool upload_batch(const BatchHost* h, int k, int precision, int wpb, int mode, BatchDev* d) {
  const BatchHostView v = batch_view(h);
  const size_t ne = (size_t)v.entries + 64;
  if (!up(d->tasks, v.tasks, sizeof(SlicedTask) * (size_t)v.num_tasks) ||
      !up(d->col, v.col, sizeof(int32_t) * ne, 0) || !up(d->rowid, v.rowid, 4 * (size_t)v.n_rowid) ||
      !up(d->long_row, v.long_row, 4 * (size_t)v.num_long) ||
      !up(d->long_first, v.long_first, 4 * (size_t)(v.num_long + 1)) ||
      !up(d->chunk_long, v.chunk_long, 4 * (size_t)v.num_chunks) ||
      !d->chunk_sum.alloc(sizeof(double) * ((size_t)v.num_chunks * k + 64)) ||
      !d->chunk_count.alloc(sizeof(int) * ((size_t)v.num_long + 16)) ||
      !VNEC_CUDA(cudaMemset(d->chunk_count.ptr, 0, d->chunk_count.bytes)))
    return false;
  const size_t nx = std::max<size_t>((size_t)v.n_cols * k, 1);
  if (precision == kPrecFP32) {
    std::vector<float> f(ne);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)ne; ++i) f[(size_t)i] = static_cast<float>(v.val[i]);
    if (!up(d->val, f.data(), sizeof(float) * ne, 0) || !d->xbuf.alloc(sizeof(float) * nx)) return false;
  } else if (precision == kPrecDF32) {
    std::vector<float> f(2 * ne);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)ne; ++i) split_df_host(v.val[i], &f[2 * (size_t)i], &f[2 * (size_t)i + 1]);
    if (!up(d->val, f.data(), sizeof(float) * 2 * ne, 0) || !d->xbuf.alloc(2 * sizeof(float) * nx) ||
        !d->flag.alloc(16) || !VNEC_CUDA(cudaMemset(d->flag.ptr, 0, 16)))
      return false;
  } else if (!up(d->val, v.val, sizeof(double) * ne, 0)) {
    return false;
  }
  BatchMatrix& m = d->m;
  m.n_rows = v.n_rows;
  m.n_cols = v.n_cols;
  m.nnz = v.nnz;
  m.entries = v.entries;
  m.k = k;
  m.lanes = v.lanes;
  m.num_tasks = v.num_tasks;
  m.num_long = v.num_long;
  m.num_chunks = v.num_chunks;
  m.tasks = d->tasks.as<SlicedTask>();
  m.val = d->val.ptr;
  m.flag = d->flag.as<int>();
  m.col = d->col.as<int32_t>();
  m.rowid = d->rowid.as<int32_t>();
  m.long_row = d->long_row.as<int32_t>();
  m.long_first = d->long_first.as<int32_t>();
  m.chunk_long = d->chunk_long.as<int32_t>();
  m.chunk_sum = d->chunk_sum.as<double>();
  m.chunk_count = d->chunk_count.as<int>();
  m.xbuf = d->xbuf.ptr;
  m.precision = precision;
  m.warps_per_block = wpb;
  m.mode = mode;
  m.grid = batch_grid(precision, k / v.lanes, wpb, mode);
  if (m.grid <= 0) {
    set_error("batch: no occupancy for the kernel");
    return false;
  }
  return true;
}

// Host CSR arrays of the batch in the builder's form (int64 offsets, int32 columns).
struct BatchSource {
  std::vector<int64_t> n_rows, n_cols;
  std::vector<const int64_t*> rp;
  std::vector<const int32_t*> ci;
  std::vector<const double*> val;
  std::vector<std::vector<int64_t>> own_rp;  // converted from 64-bit reference arrays
  std::vector<std::vector<int32_t>> own_ci;
  int size() const { return (int)n_rows.size(); }
};

bool make_source(int n, const CsrView* mats, BatchSource* s) {
  s->own_rp.resize((size_t)n);
  s->own_ci.resize((size_t)n);
  for (int m = 0; m < n; ++m) {
    const CsrView& v = mats[m];
    s->n_rows.push_back(v.n_rows);
    s->n_cols.push_back(v.n_cols);
    s->val.push_back(static_cast<const double*>(v.val));
    if (v.ptr) {
      s->rp.push_back(v.ptr);
    } else {
      auto& o = s->own_rp[(size_t)m];
      o.resize((size_t)v.n_rows + 1);
      for (int64_t r = 0; r <= v.n_rows; ++r) o[(size_t)r] = v.row_begin(r);
      s->rp.push_back(o.data());
    }
    if (v.idx) {
      s->ci.push_back(v.idx);
    } else {
      auto& o = s->own_ci[(size_t)m];
      o.resize((size_t)v.nnz);
      for (int64_t q = 0; q < v.nnz; ++q) o[(size_t)q] = (int32_t)v.col_at(q);
      s->ci.push_back(o.data());
    }
  }
  return true;
}

BatchHost* build_host(const BatchSource& s, const std::vector<int>& pick, int k, const BatchParams& prm) {
  std::vector<int64_t> nr, nc;
  std::vector<const int64_t*> rp;
  std::vector<const int32_t*> ci;
  std::vector<const double*> val;
  for (int m : pick) {
    nr.push_back(s.n_rows[(size_t)m]);
    nc.push_back(s.n_cols[(size_t)m]);
    rp.push_back(s.rp[(size_t)m]);
    ci.push_back(s.ci[(size_t)m]);
    val.push_back(s.val[(size_t)m]);
  }
  return batch_build((int)pick.size(), nr.data(), nc.data(), rp.data(), ci.data(), val.data(), k, prm);
}

// ---------------------------------------------------------------------------
// Autotuner.
// ---------------------------------------------------------------------------

struct TuneChoice {
  int lanes = 0, long_len = 1024, wpb = 8;
  int deep = 0;  // kernel mode: 1 twice the load steps in flight, 2 entries staged in registers
  // One warp per task (blocks dispatched in task order) instead of persistent
  // warps striding the task list.  The default: on the 512-matrix batch it
  // keeps the tasks in flight, and so the rows of X they gather, a compact
  // window (k = 32: DF32 27.2 -> 17.6 ms, FP32 11.6 -> 8.2 ms, FP64 31.3 ->
  // 29.4 ms per call).  The autotuner decides it on the whole batch.
  bool per_task = true;
};

std::mutex g_tune_mu;
std::map<std::string, TuneChoice>& tune_cache() {
  static auto* c = new std::map<std::string, TuneChoice>();
  return *c;
}

int ilog2(int64_t v) {
  int l = 0;
  while (v > 1) {
    v >>= 1;
    ++l;
  }
  return l;
}

// Cache key: the device and driver, the call shape and coarse features of the
// batch (log2 buckets of its size and row lengths).
std::string tune_key(const BatchSource& s, int k, int precision) {
  int dev = 0, drv = 0;
  cudaGetDevice(&dev);
  cudaDriverGetVersion(&drv);
  cudaDeviceProp prop;
  std::memset(&prop, 0, sizeof(prop));
  cudaGetDeviceProperties(&prop, dev);
  int64_t rows = 0, nnz = 0, maxlen = 0;
  for (int m = 0; m < s.size(); ++m) {
    rows += s.n_rows[(size_t)m];
    nnz += s.rp[(size_t)m][s.n_rows[(size_t)m]];
    for (int64_t r = 0; r < s.n_rows[(size_t)m]; ++r)
      maxlen = std::max(maxlen, s.rp[(size_t)m][r + 1] - s.rp[(size_t)m][r]);
  }
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s|sm%d|drv%d|k%d|p%d|n%d|r%d|z%d|a%d|m%d", prop.name, prop.multiProcessorCount,
                drv, k, precision, ilog2(s.size()), ilog2(rows), ilog2(nnz), ilog2(rows ? 4 * nnz / rows : 0),
                ilog2(maxlen));
  for (char* c = buf; *c; ++c)
    if (*c == '"' || *c == '\n') *c = '_';
  return buf;
}

// Optional persistent cache: one JSON object per line in the file named by
// VNEC_TUNE_CACHE, {"key": "...", "lanes": L, "long_row_len": N, "warps_per_block": W,
// "deep_unroll": D, "dispatch": 1 (persistent warps) or 2 (one warp per task)}.
bool cache_file_lookup(const std::string& key, TuneChoice* c) {
  const char* path = std::getenv("VNEC_TUNE_CACHE");
  if (!path || !*path) return false;
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[1024];
  bool found = false;
  while (std::fgets(line, sizeof(line), f)) {
    char k[600];
    TuneChoice t;
    int dispatch = 0;
    if (std::sscanf(line,
                    "{\"key\": \"%599[^\"]\", \"lanes\": %d, \"long_row_len\": %d, \"warps_per_block\": %d, "
                    "\"deep_unroll\": %d, \"dispatch\": %d}",
                    k, &t.lanes, &t.long_len, &t.wpb, &t.deep, &dispatch) == 6 &&
        key == k) {
      t.per_task = dispatch == 2;
      *c = t;
      found = true;
    }
  }
  std::fclose(f);
  return found;
}

void cache_file_store(const std::string& key, const TuneChoice& c) {
  const char* path = std::getenv("VNEC_TUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f,
               "{\"key\": \"%s\", \"lanes\": %d, \"long_row_len\": %d, \"warps_per_block\": %d, "
               "\"deep_unroll\": %d, \"dispatch\": %d}\n",
               key.c_str(), c.lanes, c.long_len, c.wpb, c.deep, c.per_task ? 2 : 1);
  std::fclose(f);
}

// Matrices timed by the tuner: evenly spaced in nnz order, enough of them to
// hold `target` nonzeros (or the whole batch).
std::vector<int> tune_sample(const BatchSource& s, int64_t target) {
  const int n = s.size();
  std::vector<int> order((size_t)n);
  for (int m = 0; m < n; ++m) order[(size_t)m] = m;
  auto nnz_of = [&](int m) { return s.rp[(size_t)m][s.n_rows[(size_t)m]]; };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return nnz_of(a) < nnz_of(b); });
  for (int cnt = std::min(n, 16);; cnt = std::min(n, cnt * 2)) {
    std::vector<int> pick;
    int64_t z = 0;
    for (int i = 0; i < cnt; ++i) {
      const int m = order[(size_t)((int64_t)i * n / cnt)];
      pick.push_back(m);
      z += nnz_of(m);
    }
    std::sort(pick.begin(), pick.end());
    if (z >= target || cnt == n) return pick;
  }
}

struct TuneRun {
  std::vector<TuneChoice> cand;
  std::vector<float> ms;
  int best = -1;
};

float median_ms(std::vector<float> v) {
  std::sort(v.begin(), v.end());
  return v.empty() ? 0.f : v[v.size() / 2];
}

bool autotune(const BatchSource& s, int k, int precision, const SpB_VNEC_batch_options_ext* o, TuneRun* run) {
  std::vector<int> lanes_c, long_c{256, 1024, 4096}, wpb_c{4, 8}, deep_c{0, 1, 2};
  for (int L = 1; L <= 32; L <<= 1)
    if (batch_supported(k, L)) lanes_c.push_back(L);
  if (o->lanes > 0) lanes_c = {o->lanes};
  if (o->long_row_len > 0) long_c = {o->long_row_len};
  if (o->warps_per_block > 0) wpb_c = {o->warps_per_block};
  if (o->unroll > 0) deep_c = {o->unroll - 1};
  std::vector<int> disp_c{0, 1};  // 0: persistent warps, 1: one warp per task
  if (o->dispatch == 1) disp_c = {0};
  if (o->dispatch == 2) disp_c = {1};
  const std::vector<int> pick = tune_sample(s, (int64_t)48 << 20);
  TimingStream ts;
  if (!ts.create()) {
    set_error("batch autotune: cannot create a stream or events");
    return false;
  }
  cudaStream_t st = ts.s;
  cudaEvent_t e0 = ts.e0, e1 = ts.e1;
  DeviceBuffer X, Y;
  bool ok = true;
  for (int L : lanes_c) {
    for (int ll : long_c) {
      BatchParams prm;
      prm.lanes = L;
      prm.long_len = ll;
      prm.chunk = o->chunk > 0 ? o->chunk : ll;
      if (o->window_rows > 0) prm.window_rows = o->window_rows;
      if (o->max_steps > 0) prm.max_steps = o->max_steps;
      BatchHost* h = build_host(s, pick, k, prm);
      if (!h) continue;
      const BatchHostView hv = batch_view(h);
      const size_t nx = (size_t)std::max<int64_t>(hv.n_cols, 1) * k, ny = (size_t)std::max<int64_t>(hv.n_rows, 1) * k;
      if ((X.bytes < nx * 8 && !(X.release(), X.alloc(nx * 8))) || (Y.bytes < ny * 8 && !(Y.release(), Y.alloc(ny * 8))) ||
          !VNEC_CUDA(cudaMemset(X.ptr, 0x3f, nx * 8))) {
        batch_free(h);
        ok = false;
        break;
      }
      for (int wpb : wpb_c) {
        BatchDev d;
        if (!upload_batch(h, k, precision, wpb, false, &d)) {
          ok = false;
          break;
        }
        for (int deep : deep_c) {
          // The unroll changes only the kernel: same layout, new grid.  Each
          // candidate is timed with both dispatches and keeps the faster
          // (persistent only if it wins by more than 3 %).
          d.m.mode = deep;
          d.m.grid = batch_grid(precision, k / L, wpb, d.m.mode);
          float best_ms[2] = {0.f, 0.f};
          for (int pt : disp_c) {
            d.m.per_task = pt != 0;
            std::vector<float> t;
            for (int rep = 0; rep < 7 && ok; ++rep) {
              ok = VNEC_CUDA(cudaEventRecord(e0, st)) && batch_spmm(d.m, X.as<double>(), Y.as<double>(), st) &&
                   VNEC_CUDA(cudaEventRecord(e1, st)) && VNEC_CUDA(cudaEventSynchronize(e1));
              float ms = 0.f;
              if (ok && rep >= 2 && VNEC_CUDA(cudaEventElapsedTime(&ms, e0, e1))) t.push_back(ms);
            }
            if (!ok) break;
            best_ms[pt] = median_ms(t);
          }
          if (!ok) break;
          TuneChoice c{L, ll, wpb, deep};
          if (disp_c.size() == 2)
            c.per_task = !(best_ms[0] < 0.97f * best_ms[1]);
          else
            c.per_task = disp_c[0] != 0;
          run->cand.push_back(c);
          run->ms.push_back(best_ms[c.per_task ? 1 : 0]);
        }
        if (!ok) break;
      }
      batch_free(h);
      if (!ok) break;
    }
    if (!ok) break;
  }
  if (!ok) return false;
  for (size_t i = 0; i < run->ms.size(); ++i)
    if (run->best < 0 || run->ms[i] < run->ms[(size_t)run->best]) run->best = (int)i;
  if (run->best < 0) {
    set_error("batch autotune: no candidate layout could be built");
    return false;
  }
  return true;
}

// Times the uploaded plan with persistent warps and with one warp per task
// (median of 3 calls after one warm-up each, on scratch X and Y) and keeps
// persistent warps only when they win by more than 3 %.
bool whole_batch_dispatch(BatchMatrix& m, int64_t n_rows, int64_t n_cols, int k, bool* per_task) {
  TimingStream ts;
  DeviceBuffer X, Y;
  if (!ts.create()) {
    set_error("batch dispatch timing: cannot create a stream or events");
    return false;
  }
  const size_t nx = (size_t)std::max<int64_t>(n_cols, 1) * k, ny = (size_t)std::max<int64_t>(n_rows, 1) * k;
  if (!X.alloc(nx * 8) || !Y.alloc(ny * 8) || !VNEC_CUDA(cudaMemset(X.ptr, 0x3f, nx * 8))) return false;
  float med[2] = {0.f, 0.f};
  for (int pt = 0; pt < 2; ++pt) {
    m.per_task = pt != 0;
    std::vector<float> t;
    for (int rep = 0; rep < 4; ++rep) {
      if (!VNEC_CUDA(cudaEventRecord(ts.e0, ts.s)) || !batch_spmm(m, X.as<double>(), Y.as<double>(), ts.s) ||
          !VNEC_CUDA(cudaEventRecord(ts.e1, ts.s)) || !VNEC_CUDA(cudaEventSynchronize(ts.e1)))
        return false;
      float ms = 0.f;
      if (rep >= 1 && VNEC_CUDA(cudaEventElapsedTime(&ms, ts.e0, ts.e1))) t.push_back(ms);
    }
    med[pt] = median_ms(t);
  }
  *per_task = !(med[0] < 0.97f * med[1]);
  return true;
}

// ---------------------------------------------------------------------------
// Plan.
// ---------------------------------------------------------------------------

struct BatchPlan final : Plan {
  // k = 1 batches (SpB_VNEC_batch_options_ext::k1_layout 0): one sliced plan
  // of the block-diagonal concatenation runs every call; `d` stays empty.
  std::unique_ptr<Plan> k1;
  BatchDev d;
  BatchParams prm;
  TuneRun tuning;
  int precision = kPrecFP64;
  bool use_graph = true;
  std::vector<int64_t> row_off, col_off;
  // Graph of the last (x, y) pair.
  std::mutex gmu;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* gx = nullptr;
  void* gy = nullptr;

  // Host-vector calls run in parts of whole row windows.  The concatenation
  // is block-diagonal, so the rows of a part read only the X rows of the
  // matrices they belong to: part i's X rows are copied in on in_stream, its
  // tasks run on own_stream once they have arrived, and its Y rows are copied
  // out on out_stream — copies in both directions overlap the compute.
  struct Part {
    int64_t t0, t1, r0, r1, c0, c1;  // tasks, Y rows, X rows (new in this part)
  };
  std::vector<Part> parts;
  cudaStream_t in_stream = nullptr, out_stream = nullptr;
  std::vector<cudaEvent_t> x_in, done;

  BatchPlan() : Plan(PlanKind::kBatch) {}
  ~BatchPlan() override {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (cap) cudaStreamDestroy(cap);
    for (cudaEvent_t e : x_in)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : done)
      if (e) cudaEventDestroy(e);
    if (in_stream) cudaStreamDestroy(in_stream);
    if (out_stream) cudaStreamDestroy(out_stream);
  }

  bool run_host(const void* h_x, void* h_y) override {
    if (k1) {
      std::lock_guard<std::mutex> g(host_mu);
      if (!drain_pipe()) return false;
      k1->profiling = profiling;
      return k1->run_host(h_x, h_y);
    }
    if (parts.size() < 2 || profiling) return Plan::run_host(h_x, h_y);
    std::lock_guard<std::mutex> g(host_mu);
    if (!drain_pipe()) return false;
    const size_t row_bytes = sizeof(double) * (size_t)rhs;
    if (!own_stream && !VNEC_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking))) return false;
    if (!in_stream && !VNEC_CUDA(cudaStreamCreateWithFlags(&in_stream, cudaStreamNonBlocking))) return false;
    if (!out_stream && !VNEC_CUDA(cudaStreamCreateWithFlags(&out_stream, cudaStreamNonBlocking))) return false;
    while (x_in.size() < parts.size()) {
      cudaEvent_t a = nullptr, b = nullptr;
      if (!VNEC_CUDA(cudaEventCreateWithFlags(&a, cudaEventDisableTiming)) ||
          !VNEC_CUDA(cudaEventCreateWithFlags(&b, cudaEventDisableTiming)))
        return false;
      x_in.push_back(a);
      done.push_back(b);
    }
    if (!dx.ptr && !dx.alloc(row_bytes * (size_t)std::max<int64_t>(n_cols, 1))) return false;
    if (!dy.ptr && !dy.alloc(row_bytes * (size_t)std::max<int64_t>(n_rows, 1))) return false;
    for (size_t i = 0; i < parts.size(); ++i) {
      const Part& q = parts[i];
      if (q.c1 > q.c0 &&
          !VNEC_CUDA(cudaMemcpyAsync(static_cast<char*>(dx.ptr) + row_bytes * q.c0,
                                     static_cast<const char*>(h_x) + row_bytes * q.c0, row_bytes * (q.c1 - q.c0),
                                     cudaMemcpyHostToDevice, in_stream)))
        return false;
      if (!VNEC_CUDA(cudaEventRecord(x_in[i], in_stream)) || !VNEC_CUDA(cudaStreamWaitEvent(own_stream, x_in[i], 0)) ||
          !batch_spmm_range(d.m, dx.as<double>(), dy.as<double>(), own_stream, q.t0, q.t1, q.c0, q.c1, i == 0) ||
          !VNEC_CUDA(cudaEventRecord(done[i], own_stream)) || !VNEC_CUDA(cudaStreamWaitEvent(out_stream, done[i], 0)))
        return false;
      if (q.r1 > q.r0 &&
          !VNEC_CUDA(cudaMemcpyAsync(static_cast<char*>(h_y) + row_bytes * q.r0,
                                     static_cast<char*>(dy.ptr) + row_bytes * q.r0, row_bytes * (q.r1 - q.r0),
                                     cudaMemcpyDeviceToHost, out_stream)))
        return false;
    }
    return VNEC_CUDA(cudaStreamSynchronize(out_stream)) && VNEC_CUDA(cudaStreamSynchronize(in_stream)) &&
           device_status(own_stream);
  }

  // Pipelined host calls alternate two buffer slots: direct launches (one or
  // two kernels) instead of re-pointing the graph on every call.
  bool run_slot(int, const void* d_x, void* d_y, cudaStream_t s) override {
    if (k1) {
      k1->profiling = false;
      return k1->run(d_x, d_y, s);
    }
    return batch_spmm(d.m, static_cast<const double*>(d_x), static_cast<double*>(d_y), s);
  }
  // One call's kernels on `s`: the sliced plan's for a k = 1 batch, else the batch kernel's.
  bool enqueue(const void* d_x, void* d_y, cudaStream_t s) {
    if (k1) {
      k1->profiling = profiling;
      return k1->run(d_x, d_y, s);
    }
    return batch_spmm(d.m, static_cast<const double*>(d_x), static_cast<double*>(d_y), s);
  }
  bool run_epilogue(const void* d_x, void* d_y, const SlicedEpilogue& e, cudaStream_t s) override {
    if (!k1) return Plan::run_epilogue(d_x, d_y, e, s);
    k1->profiling = profiling;
    return k1->run_epilogue(d_x, d_y, e, s);
  }

  bool capture(const void* d_x, void* d_y) {
    if (!cap && !VNEC_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking))) return false;
    if (!VNEC_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal))) return false;
    const bool ok = enqueue(d_x, d_y, cap);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cap, &g);
    if (!ok || !VNEC_CUDA(e)) {
      if (g) cudaGraphDestroy(g);
      return false;
    }
    if (exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(exec, g, &info) != cudaSuccess) {
        cudaGetLastError();
        cudaGraphExecDestroy(exec);
        exec = nullptr;
      }
    }
    if (!exec && !VNEC_CUDA(cudaGraphInstantiate(&exec, g, 0))) {
      cudaGraphDestroy(g);
      return false;
    }
    if (graph) cudaGraphDestroy(graph);
    graph = g;
    gx = d_x;
    gy = d_y;
    return true;
  }

  bool run(const void* d_x, void* d_y, cudaStream_t s) override {
    const int R = k1 ? 1 : d.m.k / d.m.lanes;
    if (R >= 2 && ((reinterpret_cast<uintptr_t>(d_x) | reinterpret_cast<uintptr_t>(d_y)) & 15)) {
      set_error("batch: x and y must be 16-byte aligned for this plan's layout");
      return false;
    }
    if (profiling && k1) return enqueue(d_x, d_y, s);
    if (profiling) {
      if (!ensure_events() || !VNEC_CUDA(cudaEventRecord(events[0], s))) return false;
      if (!batch_spmm(d.m, static_cast<const double*>(d_x), static_cast<double*>(d_y), s)) return false;
      return VNEC_CUDA(cudaEventRecord(events[1], s));
    }
    if (!use_graph) return enqueue(d_x, d_y, s);
    std::lock_guard<std::mutex> g(gmu);
    if ((!exec || gx != d_x || gy != d_y) && !capture(d_x, d_y)) return false;
    return VNEC_CUDA(cudaGraphLaunch(exec, s));
  }
  int kernel_ms(float* ms, int cap_n) const override {
    if (k1) return k1->kernel_ms(ms, cap_n);
    if (!profiling || !events[0] || cap_n < 1) return 0;
    if (cudaEventSynchronize(events[1]) != cudaSuccess) return 0;
    cudaEventElapsedTime(&ms[0], events[0], events[1]);
    return 1;
  }
  int launches_per_call() const override {
    if (k1) return k1->launches_per_call();
    return n_rows == 0 && precision != kPrecFP32 ? 0 : batch_launches(d.m);
  }
  int64_t device_bytes() const override {
    return (k1 ? k1->device_bytes() : d.bytes()) + (int64_t)(dx.bytes + dy.bytes);
  }
  int64_t algorithmic_bytes() const override {
    const int64_t vb = precision == kPrecFP32 ? 4 : 8;  // DF32 stores (hi, lo) float pairs
    return nnz * (vb + 4) + (n_rows + (int64_t)row_off.size() - 1) * 4 + (n_cols + n_rows) * rhs * 8;
  }
  void describe(SpB_VNEC_info_ext* info) const override {
    if (k1) {
      k1->describe(info);
      info->kernel = SpB_VNEC_KERNEL_BATCH;
      info->rhs = rhs;
      info->lanes = 0;
      return;
    }
    info->kernel = SpB_VNEC_KERNEL_BATCH;
    info->threads_per_block = d.m.warps_per_block * 32;
    info->items_per_thread = d.m.k / d.m.lanes;
    info->num_tiles = d.m.num_tasks;
    info->blocks = d.m.grid;
    info->precision = precision;
    info->rhs = rhs;
    info->lanes = d.m.lanes;
    info->long_row_len = prm.long_len;
  }
};

// Host-call parts: about `n_parts` groups of whole windows with equal
// entries; part i copies in the X rows of the matrices its rows belong to that
// earlier parts did not (the last part takes every remaining X row).
void plan_parts(BatchPlan* p, const BatchHostView& hv, int n_parts) {
  p->parts.clear();
  if (hv.num_windows < 2 || n_parts < 2) return;
  const int64_t W = p->prm.window_rows;
  const int n = (int)p->row_off.size() - 1;
  int64_t w0 = 0, c_done = 0;
  for (int i = 1; i <= n_parts && w0 < hv.num_windows; ++i) {
    const int64_t target = hv.win_entry[hv.num_windows] * i / n_parts;
    int64_t w1 = w0 + 1;
    while (w1 < hv.num_windows && hv.win_entry[w1] < target) ++w1;
    if (i == n_parts) w1 = hv.num_windows;
    const int64_t r0 = w0 * W, r1 = std::min<int64_t>(p->n_rows, w1 * W);
    int64_t c1 = c_done;
    if (w1 == hv.num_windows) {
      c1 = p->n_cols;
    } else if (r1 > r0) {
      // matrix of the part's last row: the last m with row_off[m] <= r1 - 1
      const int m = (int)(std::upper_bound(p->row_off.begin(), p->row_off.end(), r1 - 1) - p->row_off.begin()) - 1;
      c1 = std::max(c_done, p->col_off[(size_t)std::min(m + 1, n)]);
    }
    p->parts.push_back(BatchPlan::Part{hv.win_task[w0], hv.win_task[w1], r0, r1, c_done, c1});
    c_done = c1;
    w0 = w1;
  }
}

// A k = 1 batch as one sliced plan: the block-diagonal concatenation (matrix
// m's rows at row_off[m], its columns shifted by col_off[m]) in CSR, planned
// with the batch's precision form and the sliced defaults.
bool build_k1(BatchPlan* p, const BatchSource& s, const SpB_VNEC_batch_options_ext& o) {
  const int n = s.size();
  if (p->n_rows > INT32_MAX || p->n_cols > INT32_MAX) {
    set_error("batch: more than 2^31 rows or columns");
    return false;
  }
  std::vector<int64_t> z_off((size_t)n + 1, 0);
  for (int m = 0; m < n; ++m)
    z_off[(size_t)m + 1] = z_off[(size_t)m] + s.rp[(size_t)m][s.n_rows[(size_t)m]] - s.rp[(size_t)m][0];
  std::vector<int64_t> rp((size_t)p->n_rows + 1, 0);
  std::vector<int32_t> ci((size_t)z_off[(size_t)n]);
  std::vector<double> val((size_t)z_off[(size_t)n]);
#pragma omp parallel for schedule(dynamic, 1)
  for (int m = 0; m < n; ++m) {
    const int64_t r0 = p->row_off[(size_t)m], c0 = p->col_off[(size_t)m], z0 = z_off[(size_t)m];
    const int64_t* src_rp = s.rp[(size_t)m];
    const int64_t base = src_rp[0];
    for (int64_t r = 0; r < s.n_rows[(size_t)m]; ++r) rp[(size_t)(r0 + r + 1)] = z0 + src_rp[r + 1] - base;
    const int64_t nz = src_rp[s.n_rows[(size_t)m]] - base;
    for (int64_t q = 0; q < nz; ++q) {
      ci[(size_t)(z0 + q)] = (int32_t)(s.ci[(size_t)m][base + q] + c0);
      val[(size_t)(z0 + q)] = s.val[(size_t)m][base + q];
    }
  }
  CsrView v;
  v.type = SpB_FP64;
  v.n_rows = p->n_rows;
  v.n_cols = p->n_cols;
  v.nnz = z_off[(size_t)n];
  v.ptr = rp.data();
  v.idx = ci.data();
  v.val = val.data();
  SpB_VNEC_options_ext so;
  std::memset(&so, 0, sizeof(so));
  so.kernel = SpB_VNEC_KERNEL_S;
  so.precision = o.precision;
  so.window_rows = o.window_rows;
  so.max_steps = o.max_steps;
  so.host_parts = o.host_parts;
  p->k1 = build_sliced(v, &so);
  return p->k1 != nullptr;
}

}  // namespace

std::unique_ptr<Plan> build_batch(int n, const CsrView* mats, int k, const SpB_VNEC_batch_options_ext* opts) {
  SpB_VNEC_batch_options_ext o;
  std::memset(&o, 0, sizeof(o));
  if (opts) o = *opts;
  if (n < 1 || !mats) {
    set_error("batch: no matrices");
    return nullptr;
  }
  if (k < 1 || k > 32 || (k & (k - 1))) {
    set_error("batch: k must be 1, 2, 4, 8, 16 or 32");
    return nullptr;
  }
  if (o.precision != kPrecFP64 && o.precision != kPrecFP32 && o.precision != kPrecDF32) {
    set_error("batch: precision must be SpB_VNEC_PREC_FP64, SpB_VNEC_PREC_FP32 or SpB_VNEC_PREC_DF32");
    return nullptr;
  }
  if (o.lanes > 0 && !batch_supported(k, o.lanes)) {
    set_error("batch: lanes must divide 32 and k with k / lanes in {1, 2, 4, 8}");
    return nullptr;
  }
  if (o.warps_per_block != 0 && o.warps_per_block != 4 && o.warps_per_block != 8) {
    set_error("batch: warps_per_block must be 4 or 8");
    return nullptr;
  }
  if (o.long_row_len < 0 || o.chunk < 0 || o.window_rows < 0 || o.max_steps < 0 || o.unroll < 0 || o.unroll > 3 ||
      o.dispatch < 0 || o.dispatch > 2) {
    set_error("batch: negative option");
    return nullptr;
  }
  if (o.k1_layout != 0 && o.k1_layout != -1) {
    set_error("batch: k1_layout must be 0 (sliced plan at k = 1) or -1 (batch kernel)");
    return nullptr;
  }
  auto p = std::make_unique<BatchPlan>();
  p->type = SpB_FP64;
  p->rhs = k;
  p->precision = o.precision;
  p->use_graph = o.no_graph == 0;
  cudaGetDevice(&p->device);
  p->row_off.assign((size_t)n + 1, 0);
  p->col_off.assign((size_t)n + 1, 0);
  for (int m = 0; m < n; ++m) {
    const CsrView& v = mats[m];
    if (v.type != SpB_FP64) {
      set_error("batch: matrix " + std::to_string(m) + " is not FP64");
      return nullptr;
    }
    if (!validate_csr(v, false)) {
      set_error("batch: matrix " + std::to_string(m) + ": " + last_error());
      return nullptr;
    }
    if (o.precision == kPrecFP32) {
      const double* a = static_cast<const double*>(v.val);
      for (int64_t q = 0; q < v.nnz; ++q)
        if (!(std::fabs(a[q]) <= 3.4028234663852886e38)) {
          set_error("batch FP32 form: a value of matrix " + std::to_string(m) + " is not finite in FP32");
          return nullptr;
        }
    } else if (o.precision == kPrecDF32) {
      const double* a = static_cast<const double*>(v.val);
      for (int64_t q = 0; q < v.nnz; ++q)
        if (!df32_range_ok(a[q])) {
          set_error("batch DF32 form: a value of matrix " + std::to_string(m) + " lies outside [2^-40, 2^41)");
          return nullptr;
        }
    }
    p->row_off[(size_t)m + 1] = p->row_off[(size_t)m] + v.n_rows;
    p->col_off[(size_t)m + 1] = p->col_off[(size_t)m] + v.n_cols;
    p->nnz += v.nnz;
  }
  p->n_rows = p->row_off[(size_t)n];
  p->n_cols = p->col_off[(size_t)n];
  BatchSource src;
  make_source(n, mats, &src);
  if (k == 1 && o.k1_layout == 0) {
    if (!build_k1(p.get(), src, o)) return nullptr;
    return p;
  }

  TuneChoice choice;
  choice.lanes = o.lanes > 0 ? o.lanes : std::min(k, 32);
  if (o.lanes == 0 && k >= 8) choice.lanes = k / 4;  // four right-hand sides per lane
  if (o.long_row_len > 0) choice.long_len = o.long_row_len;
  if (o.warps_per_block > 0) choice.wpb = o.warps_per_block;
  if (o.unroll > 0) choice.deep = o.unroll - 1;
  bool fresh = false;  // layout tuned here: the dispatch is then decided on the whole batch
  std::string key;
  if (o.autotune) {
    key = tune_key(src, k, o.precision);
    bool hit = false;
    if (o.lanes == 0 && o.long_row_len == 0 && o.warps_per_block == 0 && o.unroll == 0 &&
        o.dispatch == 0) {
      std::lock_guard<std::mutex> g(g_tune_mu);
      auto it = tune_cache().find(key);
      if (it != tune_cache().end()) {
        choice = it->second;
        hit = true;
      } else if (cache_file_lookup(key, &choice)) {
        tune_cache()[key] = choice;
        hit = batch_supported(k, choice.lanes);
      }
    }
    if (!hit) {
      if (!autotune(src, k, o.precision, &o, &p->tuning)) return nullptr;
      choice = p->tuning.cand[(size_t)p->tuning.best];
      fresh = true;
    }
  }
  p->prm.lanes = choice.lanes;
  p->prm.long_len = choice.long_len;
  p->prm.chunk = o.chunk > 0 ? o.chunk : choice.long_len;
  if (o.window_rows > 0) p->prm.window_rows = o.window_rows;
  if (o.max_steps > 0) p->prm.max_steps = o.max_steps;
  std::vector<int> all((size_t)n);
  for (int m = 0; m < n; ++m) all[(size_t)m] = m;
  BatchHost* h = build_host(src, all, k, p->prm);
  if (!h) {
    set_error("batch: more than 2^31 rows, columns or layout entries");
    return nullptr;
  }
  const bool ok = upload_batch(h, k, o.precision, choice.wpb, choice.deep, &p->d);
  if (ok && fresh && o.dispatch == 0) {
    // The sample the layout was tuned on holds a fraction of the batch, so
    // how far the persistent warps' drift spreads the rows of X they gather
    // shows only on the whole batch: time both dispatches on it.
    if (!whole_batch_dispatch(p->d.m, p->n_rows, p->n_cols, k, &choice.per_task)) {
      batch_free(h);
      return nullptr;
    }
  }
  if (fresh && o.lanes == 0 && o.long_row_len == 0 && o.warps_per_block == 0 && o.unroll == 0 &&
      o.dispatch == 0) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    tune_cache()[key] = choice;
    cache_file_store(key, choice);
  }
  p->d.m.per_task = o.dispatch == 0 ? choice.per_task : o.dispatch == 2;
  if (ok) plan_parts(p.get(), batch_view(h), o.host_parts > 0 ? o.host_parts : 8);
  batch_free(h);
  if (!ok) return nullptr;
  return p;
}

bool batch_offsets(const Plan* p, int64_t* row_off, int64_t* col_off) {
  if (!p || p->kind != PlanKind::kBatch) return false;
  const auto* b = static_cast<const BatchPlan*>(p);
  if (row_off) std::copy(b->row_off.begin(), b->row_off.end(), row_off);
  if (col_off) std::copy(b->col_off.begin(), b->col_off.end(), col_off);
  return true;
}

int batch_size(const Plan* p) {
  if (!p || p->kind != PlanKind::kBatch) return 0;
  return (int)static_cast<const BatchPlan*>(p)->row_off.size() - 1;
}

int batch_tuning(const Plan* p, int* configs, float* ms, int cap, int* best) {
  if (!p || p->kind != PlanKind::kBatch) return -1;
  const TuneRun& t = static_cast<const BatchPlan*>(p)->tuning;
  const int n = (int)t.cand.size();
  for (int i = 0; i < n && i < cap; ++i) {
    if (configs) {
      configs[4 * i] = t.cand[(size_t)i].lanes;
      configs[4 * i + 1] = t.cand[(size_t)i].long_len;
      configs[4 * i + 2] = t.cand[(size_t)i].wpb;
      configs[4 * i + 3] = t.cand[(size_t)i].deep;
    }
    if (ms) ms[i] = t.ms[(size_t)i];
  }
  if (best) *best = t.best;
  return n;
}

}  // namespace vnec
