// Host builder of the sliced row-group format (sliced.h) — the GPU
// re-derivation of Build_VNEC_S (src/operation/src/spmv_vnec_S_for_mxv.c:336-588).
//
// The reference buckets each partition's rows by length, interleaves groups of
// nLanes equal-length rows (<= 32 entries) so that one SIMD lane owns one row
// (:442-585), and handles the other rows one at a time.  Here the unit is a
// warp: within windows of `window_rows` rows, rows are sorted by length and
// packed into groups of G = 32 / VW rows handled by VW lanes each (VW = 1 is
// the reference's cross-row slice with 32 lanes instead of 8), with VW chosen
// so that every lane makes at most `max_steps` loads; rows longer than
// `long_len` become chunks of `chunk` entries summed by a fix-up.  Empty rows
// get zero tasks (the reference writes 0 for them through its length-0
// buckets).  Windows keep the y writes of one group of tasks local.

#include <omp.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "sliced.h"

namespace vnec {

struct SlicedHost {
  int64_t entries = 0, n_rowid = 0, num_long = 0, num_chunks = 0;
  int64_t delta_nnz = 0, delta_rows = 0;  // nonzeros and rows stored with 16-bit column deltas
  int vpe = 1;
  std::vector<int64_t> win_task, win_long, win_entry;  // per-window offsets (windows + 1)
  std::vector<SlicedTask> tasks;
  std::unique_ptr<unsigned char[]> val;
  std::unique_ptr<int32_t[]> col;
  std::vector<int32_t> rowid, long_row, long_first;
  std::unique_ptr<uint16_t[]> col16;  // delta16 layouts only
  std::vector<int32_t> first;
  std::unique_ptr<uint16_t[]> pat16;  // shared-pattern deltas (delta16 + shared layouts)
  int64_t shared_nnz = 0, shared_steps = 0;
};

namespace {

struct Window {
  std::vector<SlicedTask> tasks;  // base / row_base relative to the window
  std::vector<int32_t> rowid;
  std::vector<int32_t> long_row;
  std::vector<int32_t> long_nchunks;
  int64_t entries = 0;
  int64_t chunks = 0;
  // group rows in fill order: (row, steps, vw_log2) per task for the fill pass
  std::vector<int32_t> order;
};

inline int vw_log2_for(int64_t len, int max_steps) {
  int l = 0;
  while (l < 5 && ((len + (1 << l) - 1) >> l) > max_steps) ++l;
  return l;
}

inline int meta(int kind, int vwl, int nrows) { return kind | (vwl << 4) | (nrows << 8); }

}  // namespace

SlicedHost* sliced_build(int64_t n_rows, int64_t /*n_cols*/, const int64_t* rp, const uint64_t* rp64, const int32_t* ci,
                         const uint64_t* ci64, const void* val, int vb, const SlicedParams& prm, int vpe,
                         const uint8_t* keep) {
  // Each entry carries `vpe` consecutive values (1 for single nonzeros, the
  // block width for dense blocks); `vb` is the size of one value.
  const int eb = vb * vpe;
  auto begin = [&](int64_t r) -> int64_t { return rp ? rp[r] : (int64_t)rp64[r]; };
  auto colat = [&](int64_t p) -> int32_t { return ci ? ci[p] : (int32_t)ci64[p]; };
  const int64_t W = prm.window_rows;
  const int64_t nwin = (n_rows + W - 1) / W;
  std::vector<Window> win((size_t)nwin);

  // Pass 1: per window, task list, row slots and entry counts.
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t w = 0; w < nwin; ++w) {
    Window& wd = win[(size_t)w];
    const int64_t r0 = w * W, r1 = std::min(n_rows, r0 + W);
    std::vector<int32_t> zero, grouped, longr;
    for (int64_t r = r0; r < r1; ++r) {
      if (keep && !keep[r]) continue;
      const int64_t len = begin(r + 1) - begin(r);
      if (len == 0)
        zero.push_back((int32_t)r);
      else if (len <= prm.long_len)
        grouped.push_back((int32_t)r);
      else
        longr.push_back((int32_t)r);
    }
    std::stable_sort(grouped.begin(), grouped.end(), [&](int32_t a, int32_t b) {
      const int64_t la = begin(a + 1) - begin(a), lb = begin(b + 1) - begin(b);
      if (la != lb) return la < lb;
      return prm.row_key && prm.row_key[a] < prm.row_key[b];
    });
    for (size_t i = 0; i < zero.size(); i += 32) {
      const int n = (int)std::min<size_t>(32, zero.size() - i);
      wd.tasks.push_back(SlicedTask{0, (int32_t)wd.rowid.size(), 0, meta(kSlicedZero, 0, n)});
      for (int k = 0; k < n; ++k) wd.rowid.push_back(zero[i + k]);
    }
    size_t i = 0;
    while (i < grouped.size()) {
      const int64_t len0 = begin(grouped[i] + 1) - begin(grouped[i]);
      int vwl = vw_log2_for(len0, prm.max_steps);
      size_t g = (size_t)32 >> vwl;
      size_t n = std::min(g, grouped.size() - i);
      int64_t maxlen = begin(grouped[i + n - 1] + 1) - begin(grouped[i + n - 1]);
      // The group's longest row may need a wider VW (fewer rows per group).
      while (vw_log2_for(maxlen, prm.max_steps) > vwl) {
        ++vwl;
        g = (size_t)32 >> vwl;
        n = std::min(g, grouped.size() - i);
        maxlen = begin(grouped[i + n - 1] + 1) - begin(grouped[i + n - 1]);
      }
      const int64_t vw = (int64_t)1 << vwl;
      const int64_t steps = (maxlen + vw - 1) / vw;
      wd.tasks.push_back(SlicedTask{(int32_t)wd.entries, (int32_t)wd.rowid.size(), (int32_t)steps,
                                    meta(kSlicedRows, vwl, (int)n)});
      for (size_t k = 0; k < n; ++k) wd.rowid.push_back(grouped[i + k]);
      wd.entries += steps * 32;
      i += n;
    }
    for (int32_t r : longr) {
      const int64_t len = begin(r + 1) - begin(r);
      const int64_t nch = (len + prm.chunk - 1) / prm.chunk;
      wd.long_row.push_back(r);
      wd.long_nchunks.push_back((int32_t)nch);
      for (int64_t c = 0; c < nch; ++c) {
        const int64_t clen = std::min<int64_t>(prm.chunk, len - c * prm.chunk);
        const int64_t steps = (clen + 31) / 32;
        wd.tasks.push_back(SlicedTask{(int32_t)wd.entries, (int32_t)(wd.chunks + c), (int32_t)steps,
                                      meta(kSlicedChunk, 5, 1)});
        wd.entries += steps * 32;
      }
      wd.chunks += nch;
    }
  }

  // Offsets across windows.
  std::vector<int64_t> off_e(nwin + 1, 0), off_r(nwin + 1, 0), off_t(nwin + 1, 0), off_c(nwin + 1, 0),
      off_l(nwin + 1, 0);
  for (int64_t w = 0; w < nwin; ++w) {
    off_e[w + 1] = off_e[w] + win[w].entries;
    off_r[w + 1] = off_r[w] + (int64_t)win[w].rowid.size();
    off_t[w + 1] = off_t[w] + (int64_t)win[w].tasks.size();
    off_c[w + 1] = off_c[w] + win[w].chunks;
    off_l[w + 1] = off_l[w] + (int64_t)win[w].long_row.size();
  }
  if (off_e[nwin] >= ((int64_t)1 << 31) || off_r[nwin] >= ((int64_t)1 << 31)) return nullptr;

  auto* h = new SlicedHost();
  h->entries = off_e[nwin];
  h->n_rowid = off_r[nwin];
  h->num_chunks = off_c[nwin];
  h->num_long = off_l[nwin];
  h->win_task = off_t;
  h->win_long = off_l;
  h->win_entry = off_e;
  h->tasks.resize((size_t)off_t[nwin]);
  h->rowid.resize((size_t)off_r[nwin]);
  h->long_row.resize((size_t)off_l[nwin]);
  h->long_first.resize((size_t)off_l[nwin] + 1);
  const int64_t pad = 64;
  h->val.reset(new unsigned char[(size_t)(h->entries + pad) * eb]);
  h->col.reset(new int32_t[(size_t)(h->entries + pad)]);
  h->vpe = vpe;
  std::memset(h->val.get() + (size_t)h->entries * eb, 0, (size_t)pad * eb);
  std::memset(h->col.get() + h->entries, 0, sizeof(int32_t) * pad);
  if (prm.delta16) {
    h->col16.reset(new uint16_t[(size_t)(h->entries + pad)]);
    std::memset(h->col16.get(), 0, sizeof(uint16_t) * (size_t)(h->entries + pad));
    h->first.assign((size_t)std::max<int64_t>(h->n_rowid, 1), 0);
    if (prm.shared) {
      const size_t np = (size_t)(h->entries / 32 + pad);
      h->pat16.reset(new uint16_t[np]);
      std::memset(h->pat16.get(), 0, sizeof(uint16_t) * np);
    }
  }

  // Pass 2: global task list and the interleaved entries.
  std::vector<int64_t> win_dnnz((size_t)nwin, 0), win_drows((size_t)nwin, 0);
  std::vector<int64_t> win_snnz((size_t)nwin, 0), win_ssteps((size_t)nwin, 0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t w = 0; w < nwin; ++w) {
    Window& wd = win[(size_t)w];
    std::copy(wd.rowid.begin(), wd.rowid.end(), h->rowid.begin() + off_r[w]);
    int64_t lc = off_c[w];
    for (size_t k = 0; k < wd.long_row.size(); ++k) {
      h->long_row[(size_t)(off_l[w] + (int64_t)k)] = wd.long_row[k];
      h->long_first[(size_t)(off_l[w] + (int64_t)k)] = (int32_t)lc;
      lc += wd.long_nchunks[k];
    }
    size_t li = 0;          // long-row cursor within the window
    int64_t chunk_in_row = 0;
    for (size_t ti = 0; ti < wd.tasks.size(); ++ti) {
      SlicedTask t = wd.tasks[ti];
      const int kind = t.meta & 15, vwl = (t.meta >> 4) & 15, nrows = (t.meta >> 8) & 0xff;
      if (kind != kSlicedZero) t.base += (int32_t)off_e[w];
      if (kind == kSlicedChunk)
        t.row_base += (int32_t)off_c[w];
      else
        t.row_base += (int32_t)off_r[w];
      h->tasks[(size_t)(off_t[w] + (int64_t)ti)] = t;
      if (kind == kSlicedZero) continue;
      const int64_t vw = (int64_t)1 << vwl;
      const int64_t span = (int64_t)t.steps * 32;
      unsigned char* vdst = h->val.get() + (size_t)t.base * eb;
      int32_t* cdst = h->col.get() + t.base;
      std::memset(vdst, 0, (size_t)span * eb);
      if (kind == kSlicedRows) {
        const int32_t pad_col = 0;
        for (int64_t e = 0; e < span; ++e) cdst[e] = pad_col;
        for (int g = 0; g < nrows; ++g) {
          const int32_t r = h->rowid[(size_t)(t.row_base + g)];
          const int64_t b = begin(r), len = begin(r + 1) - b;
          for (int64_t j = 0; j < len; ++j) {
            const int64_t pos = (j >> vwl) * 32 + g * vw + (j & (vw - 1));
            cdst[pos] = colat(b + j);
            std::memcpy(vdst + pos * eb, static_cast<const unsigned char*>(val) + (b + j) * eb, (size_t)eb);
          }
        }
        // 16-bit deltas when every row of the group has increasing columns
        // whose gaps fit (VW = 1 groups only: one lane walks one row).
        bool delta_ok = prm.delta16 && vwl == 0;
        for (int g = 0; g < nrows && delta_ok; ++g) {
          const int32_t r = h->rowid[(size_t)(t.row_base + g)];
          for (int64_t q = begin(r) + 1; q < begin(r + 1); ++q) {
            const int64_t d = (int64_t)colat(q) - colat(q - 1);
            if (d <= 0 || d > 65535) {
              delta_ok = false;
              break;
            }
          }
        }
        if (delta_ok) {
          uint16_t* ddst = h->col16.get() + t.base;
          for (int g = 0; g < nrows; ++g) {
            const int32_t r = h->rowid[(size_t)(t.row_base + g)];
            const int64_t b = begin(r), len = begin(r + 1) - b;
            h->first[(size_t)(t.row_base + g)] = colat(b);
            for (int64_t j = 1; j < len; ++j) ddst[j * 32 + g] = (uint16_t)(colat(b + j) - colat(b + j - 1));
            win_dnnz[(size_t)w] += len;
          }
          win_drows[(size_t)w] += nrows;
          int meta = kSlicedDelta;
          // Shared pattern: every row has `steps` entries and the first row's
          // deltas (at most 32 steps: one lane per step holds the pattern).
          bool shared = h->pat16 && nrows > 0 && t.steps <= 32 && t.base % 32 == 0;
          const int64_t b0 = shared ? begin(h->rowid[(size_t)t.row_base]) : 0;
          for (int g = 0; g < nrows && shared; ++g) {
            const int64_t b = begin(h->rowid[(size_t)(t.row_base + g)]);
            if (begin(h->rowid[(size_t)(t.row_base + g)] + 1) - b != t.steps) {
              shared = false;
              break;
            }
            for (int64_t j = 1; j < t.steps; ++j)
              if (colat(b + j) - colat(b + j - 1) != colat(b0 + j) - colat(b0 + j - 1)) {
                shared = false;
                break;
              }
          }
          if (shared) {
            uint16_t* pd = h->pat16.get() + t.base / 32;
            for (int64_t j = 1; j < t.steps; ++j) pd[j] = (uint16_t)(colat(b0 + j) - colat(b0 + j - 1));
            win_snnz[(size_t)w] += (int64_t)nrows * t.steps;
            win_ssteps[(size_t)w] += t.steps;
            meta |= kSlicedShared;
          }
          h->tasks[(size_t)(off_t[w] + (int64_t)ti)].meta |= meta;
        }
      } else {  // chunk of a long row
        const int32_t r = wd.long_row[li];
        const int64_t b = begin(r), len = begin(r + 1) - b;
        const int64_t lo = chunk_in_row * (int64_t)prm.chunk, hi = std::min<int64_t>(len, lo + prm.chunk);
        for (int64_t e = 0; e < span; ++e) cdst[e] = colat(b + lo);
        for (int64_t j = lo; j < hi; ++j) {
          cdst[j - lo] = colat(b + j);
          std::memcpy(vdst + (j - lo) * eb, static_cast<const unsigned char*>(val) + (b + j) * eb, (size_t)eb);
        }
        if (++chunk_in_row == wd.long_nchunks[li]) {
          chunk_in_row = 0;
          ++li;
        }
      }
    }
  }
  h->long_first[(size_t)h->num_long] = (int32_t)h->num_chunks;
  for (int64_t w = 0; w < nwin; ++w) {
    h->delta_nnz += win_dnnz[(size_t)w];
    h->delta_rows += win_drows[(size_t)w];
    h->shared_nnz += win_snnz[(size_t)w];
    h->shared_steps += win_ssteps[(size_t)w];
  }
  return h;
}

void sliced_free(SlicedHost* h) { delete h; }

SlicedHostView sliced_view(const SlicedHost* h) {
  SlicedHostView v;
  v.entries = h->entries;
  v.num_tasks = (int64_t)h->tasks.size();
  v.num_long = h->num_long;
  v.num_chunks = h->num_chunks;
  v.n_rowid = h->n_rowid;
  v.tasks = h->tasks.data();
  v.val = h->val.get();
  v.col = h->col.get();
  v.rowid = h->rowid.data();
  v.long_row = h->long_row.data();
  v.long_first = h->long_first.data();
  v.vpe = h->vpe;
  v.col16 = h->col16.get();
  v.first = h->first.empty() ? nullptr : h->first.data();
  v.num_windows = (int64_t)h->win_task.size() - 1;
  v.win_task = h->win_task.data();
  v.win_long = h->win_long.data();
  v.win_entry = h->win_entry.data();
  v.delta_nnz = h->delta_nnz;
  v.delta_rows = h->delta_rows;
  v.pat16 = h->pat16.get();
  v.shared_nnz = h->shared_nnz;
  v.shared_steps = h->shared_steps;
  return v;
}

}  // namespace vnec
