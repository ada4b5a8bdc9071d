// Host builder of the batched multi-right-hand-side layout (batch.h).
//
// The batch of matrices is laid out as its block-diagonal concatenation.
// Within windows of `window_rows` global rows, rows are split into empty rows
// (ZERO tasks of up to 32 rows), grouped rows (len <= long_len) sorted by
// length, and long rows cut into chunks of `chunk` entries.  A warp reads
// S = 32 / lanes (value, column) slots per step.  Grouped rows are packed
// G = S / V to a task, V = 2^vwl slots per row, V the smallest power of two
// (<= S) that keeps the group's longest row within max_steps steps; entry j
// of row g sits at base + (j / V) * S + g * V + j % V.  A chunk uses all S
// slots (entry j at base + j).  Padding entries carry value 0 and a column of
// their own row, whose x row the lane has already read.

#include <omp.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "batch.h"

namespace vnec {

struct BatchHost {
  int64_t n_rows = 0, n_cols = 0, nnz = 0, entries = 0, n_rowid = 0, num_long = 0, num_chunks = 0;
  int lanes = 1;
  std::vector<int64_t> win_task, win_entry;
  std::vector<SlicedTask> tasks;
  std::unique_ptr<double[]> val;
  std::unique_ptr<int32_t[]> col;
  std::vector<int32_t> rowid, long_row, long_first, chunk_long;
};

namespace {

inline int meta(int kind, int vwl, int nrows) { return kind | (vwl << 4) | (nrows << 8); }

// Smallest vwl (V = 2^vwl <= 2^max_vwl) with ceil(len / V) <= max_steps.
inline int vwl_for(int64_t len, int max_steps, int max_vwl) {
  int l = 0;
  while (l < max_vwl && ((len + (1 << l) - 1) >> l) > max_steps) ++l;
  return l;
}

struct Window {
  std::vector<SlicedTask> tasks;  // base / row_base relative to the window
  std::vector<int32_t> rowid;
  std::vector<int32_t> long_row;
  std::vector<int32_t> long_nchunks;
  int64_t entries = 0, chunks = 0;
};

// Where global row r of the concatenation comes from.
struct Source {
  int n;
  const int64_t* row_off;  // n + 1
  const int64_t* col_off;  // n
  const int64_t* const* rp;
  const int32_t* const* ci;
  const double* const* val;
  int matrix_of(int64_t r) const {
    return (int)(std::upper_bound(row_off, row_off + n + 1, r) - row_off) - 1;
  }
};

}  // namespace

BatchHost* batch_build(int n, const int64_t* n_rows, const int64_t* n_cols, const int64_t* const* row_ptr,
                       const int32_t* const* col, const double* const* val, int k, const BatchParams& prm) {
  const int L = prm.lanes > 0 ? prm.lanes : std::min(k, 32);
  if (!batch_supported(k, L) || prm.long_len < 1 || prm.chunk < 1 || prm.window_rows < 1 || prm.max_steps < 1)
    return nullptr;
  const int S = 32 / L;  // slots per step
  int max_vwl = 0;
  while ((2 << max_vwl) <= S) ++max_vwl;
  std::vector<int64_t> row_off((size_t)n + 1, 0), col_off((size_t)n, 0);
  int64_t nc = 0, nnz = 0;
  for (int m = 0; m < n; ++m) {
    row_off[m + 1] = row_off[m] + n_rows[m];
    col_off[m] = nc;
    nc += n_cols[m];
    nnz += row_ptr[m][n_rows[m]];
  }
  const int64_t nr = row_off[n];
  if (nr >= ((int64_t)1 << 31) || nc >= ((int64_t)1 << 31)) return nullptr;
  const Source src{n, row_off.data(), col_off.data(), row_ptr, col, val};

  const int64_t W = prm.window_rows;
  const int64_t nwin = (nr + W - 1) / W;
  std::vector<Window> win((size_t)nwin);
  const int64_t chunk = prm.chunk;

  // Pass 1: per window, task list, row slots and entry counts.
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t w = 0; w < nwin; ++w) {
    Window& wd = win[(size_t)w];
    const int64_t r0 = w * W, r1 = std::min(nr, r0 + W);
    std::vector<int32_t> zero, grouped, longr;
    std::vector<int32_t> len((size_t)(r1 - r0));
    int m = src.matrix_of(r0);
    for (int64_t r = r0; r < r1; ++r) {
      while (r >= row_off[m + 1]) ++m;
      const int64_t lr = r - row_off[m];
      const int64_t l = row_ptr[m][lr + 1] - row_ptr[m][lr];
      len[(size_t)(r - r0)] = (int32_t)l;
      if (l == 0)
        zero.push_back((int32_t)r);
      else if (l <= prm.long_len)
        grouped.push_back((int32_t)r);
      else
        longr.push_back((int32_t)r);
    }
    auto L_of = [&](int32_t r) { return len[(size_t)(r - r0)]; };
    std::stable_sort(grouped.begin(), grouped.end(), [&](int32_t a, int32_t b) { return L_of(a) < L_of(b); });
    for (size_t i = 0; i < zero.size(); i += 32) {
      const int c = (int)std::min<size_t>(32, zero.size() - i);
      wd.tasks.push_back(SlicedTask{0, (int32_t)wd.rowid.size(), 0, meta(kSlicedZero, 0, c)});
      for (int q = 0; q < c; ++q) wd.rowid.push_back(zero[i + q]);
    }
    size_t i = 0;
    while (i < grouped.size()) {
      int vwl = vwl_for(L_of(grouped[i]), prm.max_steps, max_vwl);
      size_t c = std::min<size_t>((size_t)(S >> vwl), grouped.size() - i);
      // The group's longest row may need a wider V (fewer rows per group).
      while (vwl_for(L_of(grouped[i + c - 1]), prm.max_steps, max_vwl) > vwl) {
        ++vwl;
        c = std::min<size_t>((size_t)(S >> vwl), grouped.size() - i);
      }
      const int64_t V = (int64_t)1 << vwl;
      const int64_t steps = (L_of(grouped[i + c - 1]) + V - 1) / V;
      wd.tasks.push_back(SlicedTask{(int32_t)wd.entries, (int32_t)wd.rowid.size(), (int32_t)steps,
                                    meta(kSlicedRows, vwl, (int)c)});
      for (size_t q = 0; q < c; ++q) wd.rowid.push_back(grouped[i + q]);
      wd.entries += steps * S;
      i += c;
    }
    for (int32_t r : longr) {
      const int64_t l = L_of(r);
      const int64_t nch = (l + chunk - 1) / chunk;
      wd.long_row.push_back(r);
      wd.long_nchunks.push_back((int32_t)nch);
      for (int64_t c = 0; c < nch; ++c) {
        const int64_t clen = std::min<int64_t>(chunk, l - c * chunk);
        const int64_t steps = (clen + S - 1) / S;
        wd.tasks.push_back(
            SlicedTask{(int32_t)wd.entries, (int32_t)(wd.chunks + c), (int32_t)steps, meta(kSlicedChunk, 0, 1)});
        wd.entries += steps * S;
      }
      wd.chunks += nch;
    }
  }

  std::vector<int64_t> off_e(nwin + 1, 0), off_r(nwin + 1, 0), off_t(nwin + 1, 0), off_c(nwin + 1, 0),
      off_l(nwin + 1, 0);
  for (int64_t w = 0; w < nwin; ++w) {
    off_e[w + 1] = off_e[w] + win[w].entries;
    off_r[w + 1] = off_r[w] + (int64_t)win[w].rowid.size();
    off_t[w + 1] = off_t[w] + (int64_t)win[w].tasks.size();
    off_c[w + 1] = off_c[w] + win[w].chunks;
    off_l[w + 1] = off_l[w] + (int64_t)win[w].long_row.size();
  }
  if (off_e[nwin] + 64 >= ((int64_t)1 << 31)) return nullptr;

  auto* h = new BatchHost();
  h->n_rows = nr;
  h->n_cols = nc;
  h->nnz = nnz;
  h->lanes = L;
  h->entries = off_e[nwin];
  h->n_rowid = off_r[nwin];
  h->num_chunks = off_c[nwin];
  h->num_long = off_l[nwin];
  h->win_task = off_t;
  h->win_entry = off_e;
  h->tasks.resize((size_t)off_t[nwin]);
  h->rowid.resize((size_t)off_r[nwin]);
  h->long_row.resize((size_t)off_l[nwin]);
  h->long_first.resize((size_t)off_l[nwin] + 1);
  h->chunk_long.resize((size_t)off_c[nwin]);
  const int64_t pad = 64;
  h->val.reset(new double[(size_t)(h->entries + pad)]);
  h->col.reset(new int32_t[(size_t)(h->entries + pad)]);
  std::fill(h->val.get() + h->entries, h->val.get() + h->entries + pad, 0.0);
  std::fill(h->col.get() + h->entries, h->col.get() + h->entries + pad, 0);

  // Pass 2: global task list and the interleaved entries.
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t w = 0; w < nwin; ++w) {
    Window& wd = win[(size_t)w];
    std::copy(wd.rowid.begin(), wd.rowid.end(), h->rowid.begin() + off_r[w]);
    int64_t lc = off_c[w];
    for (size_t q = 0; q < wd.long_row.size(); ++q) {
      const int64_t li = off_l[w] + (int64_t)q;
      h->long_row[(size_t)li] = wd.long_row[q];
      h->long_first[(size_t)li] = (int32_t)lc;
      for (int32_t c = 0; c < wd.long_nchunks[q]; ++c) h->chunk_long[(size_t)(lc + c)] = (int32_t)li;
      lc += wd.long_nchunks[q];
    }
    // Source arrays of global row r.
    auto row = [&](int32_t r, const int32_t** cp, const double** vp, int64_t* len, int32_t* coff) {
      const int m = src.matrix_of(r);
      const int64_t lr = r - row_off[m];
      const int64_t b = row_ptr[m][lr];
      *cp = col[m] + b;
      *vp = val[m] + b;
      *len = row_ptr[m][lr + 1] - b;
      *coff = (int32_t)col_off[m];
    };
    size_t li = 0;
    int64_t chunk_in_row = 0;
    for (size_t ti = 0; ti < wd.tasks.size(); ++ti) {
      SlicedTask t = wd.tasks[ti];
      const int kind = t.meta & 15, vwl = (t.meta >> 4) & 15, nrows = t.meta >> 8;
      if (kind != kSlicedZero) t.base += (int32_t)off_e[w];
      t.row_base += (int32_t)(kind == kSlicedChunk ? off_c[w] : off_r[w]);
      h->tasks[(size_t)(off_t[w] + (int64_t)ti)] = t;
      if (kind == kSlicedZero) continue;
      const int64_t span = (int64_t)t.steps * S;
      double* vdst = h->val.get() + t.base;
      int32_t* cdst = h->col.get() + t.base;
      if (kind == kSlicedRows) {
        const int64_t V = (int64_t)1 << vwl;
        const int G = S >> vwl;
        for (int g = 0; g < G; ++g) {
          const int32_t r = h->rowid[(size_t)(t.row_base + (g < nrows ? g : 0))];
          const int32_t* cp;
          const double* vp;
          int64_t len;
          int32_t coff;
          row(r, &cp, &vp, &len, &coff);
          if (g >= nrows) len = 0;
          const int32_t padc = coff + cp[(g < nrows ? len : 1) - 1];
          for (int64_t j = 0; j < t.steps * V; ++j) {
            const int64_t pos = (j / V) * S + g * V + (j % V);
            if (j < len) {
              cdst[pos] = coff + cp[j];
              vdst[pos] = vp[j];
            } else {
              cdst[pos] = padc;
              vdst[pos] = 0.0;
            }
          }
        }
      } else {
        const int32_t r = wd.long_row[li];
        const int32_t* cp;
        const double* vp;
        int64_t len;
        int32_t coff;
        row(r, &cp, &vp, &len, &coff);
        const int64_t lo = chunk_in_row * chunk, hi = std::min<int64_t>(len, lo + chunk);
        for (int64_t j = 0; j < span; ++j) {
          if (lo + j < hi) {
            cdst[j] = coff + cp[lo + j];
            vdst[j] = vp[lo + j];
          } else {
            cdst[j] = coff + cp[hi - 1];
            vdst[j] = 0.0;
          }
        }
        if (++chunk_in_row == wd.long_nchunks[li]) {
          chunk_in_row = 0;
          ++li;
        }
      }
    }
  }
  h->long_first[(size_t)h->num_long] = (int32_t)h->num_chunks;
  return h;
}

void batch_free(BatchHost* h) { delete h; }

BatchHostView batch_view(const BatchHost* h) {
  BatchHostView v;
  v.n_rows = h->n_rows;
  v.n_cols = h->n_cols;
  v.nnz = h->nnz;
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
  v.chunk_long = h->chunk_long.data();
  v.lanes = h->lanes;
  v.num_windows = (int64_t)h->win_task.size() - 1;
  v.win_task = h->win_task.data();
  v.win_entry = h->win_entry.data();
  return v;
}

bool batch_supported(int k, int lanes) {
  if (k < 1 || k > 32 || lanes < 1 || lanes > 32) return false;
  if (32 % lanes != 0 || k % lanes != 0) return false;
  const int r = k / lanes;
  return r == 1 || r == 2 || r == 4 || r == 8;
}

}  // namespace vnec
