// Seeded synthetic sparse-matrix generators (host side, OpenMP).
//
// Every generator is a pure function of its arguments: values and column
// patterns come from a counter-based hash (splitmix64 finaliser), so the result
// does not depend on the number of OpenMP threads.  Rows are emitted in CSR
// order with strictly increasing column indices inside each row, which is the
// layout the reference's CSR builder produces (qsort of (row, col) triples,
// src/core/src/SpB_Matrix_CSC_or_CSR.c:188-256) and the layout its VNEC
// builders assume (they walk each row's columns in ascending order,
// src/operation/src/spmv_vnec_D_for_mxv.c:359-392).
//
// Index widths: int64 row offsets (nnz may exceed 2^31), int32 columns.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <unordered_set>
#include <vector>
#include <omp.h>

namespace {

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;

inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Hash of (seed, stream, index): independent streams for patterns and values.
inline uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(mix64(seed * kGolden + stream * 0xD1B54A32D192ED03ull + 0x632BE59BD9B4E019ull) + i * kGolden);
}

// Uniform double in [0, 1) with 53 random bits.
inline double u01(uint64_t h) { return (double)(h >> 11) * 0x1.0p-53; }

// A splitmix64 sequence seeded from (seed, stream, row): one per row.
struct RowRng {
  uint64_t s;
  RowRng(uint64_t seed, uint64_t stream, uint64_t row) : s(hash3(seed, stream, row)) {}
  uint64_t next() { s += kGolden; return mix64(s); }
  // Integer in [0, bound): multiply-high (bias below 2^-32 for bound < 2^32).
  uint64_t below(uint64_t bound) { return (uint64_t)(((unsigned __int128)next() * bound) >> 64); }
};

struct HostCSR {
  int64_t n_rows = 0, n_cols = 0, nnz = 0;
  std::unique_ptr<int64_t[]> row_ptr;
  std::unique_ptr<int32_t[]> col;
  std::unique_ptr<double[]> val;
  void alloc(int64_t rows, int64_t cols, int64_t nz) {
    n_rows = rows; n_cols = cols; nnz = nz;
    row_ptr.reset(new int64_t[rows + 1]);
    // +16 elements of padding so that vectorised readers may touch the tail.
    col.reset(new int32_t[nz + 16]);
    val.reset(new double[nz + 16]);
    std::memset(col.get() + nz, 0, 16 * sizeof(int32_t));
    std::memset(val.get() + nz, 0, 16 * sizeof(double));
  }
};

// Exclusive prefix sum of per-row counts into row_ptr (row_ptr[0] = 0).
void prefix_rows(const int64_t* counts, int64_t n, int64_t* row_ptr) {
  row_ptr[0] = 0;
  for (int64_t r = 0; r < n; ++r) row_ptr[r + 1] = row_ptr[r] + counts[r];
}

// k distinct columns of [0, n_cols) in ascending order (Floyd's sampling).
void sample_distinct_sorted(RowRng& rng, int64_t n_cols, int64_t k, int32_t* out) {
  if (k <= 0) return;
  if (k >= n_cols) {
    for (int64_t j = 0; j < n_cols; ++j) out[j] = (int32_t)j;
    return;
  }
  int64_t m = 0;
  if (k <= 64) {
    for (int64_t j = n_cols - k; j < n_cols; ++j) {
      int32_t t = (int32_t)rng.below((uint64_t)j + 1);
      bool seen = false;
      for (int64_t q = 0; q < m; ++q) if (out[q] == t) { seen = true; break; }
      out[m++] = seen ? (int32_t)j : t;
    }
  } else if (2 * k > n_cols) {
    // Dense selection: Knuth's selection sampling over all columns.
    int64_t need = k;
    for (int64_t j = 0; j < n_cols && need > 0; ++j) {
      uint64_t left = (uint64_t)(n_cols - j);
      if (rng.below(left) < (uint64_t)need) { out[m++] = (int32_t)j; --need; }
    }
    return;  // already ascending
  } else {
    std::unordered_set<int32_t> set;
    set.reserve((size_t)k * 2);
    for (int64_t j = n_cols - k; j < n_cols; ++j) {
      int32_t t = (int32_t)rng.below((uint64_t)j + 1);
      int32_t v = set.count(t) ? (int32_t)j : t;
      set.insert(v);
      out[m++] = v;
    }
  }
  std::sort(out, out + m);
}

void fill_values(HostCSR& m, uint64_t seed, double lo, double hi) {
  const double w = hi - lo;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m.nnz; ++i) m.val[i] = lo + w * u01(hash3(seed, 2, (uint64_t)i));
}

// Stable parallel LSD radix sort of 64-bit keys over the low `bits` bits.
// Chunking is over a fixed number of slices, so the result is independent of
// the thread count.  Returns the buffer that holds the sorted keys.
uint64_t* radix_sort_u64(uint64_t* a, uint64_t* tmp, int64_t n, int bits) {
  constexpr int kDigit = 11;
  constexpr int kRadix = 1 << kDigit;
  const int slices = 64;
  std::vector<int64_t> hist((size_t)slices * kRadix);
  const int passes = (bits + kDigit - 1) / kDigit;
  for (int p = 0; p < passes; ++p) {
    const int shift = p * kDigit;
    std::fill(hist.begin(), hist.end(), 0);
#pragma omp parallel for schedule(static)
    for (int s = 0; s < slices; ++s) {
      int64_t lo = n * s / slices, hi = n * (s + 1) / slices;
      int64_t* h = hist.data() + (size_t)s * kRadix;
      for (int64_t i = lo; i < hi; ++i) h[(a[i] >> shift) & (kRadix - 1)]++;
    }
    int64_t run = 0;
    for (int d = 0; d < kRadix; ++d)
      for (int s = 0; s < slices; ++s) {
        int64_t c = hist[(size_t)s * kRadix + d];
        hist[(size_t)s * kRadix + d] = run;
        run += c;
      }
#pragma omp parallel for schedule(static)
    for (int s = 0; s < slices; ++s) {
      int64_t lo = n * s / slices, hi = n * (s + 1) / slices;
      int64_t* h = hist.data() + (size_t)s * kRadix;
      for (int64_t i = lo; i < hi; ++i) tmp[h[(a[i] >> shift) & (kRadix - 1)]++] = a[i];
    }
    std::swap(a, tmp);
  }
  return a;
}

}  // namespace

extern "C" {

// n_rows x n_cols, exactly k distinct uniformly random sorted columns per row,
// values U(lo, hi).
void* vnec_gen_uniform_k(int64_t n_rows, int64_t n_cols, int32_t k, double lo, double hi, uint64_t seed) {
  if (n_rows < 0 || n_cols <= 0 || k < 0 || k > n_cols) return nullptr;
  auto* m = new HostCSR();
  m->alloc(n_rows, n_cols, n_rows * (int64_t)k);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r <= n_rows; ++r) m->row_ptr[r] = r * (int64_t)k;
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n_rows; ++r) {
    RowRng rng(seed, 1, (uint64_t)r);
    sample_distinct_sorted(rng, n_cols, k, m->col.get() + r * (int64_t)k);
  }
  fill_values(*m, seed, lo, hi);
  return m;
}

// R-MAT (recursive matrix) graph with 2^scale rows/cols and n_edges generated
// edges with quadrant probabilities (a, b, c, 1-a-b-c); duplicate edges are
// merged (one stored entry per distinct (row, col)); self-loops are kept.
// Vertex labels are not permuted.  Values U(lo, hi).
void* vnec_gen_rmat(int32_t scale, int64_t n_edges, double a, double b, double c, double lo, double hi,
                    uint64_t seed) {
  if (scale < 1 || scale > 30 || n_edges < 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return nullptr;
  const int64_t n = (int64_t)1 << scale;
  const double k32 = 4294967296.0;
  const uint64_t ta = (uint64_t)std::floor(a * k32);
  const uint64_t tab = (uint64_t)std::floor((a + b) * k32);
  const uint64_t tabc = (uint64_t)std::floor((a + b + c) * k32);
  std::unique_ptr<uint64_t[]> keys(new uint64_t[n_edges > 0 ? n_edges : 1]);
  std::unique_ptr<uint64_t[]> tmp(new uint64_t[n_edges > 0 ? n_edges : 1]);
  const int hashes_per_edge = (scale + 1) / 2;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < n_edges; ++e) {
    uint64_t r = 0, cc = 0, h = 0;
    for (int l = 0; l < scale; ++l) {
      if ((l & 1) == 0) h = hash3(seed, 1, (uint64_t)e * hashes_per_edge + (uint64_t)(l >> 1));
      uint64_t u = (l & 1) ? (h >> 32) : (h & 0xFFFFFFFFull);
      uint64_t rb = u >= tab, cb = (u >= ta && u < tab) || u >= tabc;
      r = (r << 1) | rb;
      cc = (cc << 1) | cb;
    }
    keys[e] = (r << scale) | cc;
  }
  uint64_t* sorted = radix_sort_u64(keys.get(), tmp.get(), n_edges, 2 * scale);
  uint64_t* other = (sorted == keys.get()) ? tmp.get() : keys.get();
  // Parallel de-duplication: mark first occurrences per slice, then compact.
  const int slices = 64;
  std::vector<int64_t> cnt(slices + 1, 0);
#pragma omp parallel for schedule(static)
  for (int s = 0; s < slices; ++s) {
    int64_t b0 = n_edges * s / slices, b1 = n_edges * (s + 1) / slices, k = 0;
    for (int64_t i = b0; i < b1; ++i) k += (i == 0 || sorted[i] != sorted[i - 1]);
    cnt[s + 1] = k;
  }
  for (int s = 0; s < slices; ++s) cnt[s + 1] += cnt[s];
#pragma omp parallel for schedule(static)
  for (int s = 0; s < slices; ++s) {
    int64_t b0 = n_edges * s / slices, b1 = n_edges * (s + 1) / slices, o = cnt[s];
    for (int64_t i = b0; i < b1; ++i)
      if (i == 0 || sorted[i] != sorted[i - 1]) other[o++] = sorted[i];
  }
  const int64_t nnz = cnt[slices];
  auto* m = new HostCSR();
  m->alloc(n, n, nnz);
  const uint64_t cmask = ((uint64_t)1 << scale) - 1;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nnz; ++i) m->col[i] = (int32_t)(other[i] & cmask);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r <= n; ++r) {
    uint64_t key = (uint64_t)r << scale;
    m->row_ptr[r] = (int64_t)(std::lower_bound(other, other + nnz, key) - other);
  }
  fill_values(*m, seed, lo, hi);
  return m;
}

// 27-point stencil on a g x g x g grid (row = (z*g + y)*g + x), off-diagonal
// values U(-1, 0], diagonal = 1 + sum of |off-diagonal| (diagonally dominant).
void* vnec_gen_stencil27(int32_t g, uint64_t seed) {
  if (g < 1 || (int64_t)g * g * g >= ((int64_t)1 << 31)) return nullptr;
  const int64_t n = (int64_t)g * g * g;
  auto span = [g](int64_t i) -> int64_t { return 1 + (i > 0) + (i < g - 1); };
  const int64_t nnz = (int64_t)std::pow((double)(3 * (int64_t)g - 2), 3.0) + 0.5;
  auto* m = new HostCSR();
  m->alloc(n, n, nnz);
  {
    std::unique_ptr<int64_t[]> cnt(new int64_t[n]);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; ++r) {
      int64_t x = r % g, y = (r / g) % g, z = r / ((int64_t)g * g);
      cnt[r] = span(x) * span(y) * span(z);
    }
    prefix_rows(cnt.get(), n, m->row_ptr.get());
  }
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) {
    int64_t x = r % g, y = (r / g) % g, z = r / ((int64_t)g * g);
    int64_t p = m->row_ptr[r], diag_pos = -1;
    double sum_abs = 0.0;
    for (int dz = -1; dz <= 1; ++dz) {
      if (z + dz < 0 || z + dz >= g) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        if (y + dy < 0 || y + dy >= g) continue;
        for (int dx = -1; dx <= 1; ++dx) {
          if (x + dx < 0 || x + dx >= g) continue;
          int64_t c = ((z + dz) * g + (y + dy)) * g + (x + dx);
          m->col[p] = (int32_t)c;
          if (c == r) {
            diag_pos = p;
          } else {
            double v = -u01(hash3(seed, 2, (uint64_t)p));
            m->val[p] = v;
            sum_abs += -v;
          }
          ++p;
        }
      }
    }
    m->val[diag_pos] = 1.0 + sum_abs;
  }
  return m;
}

// Rows with lognormal lengths round(exp(mu + sigma*N(0,1))) clamped to
// [0, min(cap, n_cols)], distinct uniformly random sorted columns, values U(lo, hi).
void* vnec_gen_lognormal(int64_t n_rows, int64_t n_cols, double mu, double sigma, int32_t cap, double lo,
                         double hi, uint64_t seed) {
  if (n_rows < 0 || n_cols <= 0 || cap < 0) return nullptr;
  std::unique_ptr<int64_t[]> cnt(new int64_t[n_rows > 0 ? n_rows : 1]);
  const int64_t kmax = std::min<int64_t>(cap, n_cols);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n_rows; ++r) {
    uint64_t h1 = hash3(seed, 3, 2 * (uint64_t)r), h2 = hash3(seed, 3, 2 * (uint64_t)r + 1);
    double u1 = ((double)(h1 >> 11) + 1.0) * 0x1.0p-53;  // (0, 1]
    double u2 = u01(h2);
    double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    double len = std::floor(std::exp(mu + sigma * z) + 0.5);
    cnt[r] = (int64_t)std::min<double>(std::max<double>(len, 0.0), (double)kmax);
  }
  int64_t nnz = 0;
  for (int64_t r = 0; r < n_rows; ++r) nnz += cnt[r];
  auto* m = new HostCSR();
  m->alloc(n_rows, n_cols, nnz);
  prefix_rows(cnt.get(), n_rows, m->row_ptr.get());
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t r = 0; r < n_rows; ++r) {
    RowRng rng(seed, 1, (uint64_t)r);
    sample_distinct_sorted(rng, n_cols, cnt[r], m->col.get() + m->row_ptr[r]);
  }
  fill_values(*m, seed, lo, hi);
  return m;
}

// Dense band: row r holds every column in [r - bw/2, r + bw/2] that exists.
void* vnec_gen_banded(int64_t n, int32_t bw, double lo, double hi, uint64_t seed) {
  if (n <= 0 || bw < 1) return nullptr;
  const int64_t half = bw / 2;
  std::unique_ptr<int64_t[]> cnt(new int64_t[n]);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) cnt[r] = std::min(n - 1, r + half) - std::max<int64_t>(0, r - half) + 1;
  int64_t nnz = 0;
  for (int64_t r = 0; r < n; ++r) nnz += cnt[r];
  auto* m = new HostCSR();
  m->alloc(n, n, nnz);
  prefix_rows(cnt.get(), n, m->row_ptr.get());
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) {
    int64_t c0 = std::max<int64_t>(0, r - half), p = m->row_ptr[r];
    for (int64_t j = 0; j < cnt[r]; ++j) m->col[p + j] = (int32_t)(c0 + j);
  }
  fill_values(*m, seed, lo, hi);
  return m;
}

// Block diagonal with dense bs x bs blocks (the last block may be smaller).
void* vnec_gen_blockdiag(int64_t n, int32_t bs, double lo, double hi, uint64_t seed) {
  if (n <= 0 || bs < 1) return nullptr;
  std::unique_ptr<int64_t[]> cnt(new int64_t[n]);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) {
    int64_t b0 = (r / bs) * bs;
    cnt[r] = std::min<int64_t>(n, b0 + bs) - b0;
  }
  int64_t nnz = 0;
  for (int64_t r = 0; r < n; ++r) nnz += cnt[r];
  auto* m = new HostCSR();
  m->alloc(n, n, nnz);
  prefix_rows(cnt.get(), n, m->row_ptr.get());
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) {
    int64_t b0 = (r / bs) * bs, p = m->row_ptr[r];
    for (int64_t j = 0; j < cnt[r]; ++j) m->col[p + j] = (int32_t)(b0 + j);
  }
  fill_values(*m, seed, lo, hi);
  return m;
}

// Shape of a generated matrix; returns nnz (or -1 for a null handle).
int64_t vnec_gen_info(const void* h, int64_t* n_rows, int64_t* n_cols) {
  if (!h) return -1;
  auto* m = static_cast<const HostCSR*>(h);
  if (n_rows) *n_rows = m->n_rows;
  if (n_cols) *n_cols = m->n_cols;
  return m->nnz;
}

// Borrowed pointers to the generated arrays (valid until vnec_gen_free).
void vnec_gen_arrays(void* h, int64_t** row_ptr, int32_t** col, double** val) {
  auto* m = static_cast<HostCSR*>(h);
  if (row_ptr) *row_ptr = m->row_ptr.get();
  if (col) *col = m->col.get();
  if (val) *val = m->val.get();
}

void vnec_gen_free(void* h) { delete static_cast<HostCSR*>(h); }

// Dense vector with entries U(lo, hi).
void vnec_gen_vector(int64_t n, double lo, double hi, uint64_t seed, double* out) {
  const double w = hi - lo;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) out[i] = lo + w * u01(hash3(seed, 7, (uint64_t)i));
}

}  // extern "C"
