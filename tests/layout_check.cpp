// Host-side check of the warp-task layout builders, compiled with
// AddressSanitizer and UndefinedBehaviorSanitizer by tests/test_layout_asan.py
// (test infrastructure: the GPU kernels are not involved).
//
// For random CSR matrices (empty rows, long rows, rectangular shapes) and many
// builder parameters, the layout is decoded on the CPU exactly as the kernels
// read it and the product with an integer-valued x is compared with the CSR
// product: values and x are small integers, so both sums are exact and must
// agree bit for bit.  Any out-of-bounds access in the builders stops the run.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "batch.h"
#include "sliced.h"

using namespace vnec;

namespace {

struct Csr {
  int64_t n_rows, n_cols;
  std::vector<int64_t> rp;
  std::vector<int32_t> ci;
  std::vector<double> val;
};

Csr random_csr(std::mt19937_64& rng, int64_t n_rows, int64_t n_cols, int max_len, double p_empty, double p_long,
               int long_len) {
  Csr m{n_rows, n_cols, {0}, {}, {}};
  std::uniform_real_distribution<double> u(0, 1);
  for (int64_t r = 0; r < n_rows; ++r) {
    int64_t len = 0;
    const double t = u(rng);
    if (t < p_empty)
      len = 0;
    else if (t < p_empty + p_long)
      len = std::min<int64_t>(n_cols, long_len + (int64_t)(u(rng) * long_len));
    else
      len = std::min<int64_t>(n_cols, 1 + (int64_t)(u(rng) * max_len));
    std::vector<char> used((size_t)n_cols, 0);
    std::vector<int32_t> cols;
    while ((int64_t)cols.size() < len) {
      const int32_t c = (int32_t)(u(rng) * (double)n_cols);
      if (c < n_cols && !used[(size_t)c]) {
        used[(size_t)c] = 1;
        cols.push_back(c);
      }
    }
    std::sort(cols.begin(), cols.end());
    for (int32_t c : cols) {
      m.ci.push_back(c);
      m.val.push_back((double)(1 + (int)(u(rng) * 7)) * (u(rng) < 0.5 ? -1 : 1));
    }
    m.rp.push_back((int64_t)m.ci.size());
  }
  return m;
}

std::vector<double> csr_spmv(const Csr& m, const std::vector<double>& x, int k, int64_t col_off = 0) {
  std::vector<double> y((size_t)m.n_rows * k, 0.0);
  for (int64_t r = 0; r < m.n_rows; ++r)
    for (int64_t p = m.rp[(size_t)r]; p < m.rp[(size_t)r + 1]; ++p)
      for (int j = 0; j < k; ++j) y[(size_t)r * k + j] += m.val[(size_t)p] * x[(size_t)(m.ci[(size_t)p] + col_off) * k + j];
  return y;
}

int failures = 0;

void expect_equal(const std::vector<double>& a, const std::vector<double>& b, const char* what) {
  if (a.size() != b.size()) {
    std::printf("FAIL %s: sizes %zu vs %zu\n", what, a.size(), b.size());
    ++failures;
    return;
  }
  for (size_t i = 0; i < a.size(); ++i)
    if (a[i] != b[i]) {
      std::printf("FAIL %s: element %zu: %.17g vs %.17g\n", what, i, a[i], b[i]);
      ++failures;
      return;
    }
}

// Decodes a sliced layout (vpe = 1) the way sliced_kernel and
// sliced_long_fixup read it; y entries never written stay NaN.
std::vector<double> sliced_decode(const SlicedHostView& v, int64_t n_rows, const std::vector<double>& x) {
  std::vector<double> y((size_t)n_rows, std::nan(""));
  std::vector<double> chunk((size_t)v.num_chunks, 0.0);
  const double* val = static_cast<const double*>(v.val);
  for (int64_t t = 0; t < v.num_tasks; ++t) {
    const SlicedTask& tk = v.tasks[t];
    const int kind = tk.meta & 15, vwl = (tk.meta >> 4) & 15, nrows = (tk.meta >> 8) & 0xff;
    if (kind == kSlicedZero) {
      for (int l = 0; l < nrows; ++l) y[(size_t)v.rowid[tk.row_base + l]] = 0.0;
      continue;
    }
    const int VW = 1 << vwl;
    double lane[32] = {0};
    if (tk.meta & kSlicedDelta) {
      for (int l = 0; l < 32; ++l) {
        int64_t c = l < nrows ? v.first[tk.row_base + l] : 0;
        for (int s = 0; s < tk.steps; ++s) {
          const int64_t e = (int64_t)tk.base + (int64_t)s * 32 + l;
          c += v.col16[e];
          lane[l] += val[e] * x[(size_t)c];
        }
      }
    } else {
      for (int s = 0; s < tk.steps; ++s)
        for (int l = 0; l < 32; ++l) {
          const int64_t e = (int64_t)tk.base + (int64_t)s * 32 + l;
          lane[l] += val[e] * x[(size_t)v.col[e]];
        }
    }
    if (kind == kSlicedChunk) {
      double sum = 0;
      for (int l = 0; l < 32; ++l) sum += lane[l];
      chunk[(size_t)tk.row_base] = sum;
    } else {
      for (int g = 0; g < nrows; ++g) {
        double sum = 0;
        for (int l = g * VW; l < (g + 1) * VW; ++l) sum += lane[l];
        y[(size_t)v.rowid[tk.row_base + g]] = sum;
      }
    }
  }
  for (int64_t i = 0; i < v.num_long; ++i) {
    double sum = 0;
    for (int32_t c = v.long_first[i]; c < v.long_first[i + 1]; ++c) sum += chunk[(size_t)c];
    y[(size_t)v.long_row[i]] = sum;
  }
  return y;
}

// Decodes a batch layout the way run_tasks reads it (any k, lanes, V).
std::vector<double> batch_decode(const BatchHostView& v, int k, const std::vector<double>& X) {
  const int L = v.lanes, S = 32 / L, R = k / L;
  std::vector<double> Y((size_t)v.n_rows * k, std::nan(""));
  std::vector<double> chunk((size_t)v.num_chunks * k, 0.0);
  for (int64_t t = 0; t < v.num_tasks; ++t) {
    const SlicedTask& tk = v.tasks[t];
    const int kind = tk.meta & 15, vwl = (tk.meta >> 4) & 15, nrows = tk.meta >> 8;
    if (kind == kSlicedZero) {
      for (int l = 0; l < nrows; ++l)
        for (int j = 0; j < k; ++j) Y[(size_t)v.rowid[tk.row_base + l] * k + j] = 0.0;
      continue;
    }
    // acc[slot][rhs]
    std::vector<double> acc((size_t)S * k, 0.0);
    for (int s = 0; s < tk.steps; ++s)
      for (int slot = 0; slot < S; ++slot) {
        const int64_t e = (int64_t)tk.base + (int64_t)s * S + slot;
        for (int j = 0; j < k; ++j) acc[(size_t)slot * k + j] += v.val[e] * X[(size_t)v.col[e] * k + j];
      }
    if (kind == kSlicedChunk) {
      for (int j = 0; j < k; ++j) {
        double sum = 0;
        for (int slot = 0; slot < S; ++slot) sum += acc[(size_t)slot * k + j];
        chunk[(size_t)tk.row_base * k + j] = sum;
      }
    } else {
      const int V = 1 << vwl;
      for (int g = 0; g < nrows; ++g)
        for (int j = 0; j < k; ++j) {
          double sum = 0;
          for (int slot = g * V; slot < (g + 1) * V; ++slot) sum += acc[(size_t)slot * k + j];
          Y[(size_t)v.rowid[tk.row_base + g] * k + j] = sum;
        }
    }
  }
  for (int64_t i = 0; i < v.num_long; ++i)
    for (int j = 0; j < k; ++j) {
      double sum = 0;
      for (int32_t c = v.long_first[i]; c < v.long_first[i + 1]; ++c) sum += chunk[(size_t)c * k + j];
      Y[(size_t)v.long_row[i] * k + j] = sum;
    }
  (void)R;
  return Y;
}

}  // namespace

int main() {
  std::mt19937_64 rng(12345);
  std::uniform_int_distribution<int> xi(-3, 3);
  int cases = 0;
  // ---- sliced layout ----
  for (int trial = 0; trial < 24; ++trial) {
    const int64_t n_rows = 1 + (int64_t)(rng() % 3000), n_cols = 1 + (int64_t)(rng() % 5000);
    Csr m = random_csr(rng, n_rows, n_cols, 1 + (int)(rng() % 90), 0.1, 0.02, 40 + (int)(rng() % 3000));
    std::vector<double> x((size_t)n_cols);
    for (auto& e : x) e = xi(rng);
    const std::vector<double> want = csr_spmv(m, x, 1);
    for (int variant = 0; variant < 4; ++variant) {
      SlicedParams prm;
      prm.window_rows = variant == 1 ? 97 : 1 << 16;
      prm.long_len = variant == 2 ? 32 : 1024;
      prm.chunk = variant == 2 ? 64 : 1024;
      prm.max_steps = variant == 3 ? 1 : 32;
      prm.delta16 = variant != 1;
      // keep mask: every other row in variant 3 (the rest must stay NaN)
      std::vector<uint8_t> keep((size_t)n_rows, 1);
      if (variant == 3)
        for (int64_t r = 0; r < n_rows; r += 2) keep[(size_t)r] = 0;
      SlicedHost* h = sliced_build(n_rows, n_cols, m.rp.data(), nullptr, m.ci.data(), nullptr, m.val.data(), 8, prm,
                                   1, variant == 3 ? keep.data() : nullptr);
      if (!h) {
        std::printf("FAIL sliced_build returned null\n");
        return 1;
      }
      std::vector<double> got = sliced_decode(sliced_view(h), n_rows, x);
      std::vector<double> exp = want;
      if (variant == 3)
        for (int64_t r = 0; r < n_rows; r += 2) {
          if (!std::isnan(got[(size_t)r])) {
            std::printf("FAIL sliced keep mask: row %lld written\n", (long long)r);
            ++failures;
          }
          got[(size_t)r] = exp[(size_t)r] = 0.0;
        }
      expect_equal(got, exp, "sliced");
      sliced_free(h);
      ++cases;
    }
  }
  // ---- batch layout ----
  for (int trial = 0; trial < 8; ++trial) {
    const int nm = 1 + (int)(rng() % 7);
    std::vector<Csr> mats;
    for (int q = 0; q < nm; ++q)
      mats.push_back(random_csr(rng, (int64_t)(rng() % 400), 1 + (int64_t)(rng() % 700), 1 + (int)(rng() % 60), 0.1,
                                0.03, 50 + (int)(rng() % 900)));
    std::vector<int64_t> nr, nc;
    std::vector<const int64_t*> rp;
    std::vector<const int32_t*> ci;
    std::vector<const double*> vv;
    int64_t cols_total = 0;
    for (auto& m : mats) {
      nr.push_back(m.n_rows);
      nc.push_back(m.n_cols);
      rp.push_back(m.rp.data());
      ci.push_back(m.ci.data());
      vv.push_back(m.val.data());
      cols_total += m.n_cols;
    }
    for (int k : {1, 2, 4, 8, 16, 32})
      for (int L = 1; L <= 32; L <<= 1) {
        if (!batch_supported(k, L)) continue;
        for (int variant = 0; variant < 2; ++variant) {
          std::vector<double> X((size_t)cols_total * k);
          for (auto& e : X) e = xi(rng);
          std::vector<double> want;
          int64_t off = 0;
          for (auto& m : mats) {
            std::vector<double> Xm(X.begin() + off * k, X.begin() + (off + m.n_cols) * k);
            const std::vector<double> ym = csr_spmv(m, Xm, k);
            want.insert(want.end(), ym.begin(), ym.end());
            off += m.n_cols;
          }
          BatchParams prm;
          prm.lanes = L;
          prm.long_len = variant ? 40 : 1024;
          prm.chunk = variant ? 33 : 1024;
          prm.max_steps = variant ? 3 : 32;
          prm.window_rows = variant ? 61 : 1 << 16;
          BatchHost* h = batch_build(nm, nr.data(), nc.data(), rp.data(), ci.data(), vv.data(), k, prm);
          if (!h) {
            std::printf("FAIL batch_build returned null (k %d lanes %d)\n", k, L);
            return 1;
          }
          expect_equal(batch_decode(batch_view(h), k, X), want, "batch");
          batch_free(h);
          ++cases;
        }
      }
  }
  std::printf("%d layout cases, %d failures\n", cases, failures);
  return failures ? 1 : 0;
}
