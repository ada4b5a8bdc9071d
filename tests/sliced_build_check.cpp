// Host-only checks of the sliced builder's shared-pattern tasks
// (vnec_gb300/csrc/sliced_build.cpp), compiled with g++ and run by
// tests/test_sliced_build_cpu.py; no GPU is used.  For each matrix it reads
// every delta task back and checks that the task is flagged kSlicedShared
// exactly when all its rows have `steps` entries with the first row's column
// gaps (and at most 32 steps), that pat16 holds those gaps, and that the
// host view's counts match.  Prints one line per matrix; exits non-zero on
// any mismatch.
#include <cstdint>
#include <cstdio>
#include <random>
#include <set>
#include <vector>

#include "sliced.h"

using namespace vnec;

struct Csr {
  int64_t n = 0;
  std::vector<int64_t> ptr{0};
  std::vector<int32_t> col;
  std::vector<double> val;
  void add_row(const std::vector<int32_t>& c) {
    for (int32_t x : c) {
      col.push_back(x);
      val.push_back(1.0 + (double)col.size() * 1e-3);
    }
    ptr.push_back((int64_t)col.size());
    ++n;
  }
};

Csr stencil27(int g) {
  Csr a;
  for (int z = 0; z < g; ++z)
    for (int y = 0; y < g; ++y)
      for (int x = 0; x < g; ++x) {
        std::vector<int32_t> c;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const int X = x + dx, Y = y + dy, Z = z + dz;
              if (X >= 0 && Y >= 0 && Z >= 0 && X < g && Y < g && Z < g) c.push_back((Z * g + Y) * g + X);
            }
        a.add_row(c);
      }
  return a;
}

Csr constant_band(int n) {
  Csr a;
  const int off[] = {-40, -3, -1, 0, 2, 7, 300};
  for (int r = 0; r < n; ++r) {
    std::set<int32_t> c;
    for (int o : off) c.insert((int32_t)std::min(std::max(r + o, 0), n - 1));
    a.add_row(std::vector<int32_t>(c.begin(), c.end()));
  }
  return a;
}

Csr random_rows(int n, int k, unsigned seed) {
  Csr a;
  std::mt19937 rng(seed);
  for (int r = 0; r < n; ++r) {
    std::set<int32_t> c;
    while ((int)c.size() < k) c.insert((int32_t)(rng() % (unsigned)n));
    a.add_row(std::vector<int32_t>(c.begin(), c.end()));
  }
  return a;
}

int check(const Csr& a, const char* name, bool shared_on, int max_steps, int expect) {
  SlicedParams prm;
  prm.delta16 = true;
  prm.shared = shared_on;
  prm.max_steps = max_steps;
  SlicedHost* h = sliced_build(a.n, a.n, a.ptr.data(), nullptr, a.col.data(), nullptr, a.val.data(), 8, prm);
  if (!h) {
    std::printf("%s: build failed\n", name);
    return 1;
  }
  const SlicedHostView v = sliced_view(h);
  long long shared_tasks = 0, shared_nnz = 0, shared_steps = 0, bad = 0, missed = 0;
  for (int64_t t = 0; t < v.num_tasks; ++t) {
    const SlicedTask& k = v.tasks[t];
    const int kind = k.meta & 15, nrows = (k.meta >> 8) & 0xff;
    if (kind != kSlicedRows || !(k.meta & kSlicedDelta)) {
      bad += (k.meta & kSlicedShared) != 0;
      continue;
    }
    const int64_t b0 = a.ptr[v.rowid[k.row_base]];
    bool same = k.steps <= 32 && k.base % 32 == 0;
    for (int g = 0; g < nrows && same; ++g) {
      const int32_t r = v.rowid[k.row_base + g];
      const int64_t b = a.ptr[r];
      if (a.ptr[r + 1] - b != k.steps) same = false;
      for (int64_t j = 1; j < k.steps && same; ++j)
        same = a.col[b + j] - a.col[b + j - 1] == a.col[b0 + j] - a.col[b0 + j - 1];
    }
    if (k.meta & kSlicedShared) {
      bad += !same || !v.pat16;
      if (!v.pat16) continue;
      ++shared_tasks;
      shared_nnz += (long long)nrows * k.steps;
      shared_steps += k.steps;
      const uint16_t* p = v.pat16 + k.base / 32;
      bad += p[0] != 0;
      for (int64_t j = 1; j < k.steps; ++j) bad += p[j] != (uint16_t)(a.col[b0 + j] - a.col[b0 + j - 1]);
    } else if (same && shared_on) {
      ++missed;
    }
  }
  bad += shared_nnz != v.shared_nnz || shared_steps != v.shared_steps;
  bad += !shared_on && (v.pat16 != nullptr || shared_tasks != 0);
  const bool want = expect > 0;
  bad += shared_on && (want ? shared_tasks == 0 : shared_tasks != 0);
  std::printf("%s: shared %s, tasks %lld, shared tasks %lld (%lld nonzeros, %lld steps), mismatches %lld, missed %lld\n",
              name, shared_on ? "on" : "off", (long long)v.num_tasks, shared_tasks, shared_nnz, shared_steps, bad,
              missed);
  sliced_free(h);
  return (bad + missed) ? 1 : 0;
}

int main() {
  int fail = 0;
  const Csr s8 = stencil27(8), s20 = stencil27(20), band = constant_band(6000), rnd = random_rows(5000, 9, 7);
  fail |= check(s8, "stencil27 8^3", true, 32, 1);
  fail |= check(s20, "stencil27 20^3", true, 32, 1);
  fail |= check(s20, "stencil27 20^3", false, 32, 0);
  fail |= check(s20, "stencil27 20^3 max_steps 7", true, 7, 0);
  fail |= check(band, "constant band", true, 32, 1);
  fail |= check(rnd, "random 9 per row", true, 32, 0);
  return fail;
}
