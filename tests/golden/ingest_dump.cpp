// Loads a graph with the reference's own reader/builder (utilities/
// builder.hpp:319-344: .mtx through Reader::ReadFile + MakeGraphFromEL, which
// sorts, removes duplicate edges and self-loops; .sg through
// Reader::ReadSerializedGraph, utilities/reader.hpp:189-240) and writes the
// CSR it yields as raw little-endian uint64: num_nodes, num_edges,
// offsets[num_nodes + 1], destinations[num_edges].
// TEST INFRASTRUCTURE ONLY: compiled against the reference's headers by
// tests/golden/make_ingest_golden.py to make the ingest fixtures.
//
//   ingest_dump <graph.mtx|graph.sg> <out.bin>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <string>

#include "../utilities/builder.hpp"
#include "../utilities/graph.hpp"
#include "../include/OpenSparseBLAS.h"

template <class G>
static int dump(const G& g, const char* out) {
  std::ofstream f(out, std::ios::binary);
  uint64_t n = g.num_nodes(), m = g.num_edges();
  f.write(reinterpret_cast<const char*>(&n), 8);
  f.write(reinterpret_cast<const char*>(&m), 8);
  f.write(reinterpret_cast<const char*>(g.out_offsets()), 8 * (n + 1));
  f.write(reinterpret_cast<const char*>(g.out_destValues()), 8 * m);
  return f.good() ? 0 : 1;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <graph.mtx|graph.sg> <out.bin>\n", argv[0]);
    return 2;
  }
  const std::string in = argv[1];
  if (in.size() > 4 && in.substr(in.size() - 4) == ".mtx") {
    Builder<SpB_Index, SpB_Index, SpB_Index> b(in, false);
    auto g = b.MakeGraph();
    return dump(g, argv[2]);
  }
  Builder<SpB_Index, SpB_Index> b(in);
  auto g = b.MakeGraph();
  return dump(g, argv[2]);
}
