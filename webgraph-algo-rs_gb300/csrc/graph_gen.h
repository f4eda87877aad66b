// Host CSR container and the deterministic synthetic generators
// (graph_gen.cpp). Standard C++ only: shared by the product library and the
// oracle's library.
#pragma once

#include <cstdint>
#include <vector>

// Host CSR graph: offsets[n+1] (u64), successors[m] (u32), rows sorted.
struct Csr {
    uint64_t n = 0, m = 0;
    std::vector<uint64_t> offsets;
    std::vector<uint32_t> successors;
};

namespace hbg {
// t = the transpose of g, every row sorted
void transpose(const Csr& g, Csr& t);
// node v gets min(d, n-1) distinct uniform successors other than itself
void gen_er(uint64_t n, uint32_t d, uint64_t seed, Csr& g);
// R-MAT with 2^scale nodes and edges_per_node * 2^scale drawn arcs, (a, b, c, 1-a-b-c)
void gen_rmat(int scale, uint64_t edges_per_node, double a, double b, double c, uint64_t seed,
              Csr& g);
// Zipf(2.1) out-degrees capped at `cap`, 80% of successors within +/-window
void gen_weblike(uint64_t n, uint64_t cap, double shift, uint64_t window, uint64_t seed, Csr& g);
}  // namespace hbg
