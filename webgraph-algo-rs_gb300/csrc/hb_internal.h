// Internal declarations shared by the host engine (hb_engine.cpp), the host
// graph layer (graph_host.cpp) and the CUDA kernels (hb_kernels.cu).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/hyperball_gb300.h"

// Host CSR graph: offsets[n+1] (u64), successors[m] (u32), rows sorted.
struct Csr {
    uint64_t n = 0, m = 0;
    std::vector<uint64_t> offsets;
    std::vector<uint32_t> successors;
};

namespace hbg {
void transpose(const Csr& g, Csr& t);
void gen_er(uint64_t n, uint32_t d, uint64_t seed, Csr& g);
void gen_rmat(int scale, uint64_t edges_per_node, double a, double b, double c, uint64_t seed,
              Csr& g);
void gen_weblike(uint64_t n, uint64_t cap, double shift, uint64_t window, uint64_t seed, Csr& g);
int load_bvgraph(const std::string& basename, Csr& g, std::string& err, uint64_t* bits_checked);
}  // namespace hbg

// ---------------------------------------------------------------------------
// Device-side parameters
// ---------------------------------------------------------------------------
namespace hbk {

constexpr int MAX_DISCOUNT = 8;

// Everything the union kernels read or write in one iteration.
struct UnionArgs {
    const uint64_t* off;      // CSR offsets, n+1
    const uint32_t* succ;     // CSR successors, m
    const uint8_t* curr;      // current counters, n * counter_bytes
    uint8_t* next;            // next counters
    const uint32_t* curr_mod; // modified in the previous iteration (bitmap)
    uint32_t* next_mod;       // modified in this iteration (bitmap, cleared)
    const uint32_t* mbc;      // must be checked (systolic), bitmap
    double* est;              // cached count() of every current counter
    double* sod;              // sum of distances or null
    double* harm;             // sum of inverse distances or null
    double* disc[MAX_DISCOUNT];
    double disc_factor[MAX_DISCOUNT];
    int ndisc;
    int systolic;             // 1: scan only must-be-checked nodes
    int quirk;                // Rust i32-shift count semantics
    uint32_t iter;            // 0-based iteration number
    uint64_t n;
    double alpha_m_m;
    const double* ln_table;   // m * ln(m / z), z = 0..m
    const uint32_t* list;     // node list (team kernels) or null
    uint64_t list_len;
    uint32_t small_max_degree;// group kernel skips nodes above this degree
    unsigned long long* stats_out; // [visited arcs, modified counters, scanned nodes]
    double* nf_partials;      // one slot per block of this launch
};

struct InitArgs {
    uint8_t* curr;
    double* est;
    uint64_t n;
    int hash_kind;
    uint64_t seed;
    const uint64_t* weights;  // optional
    uint64_t weight_seed;
    double alpha_m_m;
    const double* ln_table;
    int quirk;
};

// Launchers (hb_kernels.cu). All return cudaError_t as int.
int launch_init(int log2m, const InitArgs& a, void* stream);
int launch_union_group(int log2m, const UnionArgs& a, int grid, int block, void* stream);
int launch_union_team(int log2m, int team, const UnionArgs& a, int grid, void* stream);
int launch_mark_preds(const uint32_t* next_mod, const uint64_t* toff, const uint32_t* tsucc,
                      uint32_t* next_mbc, uint64_t n, int grid, void* stream);
int launch_reduce_nf(const double* partials, int count, double* out, void* stream);
int launch_fill_u32(uint32_t* p, uint32_t v, uint64_t count, void* stream);
int launch_transpose_count(const uint32_t* succ, uint64_t m, unsigned long long* indeg,
                           void* stream);
int launch_exclusive_scan_u64(const unsigned long long* in, uint64_t* out, uint64_t count,
                              unsigned long long* scratch, uint64_t scratch_len, void* stream);
uint64_t scan_scratch_len(uint64_t count);
int launch_transpose_scatter(const uint64_t* off, const uint32_t* succ, uint64_t n,
                             unsigned long long* cursor, uint32_t* tsucc, void* stream);
int launch_validate(const uint64_t* off, const uint32_t* succ, uint64_t n, uint64_t m, int* bad,
                    void* stream);
// Occupancy-derived grid (blocks) for union kernel kind 0 group, 1 warp team, 2 CTA team.
int union_grid(int log2m, int kind, int device);

int num_sms(int device);

}  // namespace hbk
