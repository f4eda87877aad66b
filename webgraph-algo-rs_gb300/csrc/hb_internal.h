// Internal declarations shared by the host engine (hb_engine.cpp), the host
// graph layer (graph_host.cpp) and the CUDA kernels (hb_kernels.cu).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda.h>
#include <vector_types.h>

#include "../../include/hyperball_gb300.h"
#include "graph_gen.h"

namespace hbg {
int load_bvgraph(const std::string& basename, Csr& g, std::string& err, uint64_t* bits_checked);
}  // namespace hbg

// ---------------------------------------------------------------------------
// Device-side parameters
// ---------------------------------------------------------------------------
namespace hbk {

constexpr int MAX_DISCOUNT = 8;
// heavy nodes with more arcs than HEAVY_SPLIT run as segments of HEAVY_SEG
// arcs, one CTA each (k_union_heavy)
constexpr uint64_t HEAVY_SPLIT = 32768;
constexpr uint64_t HEAVY_SEG = 16384;

// What one tile (or one block of the heavy-node kernel) contributes to an
// iteration; summed in a fixed order after the union kernels.
struct TilePartial {
    double nf;                    // neighbourhood-function contribution
    unsigned long long vis;       // arcs the next iteration visits (k_finalize)
    unsigned long long mod;       // modified counters
    unsigned long long scanned;   // scanned nodes
    unsigned long long sarcs;     // arcs of the scanned nodes
    unsigned long long timeouts;  // bounded mbarrier waits that gave up (an error)
};

// The values of one iteration t that the kernels read from device memory, so
// that the launches of an iteration (and a graph captured from them) do not
// change from one iteration to the next.
struct IterConsts {
    double d1, rd1;                      // t + 1 and RN(1 / (t + 1))
    double disc_factor[MAX_DISCOUNT];    // discount function k at distance t + 1
};

// Everything the union kernels read or write in one iteration.
struct UnionArgs {
    CUtensorMap far_map;      // the current counters as rows of 2^log2m bytes (TMA gathers)
    int far_tma;              // 1: far successors by TMA gathers (far_map valid)
    uint32_t far_rows;        // a successor is far when more than this many ids from its node
    uint32_t mbar_polls;      // polls of a bounded far-gather wait (0: the default limit)
    uint32_t test_extra_tx;   // tests only: bytes added to every expected count (the wait cannot complete)
    const uint64_t* off;      // CSR offsets, n+1
    const uint32_t* succ;     // CSR successors, m
    const uint8_t* curr;      // current counters, n * 2^log2m bytes (byte per register)
    uint8_t* next;            // next counters
    const uint32_t* curr_mod; // modified in the previous iteration (bitmap)
    uint32_t* next_mod;       // modified in this iteration (bitmap, cleared)
    const uint32_t* mbc;      // must be checked (systolic), bitmap
    double* est;              // cached count() of every current counter
    double* sod;              // sum of distances or null
    double* harm;             // sum of inverse distances or null
    double* disc[MAX_DISCOUNT];
    int ndisc;
    const IterConsts* ic;     // this iteration's d = t + 1, 1/d and discount factors (device)
    int systolic;             // 1: scan only must-be-checked nodes
    int quirk;                // Rust i32-shift count semantics
    int any31;                // some register may hold 31 (only then count looks for it)
    uint64_t n;
    double alpha_m_m;
    double a_scaled;          // alpha_m_m * 2^31
    long long small_bits;     // bit pattern of 2.5 * m
    const double* ln_table;   // m * ln(m / z), z = 0..m
    const uint32_t* list;     // heavy node list
    uint64_t list_len;
    // heavy-kernel work items {heavy index, segment, segments, first partial
    // slot}, and for split nodes the partial counters of their segments and
    // one arrival count per node (at its first slot; zero between launches)
    const uint4* heavy_items;
    uint64_t heavy_len;
    uint8_t* heavy_part;
    uint32_t* heavy_arrive;
    const uint32_t* tiles;    // window k = nodes [tiles[k], tiles[k+1])
    uint32_t n_tiles;         // number of windows
    // systolic iterations: the light and medium nodes to check or to copy, in
    // node order, and their counts (device word: light | medium << 32);
    // null in standard iterations, which walk the chunk table
    const uint32_t* light_list;
    const uint32_t* medium_list;
    const uint64_t* list_counts;
    const uint2* chunks;      // {first node, count | medium << 31}, in node order
    // batches, standard iterations: the chunks of the running instances
    // (indices into chunks) and their number (device word); null otherwise
    const uint32_t* queue;
    const uint32_t* queue_len;
    const uint4* items;       // staged kernel: {first node, count | medium << 31, first arc, arcs}
    uint32_t staged;          // 1: standard iteration on the staged kernel (k_union_staged)
    int gather_all;           // merge every successor (nearly all changed before)
    const uint32_t* indeg;    // in-degree without self-loops
    double* nf_items;         // neighbourhood-function part of each work item, then of each heavy node
    uint64_t heavy_item_base; // index of the first heavy node's part
    uint64_t n_chunks;
    unsigned long long* cursor; // next chunk to take (zero at launch)
    // variant of the union kernels (same results; chosen by the autotuner)
    uint32_t pf;              // successor counters prefetched: 0 no, 1 into L2, 2 into L1
    uint32_t pd;              // prefetch distance in arcs
    uint32_t occ;             // window kernel sized for 4 resident blocks per SM instead of 3
    uint32_t tile_max_degree; // nodes above this out-degree are listed as heavy
    uint32_t acc_slot;        // partial slot accumulating the union kernels' integer totals
    TilePartial* partials;    // one per finalize block, then acc_slot
};

struct InitArgs {
    const uint32_t* perm;     // device node -> caller node (the id that is hashed)
    const uint32_t* hash_id;  // batches: device node -> id hashed (its instance's own id), or null
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
    int* any31;               // set to 1 when an initial register holds 31
};

static_assert(sizeof(IterConsts) % 8 == 0 && sizeof(TilePartial) % 8 == 0, "copied as 64-bit words");

// Launchers (hb_kernels.cu). All return cudaError_t as int.
// dst[i] = src[i], i < n, by a kernel (either side may be page-locked host
// memory, which the device reads and writes through unified addressing)
int launch_copy_u64(const uint64_t* src, uint64_t* dst, uint64_t n, void* stream);
int launch_init(int log2m, const InitArgs& a, void* stream);
// device counters (one byte per register) -> the reference's packed layout,
// in caller node order (inv: caller node -> device node)
int launch_pack_counters(int log2m, const uint8_t* src, const uint32_t* inv, uint8_t* dst,
                         uint64_t n, void* stream);
// rows[v] += indeg[v], v < n
int launch_add_indeg(unsigned long long* rows, const uint32_t* indeg, uint64_t n, void* stream);
// renumbering: deg[i] = out-degree of perm[i] (deg[n] = 0)
int launch_perm_degree(const uint64_t* off0, const uint32_t* perm, uint64_t n,
                       unsigned long long* deg, void* stream);
// arc-parallel passes: tiles of consecutive arcs; tile_start[k] (arc_tiles(m)
// words) = the node holding the first arc of tile k
uint64_t arc_tiles(uint64_t m);
int launch_tile_start(const uint64_t* off, uint64_t n, uint32_t* tile_start, void* stream);
// succ[e] = inv[succ0[off0[perm[i]] + e - off[i]]] for every arc e of node i
// (targets >= n set *bad); with indeg (zeroed): in-degrees without self-loops,
// *loops += self-loops, and with trows (zeroed) trows[i] += self-loops of i
int launch_relabel_arcs(const uint64_t* off, uint64_t n, uint64_t m, const uint32_t* tile_start,
                        const uint32_t* perm, const uint64_t* off0, const uint32_t* succ0,
                        const uint32_t* inv, uint32_t* succ, uint32_t* indeg, unsigned long long* loops,
                        unsigned long long* trows, int* bad, void* stream);
// transpose scatter with per-row cursors (positions of the next arc of each row)
int launch_scatter_arcs(const uint64_t* off, uint64_t n, uint64_t m, const uint32_t* tile_start,
                        const uint32_t* succ, unsigned long long* cursor, uint32_t* tsucc, void* stream);
// dst[u] = src[inv[u]]: a per-node array back to caller order
int launch_gather_f64(const double* src, const uint32_t* inv, double* dst, uint64_t n,
                      void* stream);
// persistent tile kernel over the worklist (or all tiles)
int launch_union_tile(int log2m, const UnionArgs& a, int grid, void* stream);
// A TMA descriptor for a counter array (n rows of 2^log2m bytes) as the union
// kernel's far gathers read it; nonzero when the TMA path is not available
// for this size (log2m > 8, n >= 2^31) or the driver cannot encode it.
int encode_far_map(int log2m, const uint8_t* counters, uint64_t n, CUtensorMap* out);
int tile_grid(int log2m, int device, int occ);
// standard iterations on the staged window kernel (items table; m < 2^32)
int launch_union_staged(int log2m, const UnionArgs& a, int grid, void* stream);
int staged_grid(int log2m, int device, int occ);
// the window work of several handles in one launch (log2m 4, 6 or 8 each):
// every job's arguments travel as kernel parameters (constant bank), so at
// most 48 jobs fit the 32 KB parameter space
constexpr int MAX_JOBS = 48;
struct JobsArgs {
    UnionArgs job[MAX_JOBS];
    int log2m[MAX_JOBS];
    uint32_t njobs;
    unsigned long long* cursor;  // zero at launch
};
int launch_union_jobs(const JobsArgs& p, int grid, void* stream);
int jobs_grid(int device);
// batches: queue = the chunks of the running instances (modified count of
// the previous iteration nonzero, or every instance when `all`), queue_len its
// length; cnt and at hold count + 1 words
int launch_inst_queue(const uint32_t* inst_chunk, const unsigned long long* inst_mod, uint32_t count,
                      int all, uint32_t n_chunks, unsigned long long* cnt, uint64_t* at,
                      unsigned long long* scratch, uint64_t scratch_len, uint32_t* queue,
                      uint32_t* queue_len, void* stream);
// inst_chunk[i] = the first chunk of instance i (count + 1 words; start has count + 1)
int launch_inst_first_chunk(const uint2* chunks, uint64_t n_chunks, const uint64_t* start,
                            uint32_t count, uint32_t* inst_chunk, void* stream);
// items[k] = {first, count | medium << 31, off[first], arcs of the chunk}
int launch_chunk_items(const uint2* chunks, uint64_t n_chunks, const uint64_t* off, uint4* items,
                       void* stream);
// nodes and staged arcs one tile holds at this log2m
int tile_capacity(int log2m, uint32_t* nodes, uint32_t* arcs);
// heavy nodes, one CTA each
int launch_union_heavy(int log2m, const UnionArgs& a, int grid, void* stream);
int heavy_grid(int log2m, int device);
// batches: per instance [starts[i], starts[i+1]) the modified counters of the
// iteration (next_mod) and the sum of the cached estimates
int launch_inst_stats(const uint32_t* next_mod, const double* est, const uint64_t* starts,
                      uint32_t count, unsigned long long* mods, double* nfs, void* stream);
// fixed-order sum of count doubles into *out (scratch: 256 doubles)
int launch_sum_f64(const double* in, uint64_t count, double* scratch, double* out, void* stream);
// systolic work lists: every light / medium node set in mbc | curr_mod, in
// node order (medium_bits / light_bits: the medium / light nodes). cnt and
// off hold nwords + 1 words; off[nwords] gets the counts (light | medium << 32).
int launch_work_lists(const uint32_t* mbc, const uint32_t* curr_mod, const uint32_t* medium_bits,
                      const uint32_t* light_bits, uint64_t n, unsigned long long* cnt, uint64_t* off,
                      unsigned long long* scratch, uint64_t scratch_len, uint32_t* light_list,
                      uint32_t* medium_list, void* stream);
// nodes per chunk of the union kernel: light nodes (lane-group each) and
// medium nodes (team each)
int chunk_nodes(int log2m, uint32_t* light, uint32_t* medium);
// fixed-order sum of `count` partials; scratch holds 256 partials
int launch_reduce_partials(const TilePartial* in, uint64_t count, TilePartial* scratch,
                           TilePartial* out, void* stream);
int launch_mark_preds(const uint32_t* next_mod, const uint64_t* toff, const uint32_t* tsucc,
                      uint32_t* next_mbc, uint64_t n, int grid, void* stream);
int launch_fill_u32(uint32_t* p, uint32_t v, uint64_t count, void* stream);
int launch_transpose_count(const uint32_t* succ, uint64_t m, unsigned long long* indeg,
                           void* stream);
int launch_exclusive_scan_u64(const unsigned long long* in, uint64_t* out, uint64_t count,
                              unsigned long long* scratch, uint64_t scratch_len, void* stream);
uint64_t scan_scratch_len(uint64_t count);
// The fixed device scratch of hb_device_transpose_noalloc on the current
// device (looked up on first use per device) and its size in words.
constexpr uint64_t NOALLOC_MAX_NODES = 1ull << 20;
int noalloc_scratch(unsigned long long** out, uint64_t* words);
int launch_transpose_scatter(const uint64_t* off, const uint32_t* succ, uint64_t n,
                             unsigned long long* cursor, uint32_t* tsucc, void* stream);
// work partition: per segment tiles[w] .. tiles[w + 1] (at most the tile
// window of nodes) its chunk count and heavy count (index nseg: zeros) ...
int launch_part_count(const uint64_t* off, const uint32_t* tiles, uint64_t nseg, uint64_t small_max,
                      uint64_t medium_max, uint32_t per_light, uint32_t per_medium,
                      unsigned long long* seg_chunks, unsigned long long* seg_heavy, void* stream);
// ... then, from their exclusive scans, the renumbering (perm, inv), the chunk
// table, the heavy keys (inverted degree << 32 | new id, segment order), the
// kind bitmaps (zeroed by the caller) and, when seg_base is given, hash_id[new]
// = caller id - seg_base[segment]
int launch_part_place(const uint64_t* off, const uint32_t* tiles, uint64_t nseg, uint64_t small_max,
                      uint64_t medium_max, uint32_t per_light, uint32_t per_medium,
                      const unsigned long long* chunk_at, const unsigned long long* heavy_at,
                      const uint32_t* seg_base, uint32_t* perm, uint32_t* inv, uint2* chunks,
                      unsigned long long* heavy_keys, uint32_t* light_bits, uint32_t* medium_bits,
                      uint32_t* hash_id, void* stream);
int launch_validate(const uint64_t* off, const uint32_t* succ, uint64_t n, uint64_t m, int* bad,
                    void* stream);

int num_sms(int device);
// kernels launched so far by the calling host thread (a graph launch adds the
// kernels it runs)
uint64_t launch_count();
void count_launches(int64_t delta);

}  // namespace hbk

// ---------------------------------------------------------------------------
// Several handles advanced together (hb_engine.cpp; used by the job server):
// each step runs one iteration of every handle given, with one shared union
// launch. Handles must be on the context's device and idle.
// ---------------------------------------------------------------------------
struct hb_multi;
int hb_multi_create(int device, void* stream, hb_multi** out, std::string& err);
void hb_multi_destroy(hb_multi* m);
// hb_init of a handle that will be stepped (its own stream, synchronous)
int hb_multi_start(hb_handle* h);
// one iteration of each of the count handles (count <= MAX_JOBS)
// moves the handle's later work to `stream` (its earlier work is waited for)
int hb_multi_set_stream(hb_handle* h, void* stream);
int hb_multi_step(hb_multi* m, hb_handle* const* hs, uint32_t count, std::string& err);
// the shared union launch leaves `sms` SMs free (its grid is that much smaller)
void hb_multi_reserve_sms(hb_multi* m, uint32_t sms);
// the handle's run is over: its last iteration modified no counter, or it
// ran num_nodes iterations (the stop rules of run_until_done, HB:541, HB:559-570)
bool hb_multi_done(const hb_handle* h);
// steps run so far, of them replayed from graphs, device time of the union
// parts (shared launch and heavy kernels), host time planning and launching,
// host time waiting for the steps, device time before and after the union parts
uint64_t hb_multi_steps(const hb_multi* m, uint64_t* replays, double* union_ms, double* host_ms,
                        double* wait_ms, double* pre_ms, double* post_ms);

