// Host engine and C ABI of the GB300 HyperBall.
//
// The control flow restates HyperBall::iterate / run
// (src/algo/hyperball/hyperball_impl.rs:534-949) over device-resident state:
//   * mode choice with the reference's integer thresholds (HB:795-810):
//     systolic iff a transpose exists, iteration > 0 and modified < n/4;
//     local / pre_local as in the reference (reported; on the device the
//     local checklist is the must-be-checked bitmap);
//   * neighbourhood function: standard iterations sum every scanned node's
//     count, systolic ones add (post - pre) to the previous unclamped value,
//     then the monotone clamp and relative increment (HB:916-944);
//   * termination exactly as run() (HB:541-577).
// Device layout (HBM): CSR offsets u64[n+1], successors u32[m], optional
// transpose CSR, two counter arrays n*B bytes (B = 2^log2m*5/8, reference
// layout), cached counts f64[n], the optional per-node sums f64[n], four
// n-bit bitmaps (modified current/next, must-be-checked current/next).
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "hb_internal.h"

namespace {

thread_local std::string g_global_err;

constexpr double LN_2 = 0.693147180559945309417232121458176568;

uint64_t rust_f64_to_u64(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 18446744073709551616.0) return UINT64_MAX;
    return (uint64_t)x;
}

// hyper_log_log_logic.rs:301-303
int register_size(uint64_t n) {
    double v = std::log((std::log((double)n) / LN_2) / LN_2);
    uint64_t c = rust_f64_to_u64(std::ceil(v));
    return (int)std::max<uint64_t>(5, c);
}

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// The library's device-memory pool of `device`, created on first use. Freed
// blocks are kept (no release threshold) for later allocations.
cudaError_t lib_pool(int device, cudaMemPool_t* out) {
    constexpr int MAX_DEVICES = 64;
    static std::mutex mu;
    static cudaMemPool_t pools[MAX_DEVICES] = {};
    if (device < 0 || device >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!pools[device]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t p = nullptr;
        cudaError_t e = cudaMemPoolCreate(&p, &props);
        if (e != cudaSuccess) return e;
        uint64_t keep = UINT64_MAX;
        e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(p);
            return e;
        }
        pools[device] = p;
    }
    *out = pools[device];
    return cudaSuccess;
}

// A non-blocking stream at the device's highest priority: its blocks are
// scheduled ahead of pending blocks of default-priority streams (the job
// server's creation work runs at the default priority beside the steps).
cudaError_t high_priority_stream(cudaStream_t* s) {
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return e;
    return cudaStreamCreateWithPriority(s, cudaStreamNonBlocking, greatest);
}

cudaError_t pool_alloc(int device, void** p, size_t bytes, cudaStream_t s) {
    cudaMemPool_t pool = nullptr;
    cudaError_t e = lib_pool(device, &pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

// Page-locked host blocks for the per-iteration totals and constants of a
// handle. Freed blocks are kept for the next handle instead of going back
// through cudaFreeHost, which may synchronise the device under the other
// handles' work (the job server destroys handles while others run).
std::mutex g_pinned_mu;
std::multimap<size_t, void*> g_pinned_free;

size_t pinned_class(size_t bytes) {
    size_t c = 256;
    while (c < bytes) c <<= 1;
    return c;
}

cudaError_t pinned_alloc(void** p, size_t bytes) {
    const size_t c = pinned_class(bytes);
    {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        auto it = g_pinned_free.find(c);
        if (it != g_pinned_free.end()) {
            *p = it->second;
            g_pinned_free.erase(it);
            return cudaSuccess;
        }
    }
    return cudaMallocHost(p, c);
}

void pinned_free(void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    g_pinned_free.emplace(pinned_class(bytes), p);
}

}  // namespace

struct hb_graph {
    Csr g;
};

// ---------------------------------------------------------------------------
// Autotuner of the union kernels. The variants differ only in how successor
// counters are requested (software prefetch into L1 or L2 ahead of the plain
// loads) and in the registers per thread (3 or 4 resident blocks per SM); they
// give the same counters, sums and statistics, so the engine may switch
// between them at any iteration. Per kind of iteration (standard merging every
// successor, standard merging modified successors) each variant is timed on
// one iteration that scans at least an eighth of the arcs and merges at least
// half of what it scans, as union time per scanned-plus-merged arc; the
// fastest is kept for the rest of the handle's life and remembered for later
// handles of a graph with the same shape. A variant other than the first
// must be at least 3% faster to be kept (one sample each). Systolic
// iterations vary too much from one to the next to be compared, and
// prefetching measured slower there: they run the first variant.
// ---------------------------------------------------------------------------
struct UnionVariant {
    uint32_t pf, pd, occ, staged;
};
// The window kernel with plain loads, L1 prefetch, 4 blocks per SM, both,
// L2 prefetch, 2 blocks per SM with two counter loads in flight per light
// lane (occ 2); the staged kernel (standard iterations) with the successor
// ids staged (staged 1) or read from global memory (staged 2), at 3 and 4
// blocks per SM.
constexpr UnionVariant kVariants[] = {{0, 0, 0, 0}, {2, 2, 0, 0}, {0, 0, 1, 0}, {2, 2, 1, 0},
                                      {1, 4, 0, 0}, {0, 0, 0, 1}, {0, 0, 1, 1}, {0, 0, 0, 2},
                                      {0, 0, 1, 2}, {0, 0, 2, 0}};
constexpr int kNumVariants = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
constexpr int kTunedClasses = 2;  // gather-all standard, filtered standard
constexpr uint64_t kTuneMinArcs = 1ull << 22;  // smaller graphs keep the first variant
constexpr double kTuneMargin = 0.97;

struct Tuner {
    int fixed = -1;                            // a variant forced by the options
    int chosen[kTunedClasses] = {-1, -1};
    double best[kTunedClasses][kNumVariants] = {};
    bool timed[kTunedClasses][kNumVariants] = {};
    int last = 0;                              // the variant of the iteration in flight
    int last_class = -1;                       // its class when it is a sample, else -1
};

struct TuneKey {
    int device, log2m;
    uint64_t n, m;
    bool operator<(const TuneKey& o) const {
        return std::tie(device, log2m, n, m) < std::tie(o.device, o.log2m, o.n, o.m);
    }
};
static std::mutex g_tune_mu;
static std::map<TuneKey, std::array<int, kTunedClasses>> g_tune_cache;

// The shape of an iteration: everything that fixes the arguments of its
// launches (state parities, mode, union-kernel variant).
struct GraphKey {
    int cur, mbc_cur;
    bool systolic, first_systolic, gather_all;
    int variant;
    bool operator==(const GraphKey& o) const {
        return cur == o.cur && mbc_cur == o.mbc_cur && systolic == o.systolic &&
               first_systolic == o.first_systolic && gather_all == o.gather_all && variant == o.variant;
    }
};

struct GraphEntry {
    GraphKey key;
    cudaGraphExec_t exec;
    uint64_t launches;  // kernels one launch of it runs
};
constexpr size_t kMaxGraphs = 32;

struct hb_handle {
    // configuration
    int device = 0;
    cudaStream_t stream = nullptr;
    // the heavy-node kernel runs here, beside the window kernel
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    uint64_t n = 0, m = 0;
    int log2m = 4;
    uint64_t counter_bytes = 0;   // the reference's packed counter size, 2^log2m * 5 / 8
    uint64_t stride = 0;          // device bytes per counter: one byte per register
    int hash_kind = HB_HASH_SIP13;
    uint64_t hash_seed = 0;
    uint64_t num_elements = 0;
    bool do_sod = false, do_harm = false, quirk = true;
    bool has_transpose = false;
    uint64_t arc_granularity = 16 * 1024;
    uint32_t small_max = 0, medium_max = 0;
    double alpha_m_m = 0.0;
    std::vector<hb_discount_fn> disc_fn;
    std::vector<void*> disc_ctx;
    uint64_t weight_seed = 0;
    bool has_weights = false;

    // device state
    std::vector<DevBuf> bufs;
    uint64_t* d_off = nullptr;
    uint32_t* d_succ = nullptr;
    uint64_t* d_toff = nullptr;
    uint32_t* d_tsucc = nullptr;
    uint8_t* d_cnt[2] = {nullptr, nullptr};
    uint32_t* d_bits[4] = {nullptr, nullptr, nullptr, nullptr};  // curr_mod, next_mod, mbc, next_mbc
    double* d_est = nullptr;
    double* d_sod = nullptr;
    double* d_harm = nullptr;
    std::vector<double*> d_disc;
    double* d_lnt = nullptr;
    uint64_t* d_weights = nullptr;
    uint32_t* d_tiles = nullptr;  // window boundaries
    uint32_t* d_arc_tiles = nullptr;  // creation only: first node of each arc tile of d_off
    // TMA descriptors of d_cnt[0] / d_cnt[1] for the far gathers, when usable
    CUtensorMap far_map[2];
    bool far_ok = false;
    uint32_t far_rows = 8192;
    uint32_t far_polls = 0;       // hb_debug_far_wait: poll limit (0: default)
    uint32_t far_extra_tx = 0;    // hb_debug_far_wait: bytes that never arrive
    uint64_t n_tiles = 0;         // number of windows
    uint2* d_chunks = nullptr;      // work units of the union kernel, in node order
    uint32_t* d_indeg = nullptr;    // in-degree without self-loops
    std::vector<uint64_t> inst_start; // batch: instance starts (caller ids), then num_nodes
    uint32_t* d_hash_id = nullptr;    // batch: device node -> its instance's own id
    uint64_t* d_inst_start = nullptr;
    uint32_t* d_inst_chunk = nullptr;  // batch: first chunk of each instance, then n_chunks
    uint32_t* d_queue = nullptr;       // batch: chunks of the running instances (standard iterations)
    uint32_t* d_queue_len = nullptr;
    unsigned long long* d_q_cnt = nullptr;  // batch: queue construction, instances + 1
    uint64_t* d_q_at = nullptr;
    unsigned long long* d_q_scratch = nullptr;
    uint64_t q_scratch_len = 0;
    unsigned long long* d_inst_mod = nullptr;
    double* d_inst_nf = nullptr;
    std::vector<unsigned long long> inst_mod;    // last iteration, per instance
    std::vector<double> inst_sum;                // last iteration, per instance
    std::vector<uint64_t> inst_iters;            // iterations run so far
    std::vector<uint8_t> inst_done;              // stopped (HB:559-570)
    std::vector<std::vector<double>> inst_nf;    // neighbourhood function per instance
    uint64_t self_loops = 0;
    uint64_t pending_visited = 0;   // arcs the next iteration visits
    uint32_t* d_perm = nullptr;     // device node -> caller node
    uint32_t* d_inv = nullptr;      // caller node -> device node
    uint64_t n_chunks = 0;
    uint32_t* d_light_bits = nullptr;           // light nodes (device ids)
    uint32_t* d_medium_bits = nullptr;          // medium nodes (device ids)
    unsigned long long* d_word_cnt = nullptr;   // systolic lists: per bitmap word counts
    uint64_t* d_word_off = nullptr;             // their exclusive prefix sum (+ totals)
    unsigned long long* d_list_scratch = nullptr;
    uint64_t list_scratch_len = 0;
    uint32_t* d_light_list = nullptr;           // systolic: light nodes to check or copy
    uint32_t* d_medium_list = nullptr;          // systolic: medium nodes to check or copy
    uint32_t* d_heavy = nullptr;
    uint64_t n_heavy = 0;
    uint4* d_heavy_items = nullptr;     // heavy-kernel items (whole nodes or segments)
    uint64_t n_heavy_items = 0;
    uint8_t* d_heavy_part = nullptr;    // partial counters of split nodes' segments
    uint32_t* d_heavy_arrive = nullptr; // arrival counts of split nodes
    hbk::TilePartial* d_partials = nullptr;  // one per tile, then one per heavy block
    uint64_t n_partials = 0;
    double* d_nf_items = nullptr;     // neighbourhood-function part per work item / heavy node
    double* d_nf_scratch = nullptr;
    unsigned long long* d_cursor = nullptr;  // chunk cursor of the union kernel
    int* d_any31 = nullptr;
    bool any31 = false;
    int grid_tile = 1, grid_heavy = 1, grid_mark = 1;
    int grid_tile_occ = 1;           // the window kernel's grid in its 4-blocks-per-SM variant
    int grid_tile_two = 1;           // ... and in its 2-blocks-per-SM variant
    int grid_staged = 1, grid_staged_occ = 1;  // the staged kernel's grids
    uint4* d_items = nullptr;        // item table of the staged kernel (null: not usable)
    Tuner tuner;
    // iterations as CUDA graphs: captured on `cap`, launched on `stream`
    bool use_graphs = true;
    bool capture_in_run = false;        // batches: capture a shape the second time it comes
    cudaStream_t cap = nullptr;
    std::vector<GraphEntry> graphs;
    std::vector<GraphKey> shapes_run;   // iteration shapes of the current run
    std::vector<GraphKey> shapes_seen;  // ... of the earlier runs of this handle
    hbk::IterConsts* d_ic = nullptr;           // this iteration's constants (device)
    hbk::IterConsts* h_ic = nullptr;           // ... staged in page-locked host memory
    hbk::TilePartial* h_tot = nullptr;         // the iteration's totals (page-locked)
    unsigned long long* h_inst_mod = nullptr;  // batches: per instance (page-locked)
    double* h_inst_sum = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

    // reference state (IterationContext + HyperBall fields)
    int cur = 0;         // index of the current counter array
    int mod_cur = 0;     // d_bits[mod_cur] = curr_mod, d_bits[mod_cur ^ 1] = next_mod
    int mbc_cur = 2;     // d_bits[mbc_cur] = mbc, d_bits[mbc_cur ^ 1] = next_mbc
    uint64_t iteration = 0;
    uint64_t launches = 0;          // kernels launched for this handle
    bool systolic = false, local = false, pre_local = false;
    uint64_t modified_counters = 0;
    double last = 0.0, relative_increment = 0.0;
    std::vector<double> nf;
    std::vector<hb_iter_stats> stats;
    bool initialised = false;

    std::string err;
};

namespace {

int set_err(hb_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    g_global_err = msg;
    return code;
}

int cuda_err(hb_handle* h, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return HB_OK;
    int code = (e == cudaErrorMemoryAllocation) ? HB_ERR_OOM
               : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? HB_ERR_NO_DEVICE
                                                                               : HB_ERR_CUDA;
    return set_err(h, code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define HB_CUDA(h, call)                                          \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_err((h), _e, #call);   \
    } while (0)

#define HB_LAUNCH(h, call)                                                    \
    do {                                                                      \
        int _e = (call);                                                      \
        if (_e != 0) return cuda_err((h), (cudaError_t)_e, #call);            \
    } while (0)

// NVTX range for the scope (iterations, steps, creation): visible in a
// profiler's timeline, free without one
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

// hb_debug_fail_allocations: the device allocation of a handle that brings
// this count to zero fails (once); -1: none
std::atomic<long long> g_fail_alloc_after{-1};

template <class T>
int dalloc(hb_handle* h, T** out, size_t count) {
    *out = nullptr;
    if (g_fail_alloc_after.load(std::memory_order_relaxed) >= 0 &&
        g_fail_alloc_after.fetch_sub(1) == 0)
        return set_err(h, HB_ERR_OOM, "device allocation failed (injected by hb_debug_fail_allocations)");
    size_t bytes = std::max<size_t>(count * sizeof(T), 256);
    void* p = nullptr;
    // stream-ordered: freeing never synchronises the whole device, so other
    // work (other handles, other jobs of a server) keeps running. The block
    // is valid in the handle's stream order; creation and hb_init end with a
    // synchronisation before any other stream uses it. (A synchronisation
    // after every allocation cost a served job's creation up to one step of
    // the other jobs per allocation: its stream waits for SMs the shared
    // union launch holds.)
    cudaError_t e = pool_alloc(h->device, &p, bytes, h->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_err(h, e, "cudaMallocFromPoolAsync");
    }
    h->bufs.push_back({p, bytes});
    *out = (T*)p;
    return HB_OK;
}

void release(hb_handle* h) {
    if (!h) return;
    for (auto& b : h->bufs) cudaFreeAsync(b.p, h->stream);
    cudaStreamSynchronize(h->stream);
    h->bufs.clear();
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    if (h->fork) cudaEventDestroy(h->fork);
    if (h->join) cudaEventDestroy(h->join);
    if (h->side) cudaStreamDestroy(h->side);
    for (GraphEntry& g : h->graphs) cudaGraphExecDestroy(g.exec);
    h->graphs.clear();
    if (h->cap) cudaStreamDestroy(h->cap);
    const size_t ni = h->inst_start.empty() ? 1 : std::max<size_t>(h->inst_start.size() - 1, 1);
    pinned_free(h->h_ic, sizeof(hbk::IterConsts));
    pinned_free(h->h_tot, sizeof(hbk::TilePartial));
    pinned_free(h->h_inst_mod, ni * 8);
    pinned_free(h->h_inst_sum, ni * 8);
    h->h_ic = nullptr;
    h->h_tot = nullptr;
    h->h_inst_mod = nullptr;
    h->h_inst_sum = nullptr;
}

// Static work order of the union kernels (the graph does not change), and the
// node renumbering that follows it. Nodes are cut into segments of at most
// `win_nodes` consecutive ids, which also end at every instance boundary of a
// batch (h->inst_start: sorted instance starts, or empty); inside a segment
// the heavy nodes (out-degree > medium_max), the medium nodes (small_max <
// out-degree <= medium_max) and the light nodes (out-degree <= small_max)
// take the segment's ids in that order, each kind by decreasing out-degree,
// ties by id: perm[new] = caller id, inv[caller] = new. Renumbering never
// leaves a segment, so an instance keeps its id range. The light and medium
// runs are cut into chunks of one warp-step (`per_light` or `per_medium`
// nodes); heavy nodes are listed by decreasing degree, ties in id order;
// light / medium bitmaps mark the light / medium nodes (device ids). The
// segment cuts are made on the host, everything per node on the device from
// the uploaded offsets `off0` (caller ids).
void dfree(hb_handle* h, void* p);

int device_partition(hb_handle* h, const uint64_t* off0, uint32_t win_nodes, uint32_t per_light,
                     uint32_t per_medium) {
    const uint64_t n = h->n;
    const std::vector<uint64_t>& bounds = h->inst_start;
    std::vector<uint32_t> seg, base;
    {
        size_t bi = 0;
        uint64_t inst0 = 0;
        for (uint64_t w0 = 0; w0 < n;) {
            while (bi < bounds.size() && bounds[bi] <= w0) inst0 = bounds[bi++];
            uint64_t w1 = std::min<uint64_t>(n, w0 + win_nodes);
            if (bi < bounds.size() && bounds[bi] < w1) w1 = bounds[bi];
            seg.push_back((uint32_t)w0);
            base.push_back((uint32_t)inst0);
            w0 = w1;
        }
        seg.push_back((uint32_t)n);
    }
    const uint64_t nseg = seg.size() - 1;
    const uint64_t words = (n + 31) / 32;
    int r;
    h->n_tiles = nseg;
    if ((r = dalloc(h, &h->d_tiles, seg.size()))) return r;
    if ((r = dalloc(h, &h->d_perm, n))) return r;
    if ((r = dalloc(h, &h->d_inv, n))) return r;
    if ((r = dalloc(h, &h->d_light_bits, words))) return r;
    if ((r = dalloc(h, &h->d_medium_bits, words))) return r;
    const bool batch = !bounds.empty();
    uint32_t* d_base = nullptr;
    if (batch) {
        if ((r = dalloc(h, &h->d_hash_id, n))) return r;
        if ((r = dalloc(h, &d_base, base.size()))) return r;
        HB_CUDA(h, cudaMemcpyAsync(d_base, base.data(), base.size() * 4, cudaMemcpyHostToDevice,
                                   h->stream));
    }
    HB_CUDA(h, cudaMemcpyAsync(h->d_tiles, seg.data(), seg.size() * 4, cudaMemcpyHostToDevice,
                               h->stream));
    HB_CUDA(h, cudaMemsetAsync(h->d_light_bits, 0, words * 4, h->stream));
    HB_CUDA(h, cudaMemsetAsync(h->d_medium_bits, 0, words * 4, h->stream));
    unsigned long long *seg_chunks = nullptr, *seg_heavy = nullptr, *scratch = nullptr;
    uint64_t *chunk_at = nullptr, *heavy_at = nullptr;
    const uint64_t sl = hbk::scan_scratch_len(nseg + 1);
    if ((r = dalloc(h, &seg_chunks, nseg + 1))) return r;
    if ((r = dalloc(h, &seg_heavy, nseg + 1))) return r;
    if ((r = dalloc(h, &chunk_at, nseg + 1))) return r;
    if ((r = dalloc(h, &heavy_at, nseg + 1))) return r;
    if ((r = dalloc(h, &scratch, sl))) return r;
    HB_LAUNCH(h, hbk::launch_part_count(off0, h->d_tiles, nseg, h->small_max, h->medium_max, per_light,
                                        per_medium, seg_chunks, seg_heavy, h->stream));
    HB_LAUNCH(h, hbk::launch_exclusive_scan_u64(seg_chunks, chunk_at, nseg + 1, scratch, sl, h->stream));
    HB_LAUNCH(h, hbk::launch_exclusive_scan_u64(seg_heavy, heavy_at, nseg + 1, scratch, sl, h->stream));
    uint64_t totals[2] = {0, 0};
    HB_CUDA(h, cudaMemcpyAsync(&totals[0], chunk_at + nseg, 8, cudaMemcpyDeviceToHost, h->stream));
    HB_CUDA(h, cudaMemcpyAsync(&totals[1], heavy_at + nseg, 8, cudaMemcpyDeviceToHost, h->stream));
    HB_CUDA(h, cudaStreamSynchronize(h->stream));
    h->n_chunks = totals[0];
    h->n_heavy = totals[1];
    unsigned long long* heavy_keys = nullptr;
    if ((r = dalloc(h, &h->d_chunks, h->n_chunks))) return r;
    if ((r = dalloc(h, &heavy_keys, h->n_heavy))) return r;
    HB_LAUNCH(h, hbk::launch_part_place(off0, h->d_tiles, nseg, h->small_max, h->medium_max, per_light,
                                        per_medium, (const unsigned long long*)chunk_at,
                                        (const unsigned long long*)heavy_at, d_base, h->d_perm,
                                        h->d_inv, h->d_chunks, heavy_keys, h->d_light_bits,
                                        h->d_medium_bits, h->d_hash_id, h->stream));
    if (h->n_heavy) {
        // all heavy nodes by decreasing degree, ties in segment order (few
        // nodes: sorted on the host)
        std::vector<unsigned long long> keys(h->n_heavy);
        HB_CUDA(h, cudaMemcpyAsync(keys.data(), heavy_keys, h->n_heavy * 8, cudaMemcpyDeviceToHost,
                                   h->stream));
        HB_CUDA(h, cudaStreamSynchronize(h->stream));
        std::sort(keys.begin(), keys.end());
        std::vector<uint32_t> heavy(h->n_heavy);
        for (uint64_t i = 0; i < h->n_heavy; i++) heavy[i] = (uint32_t)keys[i];
        if ((r = dalloc(h, &h->d_heavy, h->n_heavy))) return r;
        HB_CUDA(h, cudaMemcpyAsync(h->d_heavy, heavy.data(), h->n_heavy * 4, cudaMemcpyHostToDevice,
                                   h->stream));
        // heavy-kernel items: a node of more than HEAVY_SPLIT arcs becomes
        // segments of HEAVY_SEG arcs; items by decreasing arcs (ties in list
        // order), so the longest start first. The key holds 2^32 - 1 - degree.
        struct Item {
            uint64_t arcs;
            uint32_t hi, seg, nseg, slot;
        };
        std::vector<Item> items;
        uint32_t slots = 0;
        for (uint64_t i = 0; i < h->n_heavy; i++) {
            const uint64_t d = 0xffffffffull - (keys[i] >> 32);
            if (d > hbk::HEAVY_SPLIT) {
                const uint32_t nseg = (uint32_t)((d + hbk::HEAVY_SEG - 1) / hbk::HEAVY_SEG);
                for (uint32_t k = 0; k < nseg; k++)
                    items.push_back({std::min<uint64_t>(hbk::HEAVY_SEG, d - (uint64_t)k * hbk::HEAVY_SEG),
                                     (uint32_t)i, k, nseg, slots});
                slots += nseg;
            } else {
                items.push_back({d, (uint32_t)i, 0, 1, 0});
            }
        }
        std::stable_sort(items.begin(), items.end(),
                         [](const Item& x, const Item& y) { return x.arcs > y.arcs; });
        std::vector<uint4> table(items.size());
        for (size_t k = 0; k < items.size(); k++)
            table[k] = make_uint4(items[k].hi, items[k].seg, items[k].nseg, items[k].slot);
        h->n_heavy_items = table.size();
        if ((r = dalloc(h, &h->d_heavy_items, table.size()))) return r;
        HB_CUDA(h, cudaMemcpyAsync(h->d_heavy_items, table.data(), table.size() * sizeof(uint4),
                                   cudaMemcpyHostToDevice, h->stream));
        if (slots) {
            if ((r = dalloc(h, &h->d_heavy_part, (size_t)slots * h->stride))) return r;
            if ((r = dalloc(h, &h->d_heavy_arrive, slots))) return r;
            HB_CUDA(h, cudaMemsetAsync(h->d_heavy_arrive, 0, (size_t)slots * 4, h->stream));
        }
        // host copies are read by the copies above before they return
        HB_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    HB_CUDA(h, cudaStreamSynchronize(h->stream));
    for (void* p : {(void*)seg_chunks, (void*)seg_heavy, (void*)chunk_at, (void*)heavy_at,
                    (void*)scratch, (void*)heavy_keys, (void*)d_base})
        if (p) dfree(h, p);
    return HB_OK;
}

bool check_view(const hb_graph_view* g, std::string& why) {
    if (!g) {
        why = "graph is NULL";
        return false;
    }
    if (g->num_nodes > 0xffffffffull) {
        why = "more than 2^32 nodes do not fit u32 successors";
        return false;
    }
    if (!g->offsets) {
        why = "offsets is NULL";
        return false;
    }
    if (g->num_arcs > 0 && !g->successors) {
        why = "successors is NULL";
        return false;
    }
    if (g->offsets[0] != 0 || g->offsets[g->num_nodes] != g->num_arcs) {
        why = "offsets[0] must be 0 and offsets[num_nodes] must equal num_arcs";
        return false;
    }
    return true;
}

int upload_csr(hb_handle* h, const hb_graph_view* g, uint64_t** d_off, uint32_t** d_succ) {
    int r;
    // HB_TRACE: the allocations' host time and the copies' device time
    const bool trace = std::getenv("HB_TRACE") != nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    if ((r = dalloc(h, d_off, g->num_nodes + 1))) return r;
    if ((r = dalloc(h, d_succ, g->num_arcs))) return r;
    const auto t1 = std::chrono::steady_clock::now();
    if (trace) cudaEventRecord(h->ev[0], h->stream);
    HB_CUDA(h, cudaMemcpyAsync(*d_off, g->offsets, (g->num_nodes + 1) * 8, cudaMemcpyHostToDevice,
                               h->stream));
    if (g->num_arcs)
        HB_CUDA(h, cudaMemcpyAsync(*d_succ, g->successors, g->num_arcs * 4, cudaMemcpyHostToDevice,
                                   h->stream));
    if (trace) {
        cudaEventRecord(h->ev[1], h->stream);
        cudaEventSynchronize(h->ev[1]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
        std::fprintf(stderr, "hb_create   allocations %.2f ms (host), copies %.2f ms (device), %.2f ms (host)\n",
                     std::chrono::duration<double, std::milli>(t1 - t0).count(), ms,
                     std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count());
    }
    // reject decreasing offsets before any kernel sizes work by them (the
    // successors are checked where they are renumbered)
    int* d_bad = nullptr;
    if ((r = dalloc(h, &d_bad, 1))) return r;
    HB_CUDA(h, cudaMemsetAsync(d_bad, 0, sizeof(int), h->stream));
    HB_LAUNCH(h, hbk::launch_validate(*d_off, *d_succ, g->num_nodes, 0, d_bad, h->stream));
    int bad = 0;
    HB_CUDA(h, cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    HB_CUDA(h, cudaStreamSynchronize(h->stream));
    dfree(h, d_bad);
    if (bad) return set_err(h, HB_ERR_INVALID, "graph has decreasing offsets");
    return HB_OK;
}

// Frees one buffer of the handle before its end of life.
void dfree(hb_handle* h, void* p) {
    for (auto it = h->bufs.begin(); it != h->bufs.end(); ++it)
        if (it->p == p) {
            // stream-ordered: later allocations reuse the block after the
            // work before this point (no synchronisation)
            cudaFreeAsync(p, h->stream);
            h->bufs.erase(it);
            return;
        }
}

// CSR (caller ids) -> CSR of the renumbered graph: node i is caller node
// perm[i], successor u becomes inv[u].
// The renumbered CSR of a caller CSR (off0 / succ0, offsets checked): row i
// is caller row perm[i], targets mapped through inv; out-of-range targets are
// an error. With indeg (zeroed), the same pass counts the in-degrees without
// self-loops, the self-loops into *loops and, with trows (zeroed), each node's
// self-loops. With arc_tiles, the arc tiles of the result are returned there
// (to be freed by the caller).
int relabel_csr(hb_handle* h, const uint64_t* off0, const uint32_t* succ0, uint64_t** d_off,
                uint32_t** d_succ, uint32_t* indeg, unsigned long long* loops,
                unsigned long long* trows, uint32_t** arc_tiles) {
    const uint64_t n = h->n, m = h->m;
    int r;
    unsigned long long* deg = nullptr;
    unsigned long long* scratch = nullptr;
    uint32_t* tiles = nullptr;
    int* bad = nullptr;
    const uint64_t sl = hbk::scan_scratch_len(n + 1);
    if ((r = dalloc(h, d_off, n + 1))) return r;
    // padded: the staged kernel copies successor ids in aligned 16-byte units
    if ((r = dalloc(h, d_succ, m + 8))) return r;
    HB_CUDA(h, cudaMemsetAsync(*d_succ + m, 0, 8 * sizeof(uint32_t), h->stream));
    if ((r = dalloc(h, &deg, n + 1))) return r;
    if ((r = dalloc(h, &scratch, sl))) return r;
    if ((r = dalloc(h, &tiles, hbk::arc_tiles(m) + 1))) return r;
    if ((r = dalloc(h, &bad, 1))) return r;
    HB_CUDA(h, cudaMemsetAsync(bad, 0, sizeof(int), h->stream));
    HB_LAUNCH(h, hbk::launch_perm_degree(off0, h->d_perm, n, deg, h->stream));
    HB_LAUNCH(h, hbk::launch_exclusive_scan_u64(deg, *d_off, n + 1, scratch, sl, h->stream));
    HB_LAUNCH(h, hbk::launch_tile_start(*d_off, n, tiles, h->stream));
    HB_LAUNCH(h, hbk::launch_relabel_arcs(*d_off, n, m, tiles, h->d_perm, off0, succ0, h->d_inv, *d_succ,
                                          indeg, loops, trows, bad, h->stream));
    int bad_host = 0;
    HB_CUDA(h, cudaMemcpyAsync(&bad_host, bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    HB_CUDA(h, cudaStreamSynchronize(h->stream));
    dfree(h, deg);
    dfree(h, scratch);
    dfree(h, bad);
    if (arc_tiles)
        *arc_tiles = tiles;
    else
        dfree(h, tiles);
    if (bad_host) return set_err(h, HB_ERR_INVALID, "graph has successors >= num_nodes");
    return HB_OK;
}

// Transpose of a device CSR (n nodes, m arcs) into toff[n + 1] / tsucc[m]:
// in-degrees into `cursor` (n + 1 words, zeroed here), exclusive scan into
// toff (`scan`: scan_scratch_len(n + 1) words), scatter with `cursor` as the
// per-row write position. Rows of the result are in no particular order.
cudaError_t transpose_core(const uint64_t* off, const uint32_t* succ, uint64_t n, uint64_t m,
                           uint64_t* toff, uint32_t* tsucc, unsigned long long* cursor,
                           unsigned long long* scan, uint64_t scan_len, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(cursor, 0, (n + 1) * 8, s);
    if (e != cudaSuccess) return e;
    int r = m ? hbk::launch_transpose_count(succ, m, cursor, s) : 0;
    if (!r) r = hbk::launch_exclusive_scan_u64(cursor, toff, n + 1, scan, scan_len, s);
    if (r || n == 0 || m == 0) return (cudaError_t)r;
    e = cudaMemcpyAsync(cursor, toff, n * 8, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    return (cudaError_t)hbk::launch_transpose_scatter(off, succ, n, cursor, tsucc, s);
}

// The transpose of the renumbered graph; `rows` (n + 1 words) holds each
// node's self-loops (from the renumbering pass), to which the in-degrees
// without self-loops are added; the scatter walks the arc tiles of the
// renumbering. `rows` is released here.
int build_transpose_on_device(hb_handle* h, unsigned long long* rows) {
    const uint64_t n = h->n, m = h->m;
    int r;
    if ((r = dalloc(h, &h->d_toff, n + 1))) return r;
    if ((r = dalloc(h, &h->d_tsucc, m))) return r;
    const uint64_t sl = hbk::scan_scratch_len(n + 1);
    unsigned long long* scratch = nullptr;
    if ((r = dalloc(h, &scratch, sl))) return r;
    HB_LAUNCH(h, hbk::launch_add_indeg(rows, h->d_indeg, n, h->stream));
    HB_LAUNCH(h, hbk::launch_exclusive_scan_u64(rows, h->d_toff, n + 1, scratch, sl, h->stream));
    if (n && m) {
        HB_CUDA(h, cudaMemcpyAsync(rows, h->d_toff, n * 8, cudaMemcpyDeviceToDevice, h->stream));
        HB_LAUNCH(h, hbk::launch_scatter_arcs(h->d_off, n, m, h->d_arc_tiles, h->d_succ, rows, h->d_tsucc,
                                              h->stream));
    }
    HB_CUDA(h, cudaStreamSynchronize(h->stream));
    // temporaries are released right away
    dfree(h, rows);
    dfree(h, scratch);
    h->has_transpose = true;
    return HB_OK;
}

hbk::UnionArgs union_args(hb_handle* h) {
    hbk::UnionArgs a{};
    a.off = h->d_off;
    a.succ = h->d_succ;
    a.curr = h->d_cnt[h->cur];
    a.next = h->d_cnt[h->cur ^ 1];
    a.curr_mod = h->d_bits[h->mod_cur];
    a.next_mod = h->d_bits[h->mod_cur ^ 1];
    a.mbc = h->d_bits[h->mbc_cur];
    a.est = h->d_est;
    a.sod = h->d_sod;
    a.harm = h->d_harm;
    a.ndisc = (int)h->d_disc.size();
    for (int k = 0; k < a.ndisc; k++) a.disc[k] = h->d_disc[k];
    a.ic = h->d_ic;
    a.systolic = h->systolic ? 1 : 0;
    a.quirk = h->quirk ? 1 : 0;
    a.any31 = h->any31 ? 1 : 0;
    a.n = h->n;
    a.alpha_m_m = h->alpha_m_m;
    a.a_scaled = h->alpha_m_m * 2147483648.0;  // exact: power-of-two scaling
    {
        const double small = 2.5 * (double)(1ull << h->log2m);
        long long bits;
        std::memcpy(&bits, &small, sizeof bits);
        a.small_bits = bits;
    }
    a.ln_table = h->d_lnt;
    a.tiles = h->d_tiles;
    a.n_tiles = (uint32_t)h->n_tiles;
    a.light_list = nullptr;
    a.medium_list = nullptr;
    a.list_counts = nullptr;
    a.chunks = h->d_chunks;
    a.items = h->d_items;
    a.staged = 0;
    a.gather_all = 0;
    a.indeg = h->d_indeg;
    a.nf_items = h->d_nf_items;
    a.heavy_item_base = h->n_chunks;
    a.n_chunks = h->n_chunks;
    a.tile_max_degree = h->medium_max;
    a.acc_slot = (uint32_t)(h->n_partials - 1);
    a.cursor = h->d_cursor;
    a.partials = h->d_partials;
    a.far_tma = h->far_ok ? 1 : 0;
    a.far_rows = h->far_rows;
    a.mbar_polls = h->far_polls;
    a.test_extra_tx = h->far_extra_tx;
    a.pf = 0;
    a.pd = 0;
    a.occ = 0;
    if (h->far_ok) a.far_map = h->far_map[h->cur];
    return a;
}

// Adds the kernels launched by this thread during its lifetime to h->launches.
struct LaunchTally {
    hb_handle* h;
    uint64_t c0;
    explicit LaunchTally(hb_handle* hh) : h(hh), c0(hbk::launch_count()) {}
    ~LaunchTally() { h->launches += hbk::launch_count() - c0; }
};

// The union-kernel variant of the next iteration. `cls`: 0 standard merging
// every successor, 1 standard merging modified successors, -1 systolic;
// `sample`: the iteration is large and typical enough to time a variant on.
int choose_variant(hb_handle* h, int cls, bool sample) {
    Tuner& t = h->tuner;
    t.last_class = -1;
    if (t.fixed >= 0) return t.last = t.fixed;
    if (h->far_ok) return t.last = 0;  // the TMA-gather kernel is its own opt-in variant
    if (cls < 0) return t.last = 0;
    if (t.chosen[cls] >= 0) return t.last = t.chosen[cls];
    if (sample)
        for (int v = 0; v < kNumVariants; v++)
            if (!t.timed[cls][v]) {
                t.last_class = cls;
                return t.last = v;
            }
    return t.last = 0;
}

// Records the union time per scanned-plus-merged arc of a sampled iteration;
// once every variant of the class has a time, keeps the fastest.
void record_variant(hb_handle* h, double union_ms, uint64_t arcs) {
    Tuner& t = h->tuner;
    const int cls = t.last_class;
    if (cls < 0 || arcs == 0) return;
    t.best[cls][t.last] = union_ms / (double)arcs;
    t.timed[cls][t.last] = true;
    int best = 0;
    for (int v = 0; v < kNumVariants; v++) {
        if (!t.timed[cls][v]) return;
        if (t.best[cls][v] < t.best[cls][best]) best = v;
    }
    // one sample each: another variant must beat the first by a clear margin
    if (t.best[cls][best] > kTuneMargin * t.best[cls][0]) best = 0;
    t.chosen[cls] = best;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto& e = g_tune_cache.try_emplace(TuneKey{h->device, h->log2m, h->n, h->m},
                                       std::array<int, kTunedClasses>{-1, -1})
                  .first->second;
    e[cls] = best;
}

int do_init(hb_handle* h) {
    const uint64_t n = h->n;
    HB_CUDA(h, cudaMemsetAsync(h->d_cnt[0], 0, n * h->stride, h->stream));
    HB_CUDA(h, cudaMemsetAsync(h->d_cnt[1], 0, n * h->stride, h->stream));
    h->cur = 0;
    h->mod_cur = 0;
    h->mbc_cur = 2;
    // every counter is modified at init, so iteration 1 visits every non-loop arc
    h->pending_visited = h->m - h->self_loops;
    hbk::InitArgs ia{};
    ia.perm = h->d_perm;
    ia.hash_id = h->d_hash_id;
    ia.curr = h->d_cnt[0];
    ia.est = h->d_est;
    ia.n = n;
    ia.hash_kind = h->hash_kind;
    ia.seed = h->hash_seed;
    ia.weights = h->d_weights;
    ia.weight_seed = h->weight_seed;
    ia.alpha_m_m = h->alpha_m_m;
    ia.ln_table = h->d_lnt;
    ia.quirk = h->quirk ? 1 : 0;
    ia.any31 = h->d_any31;
    HB_CUDA(h, cudaMemsetAsync(h->d_any31, 0, sizeof(int), h->stream));
    if (n) HB_LAUNCH(h, hbk::launch_init(h->log2m, ia, h->stream));
    int any31 = 0;
    HB_CUDA(h, cudaMemcpyAsync(&any31, h->d_any31, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (h->d_sod) HB_CUDA(h, cudaMemsetAsync(h->d_sod, 0, n * 8, h->stream));
    if (h->d_harm) HB_CUDA(h, cudaMemsetAsync(h->d_harm, 0, n * 8, h->stream));
    for (double* d : h->d_disc) HB_CUDA(h, cudaMemsetAsync(d, 0, n * 8, h->stream));
    const uint64_t words = (n + 31) / 32;
    // curr_modified = all ones (HB:1208); bits beyond n stay zero
    HB_LAUNCH(h, hbk::launch_fill_u32(h->d_bits[0], 0xffffffffu, words, h->stream));
    if (n % 32) {
        uint32_t last = (1u << (n % 32)) - 1u;
        HB_CUDA(h, cudaMemcpyAsync(h->d_bits[0] + words - 1, &last, 4, cudaMemcpyHostToDevice,
                                   h->stream));
    }
    for (int b = 1; b < 4; b++) HB_CUDA(h, cudaMemsetAsync(h->d_bits[b], 0, words * 4, h->stream));
    // every batch instance runs in the first iteration (the queue keeps
    // instances whose modified count of the previous iteration is nonzero)
    if (h->d_inst_mod)
        HB_CUDA(h, cudaMemsetAsync(h->d_inst_mod, 0xff, (h->inst_start.size() - 1) * 8, h->stream));
    HB_CUDA(h, cudaStreamSynchronize(h->stream));
    h->any31 = any31 != 0;
    h->iteration = 0;
    h->systolic = h->local = h->pre_local = false;
    h->modified_counters = 0;
    h->last = (double)n;
    h->relative_increment = 0.0;
    h->nf.assign(1, h->last);
    h->stats.clear();
    const size_t ni = h->inst_start.empty() ? 0 : h->inst_start.size() - 1;
    h->inst_iters.assign(ni, 0);
    h->inst_done.assign(ni, 0);
    h->inst_nf.assign(ni, std::vector<double>());
    for (size_t i = 0; i < ni; i++) {
        const uint64_t ni_nodes = h->inst_start[i + 1] - h->inst_start[i];
        h->inst_nf[i].assign(1, (double)ni_nodes);
        // run() caps the iterations at the number of nodes (HB:541)
        h->inst_done[i] = ni_nodes == 0;
    }
    // a new run: the shapes of the last one may now be captured
    for (const GraphKey& k : h->shapes_run)
        if (std::find(h->shapes_seen.begin(), h->shapes_seen.end(), k) == h->shapes_seen.end())
            h->shapes_seen.push_back(k);
    h->shapes_run.clear();
    h->initialised = true;
    return HB_OK;
}

// An iteration's launches in three parts: enqueue_pre (clears, the systolic
// work lists, a batch's queue of running instances; fills a's lists),
// enqueue_union (the union kernels of this handle alone) and enqueue_post
// (predecessor marks, the fixed-order NF sum, totals to the host). Several
// handles can run their pre and post parts around one shared union launch
// (multi_iterate).
int enqueue_pre(hb_handle* h, hbk::UnionArgs& a, bool first_systolic, cudaStream_t s,
                bool external) {
    const uint64_t n = h->n;
    const uint64_t words = (n + 31) / 32;
    auto rec = [&](cudaEvent_t e) {
        return external ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal) : cudaEventRecord(e, s);
    };
    HB_CUDA(h, rec(h->ev[0]));
    HB_CUDA(h, cudaMemsetAsync(h->d_bits[h->mod_cur ^ 1], 0, words * 4, s));
    if (h->systolic) {
        HB_CUDA(h, cudaMemsetAsync(h->d_bits[h->mbc_cur ^ 1], 0, words * 4, s));
        if (first_systolic) {
            // The reference scans every node in the first systolic iteration
            // (HB:853-857); scanning the predecessors of the nodes modified in
            // the previous iteration gives the same counters.
            HB_CUDA(h, cudaMemsetAsync(h->d_bits[h->mbc_cur], 0, words * 4, s));
            HB_LAUNCH(h, hbk::launch_mark_preds(h->d_bits[h->mod_cur], h->d_toff, h->d_tsucc,
                                                h->d_bits[h->mbc_cur], n, h->grid_mark, s));
        }
    }
    HB_CUDA(h, cudaMemsetAsync(h->d_partials, 0, h->n_partials * sizeof(hbk::TilePartial), s));
    HB_CUDA(h, cudaMemsetAsync(h->d_nf_items, 0, (h->n_chunks + h->n_heavy) * sizeof(double), s));
    HB_CUDA(h, cudaMemsetAsync(h->d_cursor, 0, sizeof(unsigned long long), s));
    // the per-iteration constants and, after the union, the totals move
    // between the pinned host blocks and the device by a small kernel, not by
    // the copy engines: a served job's step would otherwise queue behind the
    // other jobs' CSR uploads and result downloads
    HB_LAUNCH(h, hbk::launch_copy_u64(reinterpret_cast<const uint64_t*>(h->h_ic),
                                      reinterpret_cast<uint64_t*>(h->d_ic), sizeof(hbk::IterConsts) / 8, s));
    if (h->systolic && h->n_tiles) {
        // the light and medium nodes to check or to copy
        HB_LAUNCH(h, hbk::launch_work_lists(a.mbc, a.curr_mod, h->d_medium_bits, h->d_light_bits, n,
                                            h->d_word_cnt, h->d_word_off, h->d_list_scratch,
                                            h->list_scratch_len, h->d_light_list,
                                            h->d_medium_list, s));
        a.light_list = h->d_light_list;
        a.medium_list = h->d_medium_list;
        a.list_counts = h->d_word_off + words;
    } else if (h->d_queue && h->n_tiles) {
        // a batch's standard iteration scans the instances still running
        const uint32_t ni = (uint32_t)(h->inst_start.size() - 1);
        HB_LAUNCH(h, hbk::launch_inst_queue(h->d_inst_chunk, h->d_inst_mod, ni, 0,
                                            (uint32_t)h->n_chunks, h->d_q_cnt, h->d_q_at,
                                            h->d_q_scratch, h->q_scratch_len, h->d_queue,
                                            h->d_queue_len, s));
        a.queue = h->d_queue;
        a.queue_len = h->d_queue_len;
        a.staged = 0;
    }
    HB_CUDA(h, rec(h->ev[1]));
    return HB_OK;
}

// The heavy-node kernel (side stream) and the window kernel of this handle.
int enqueue_union(hb_handle* h, const hbk::UnionArgs& a, cudaStream_t s, bool window) {
    if (h->n_heavy) {
        // The heavy nodes (one CTA each) start first on the side stream; the
        // window kernel's blocks take the SMs as they free up, so the long
        // heavy nodes overlap the window work instead of forming a tail.
        // They touch disjoint nodes; shared totals are atomics.
        hbk::UnionArgs ah = a;
        ah.list = h->d_heavy;
        ah.list_len = h->n_heavy;
        ah.heavy_items = h->d_heavy_items;
        ah.heavy_len = h->n_heavy_items;
        ah.heavy_part = h->d_heavy_part;
        ah.heavy_arrive = h->d_heavy_arrive;
        HB_CUDA(h, cudaEventRecord(h->fork, s));
        HB_CUDA(h, cudaStreamWaitEvent(h->side, h->fork, 0));
        HB_LAUNCH(h, hbk::launch_union_heavy(h->log2m, ah, h->grid_heavy, h->side));
        HB_CUDA(h, cudaEventRecord(h->join, h->side));
    }
    if (window && h->n_tiles && a.staged)
        HB_LAUNCH(h, hbk::launch_union_staged(h->log2m, a, a.occ ? h->grid_staged_occ : h->grid_staged, s));
    else if (window && h->n_tiles)
        HB_LAUNCH(h, hbk::launch_union_tile(h->log2m, a,
                                            a.occ == 2 ? h->grid_tile_two : a.occ ? h->grid_tile_occ : h->grid_tile,
                                            s));
    return HB_OK;
}

int enqueue_join(hb_handle* h, cudaStream_t s) {
    if (h->n_heavy) HB_CUDA(h, cudaStreamWaitEvent(s, h->join, 0));
    return HB_OK;
}

int enqueue_post(hb_handle* h, const hbk::UnionArgs& a, cudaStream_t s, bool external) {
    const uint64_t n = h->n;
    auto rec = [&](cudaEvent_t e) {
        return external ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal) : cudaEventRecord(e, s);
    };
    (void)a;
    HB_CUDA(h, rec(h->ev[2]));
    if (h->systolic)
        HB_LAUNCH(h, hbk::launch_mark_preds(h->d_bits[h->mod_cur ^ 1], h->d_toff, h->d_tsucc,
                                            h->d_bits[h->mbc_cur ^ 1], n, h->grid_mark, s));
    // the neighbourhood-function parts, in a fixed order, into partials[0].nf
    HB_LAUNCH(h, hbk::launch_sum_f64(h->d_nf_items, h->n_chunks + h->n_heavy, h->d_nf_scratch,
                                     &h->d_partials[0].nf, s));
    const size_t n_inst = h->inst_start.empty() ? 0 : h->inst_start.size() - 1;
    if (n_inst) {
        HB_LAUNCH(h, hbk::launch_inst_stats(h->d_bits[h->mod_cur ^ 1], h->d_est, h->d_inst_start,
                                            (uint32_t)n_inst, h->d_inst_mod, h->d_inst_nf, s));
        HB_LAUNCH(h, hbk::launch_copy_u64(reinterpret_cast<const uint64_t*>(h->d_inst_mod),
                                          reinterpret_cast<uint64_t*>(h->h_inst_mod), n_inst, s));
        HB_LAUNCH(h, hbk::launch_copy_u64(reinterpret_cast<const uint64_t*>(h->d_inst_nf),
                                          reinterpret_cast<uint64_t*>(h->h_inst_sum), n_inst, s));
    }
    HB_LAUNCH(h, hbk::launch_copy_u64(reinterpret_cast<const uint64_t*>(h->d_partials),
                                      reinterpret_cast<uint64_t*>(h->h_tot), sizeof(hbk::TilePartial) / 8, s));
    HB_CUDA(h, rec(h->ev[3]));
    return HB_OK;
}

// One iteration's launches on s (the union kernels of this handle alone; the
// heavy-node kernel on h->side, forked from s and joined back). `external`:
// the timing events are recorded as graph nodes (stream capture). The host
// reads the totals from h->h_tot (and, for batches, h->h_inst_*) once s is
// synchronised; the per-iteration constants come from h->h_ic.
int enqueue_iteration(hb_handle* h, hbk::UnionArgs a, bool first_systolic, cudaStream_t s,
                      bool external) {
    int r = enqueue_pre(h, a, first_systolic, s, external);
    if (!r) r = enqueue_union(h, a, s, true);
    if (!r) r = enqueue_join(h, s);
    if (!r) r = enqueue_post(h, a, s, external);
    return r;
}

// The executable graph of an iteration of this shape, or null. A shape is
// captured once an earlier run of the handle has shown it (the first run of a
// handle launches directly, so a handle that runs once pays no capture); the
// later runs replay it. A batch, which usually runs once, captures a shape the
// second time it comes in the run (shapes alternate with the state parities). Kernel arguments are fixed by the shape: the state
// parities, the mode, the union-kernel variant; the values that change every
// iteration reach the kernels through h->d_ic.
cudaGraphExec_t iteration_graph(hb_handle* h, const GraphKey& key, const hbk::UnionArgs& a,
                                bool first_systolic) {
    if (!h->use_graphs) return nullptr;
    for (const GraphEntry& g : h->graphs)
        if (g.key == key) {
            hbk::count_launches((int64_t)g.launches);
            return g.exec;
        }
    if (h->graphs.size() >= kMaxGraphs) return nullptr;
    if (std::find(h->shapes_seen.begin(), h->shapes_seen.end(), key) == h->shapes_seen.end()) {
        const bool in_run = std::find(h->shapes_run.begin(), h->shapes_run.end(), key) != h->shapes_run.end();
        if (!in_run) h->shapes_run.push_back(key);
        if (!(in_run && h->capture_in_run)) return nullptr;
    }
    // A capture that fails turns graphs off for the handle; the iteration
    // then launches directly (graphs change no result).
    auto give_up = [&]() -> cudaGraphExec_t {
        cudaGetLastError();
        h->use_graphs = false;
        h->err.clear();
        return nullptr;
    };
    const uint64_t c0 = hbk::launch_count();
    cudaError_t e = cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return give_up();
    const int r = enqueue_iteration(h, a, first_systolic, h->cap, true);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(h->cap, &graph);
    const uint64_t launches = hbk::launch_count() - c0;
    hbk::count_launches(-(int64_t)launches);  // captured, not launched
    if (r != HB_OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return give_up();
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return give_up();
    h->graphs.push_back(GraphEntry{key, exec, launches});
    hbk::count_launches((int64_t)launches);
    return exec;
}

// The host side of one iteration around its launches: iter_plan takes the
// mode decisions of HB:795-810 and fixes the launch arguments; iter_finish
// reads the totals back and does the bookkeeping of HB:899-944.
struct IterPlan {
    hbk::UnionArgs a;
    GraphKey key;
    bool first_systolic = false;
    int variant = 0;
    uint64_t merged = 0;
    uint64_t launches0 = 0;
    double current_nf = 0.0;
};

void iter_plan(hb_handle* h, IterPlan& p) {
    const uint64_t n = h->n, m = h->m;
    const uint64_t prev_mod = h->modified_counters;
    const bool prev_was_systolic = h->systolic;
    // HB:795-810
    h->systolic = h->has_transpose && h->iteration > 0 && prev_mod < n / 4;
    p.current_nf = h->systolic ? h->last : 0.0;
    h->local = h->pre_local;
    h->pre_local = h->systolic && m > 0 && prev_mod < (n * n) / (m * 10);

    p.launches0 = hbk::launch_count();
    hbk::UnionArgs& a = p.a;
    a = union_args(h);
    // nearly every counter changed in the previous iteration: merge all
    // successors without waiting for their modified bits (init marks every
    // counter modified, HB:1208, so the first iteration merges them all)
    const uint64_t changed_before = h->iteration == 0 ? n : prev_mod;
    a.gather_all = !h->systolic && changed_before >= n - n / 8;
    // the union-kernel variant (identical results; see Tuner)
    p.merged = a.gather_all ? m - h->self_loops : h->pending_visited;
    const int cls = h->systolic ? -1 : a.gather_all ? 0 : 1;
    const bool sample = h->iteration > 0 && m >= kTuneMinArcs && 2 * p.merged >= m;
    p.variant = choose_variant(h, cls, sample);
    a.pf = kVariants[p.variant].pf;
    a.pd = kVariants[p.variant].pd;
    a.occ = kVariants[p.variant].occ;
    // the staged kernel runs standard iterations (systolic ones walk node lists)
    a.staged = !h->systolic && h->d_items ? kVariants[p.variant].staged : 0;
    // the values that change from one iteration to the next
    h->h_ic->d1 = (double)(h->iteration + 1);
    h->h_ic->rd1 = 1.0 / h->h_ic->d1;
    for (size_t k = 0; k < h->d_disc.size(); k++)
        h->h_ic->disc_factor[k] = h->disc_fn[k](h->iteration + 1, h->disc_ctx[k]);
    p.first_systolic = h->systolic && !prev_was_systolic;
    p.key = GraphKey{h->cur, h->mbc_cur, h->systolic, p.first_systolic, (bool)a.gather_all, p.variant};
}

// After the iteration's launches completed (the stream was synchronised).
// union_ms >= 0 replaces the handle's own union timing (a shared launch).
int iter_finish(hb_handle* h, IterPlan& p, bool from_graph, double union_ms, hb_iter_stats* out) {
    const hbk::TilePartial tot = *h->h_tot;
    if (tot.timeouts)
        return set_err(h, HB_ERR_TIMEOUT, "a TMA gather did not complete within its bounded wait");
    const size_t n_inst = h->inst_start.empty() ? 0 : h->inst_start.size() - 1;
    if (n_inst) {
        h->inst_mod.assign(h->h_inst_mod, h->h_inst_mod + n_inst);
        h->inst_sum.assign(h->h_inst_sum, h->h_inst_sum + n_inst);
    }
    struct {
        unsigned long long st[4];
        double nf;
    } host{{tot.vis, tot.mod, tot.scanned, tot.sarcs}, tot.nf};

    // swap states (HB:909-914)
    h->cur ^= 1;
    h->mod_cur ^= 1;
    if (h->systolic) h->mbc_cur ^= 1;

    h->modified_counters = host.st[1];
    // arcs visited in this iteration were fixed by the previous one
    const uint64_t visited = h->pending_visited;
    h->pending_visited = host.st[0];
    double current_nf = p.current_nf + host.nf;
    h->last = current_nf;
    const double last_output = h->nf.back();
    if (current_nf < last_output) current_nf = last_output;
    h->relative_increment = current_nf / last_output;
    h->nf.push_back(current_nf);
    h->iteration += 1;
    // batch instances still running: the reference's output for each
    // (HB:916-944: monotone neighbourhood function; it stops after the first
    // iteration that modifies no counter of the instance)
    for (size_t i = 0; i < n_inst; i++) {
        if (h->inst_done[i]) continue;
        std::vector<double>& f = h->inst_nf[i];
        f.push_back(std::max(h->inst_sum[i], f.back()));
        h->inst_iters[i] = h->iteration;
        const uint64_t ni_nodes = h->inst_start[i + 1] - h->inst_start[i];
        if (h->inst_mod[i] == 0 || h->iteration >= ni_nodes) h->inst_done[i] = 1;
    }

    hb_iter_stats st{};
    st.iteration = h->iteration;
    st.modified_counters = host.st[1];
    st.visited_arcs = visited;
    st.scanned_nodes = host.st[2];
    st.neighborhood_function = current_nf;
    st.relative_increment = h->relative_increment;
    st.systolic = h->systolic;
    st.local = h->local;
    st.pre_local = h->pre_local;
    float ms_union = 0.f, ms_all = 0.f;
    cudaEventElapsedTime(&ms_union, h->ev[1], h->ev[2]);
    cudaEventElapsedTime(&ms_all, h->ev[0], h->ev[3]);
    st.union_ms = union_ms >= 0.0 ? union_ms : ms_union;
    st.iteration_ms = ms_all;
    st.scanned_arcs = host.st[3];
    st.union_variant = h->tuner.last;
    st.from_graph = from_graph;
    if (union_ms < 0.0) record_variant(h, ms_union, host.st[3] + p.merged);
    st.kernel_launches = hbk::launch_count() - p.launches0;
    h->stats.push_back(st);
    if (out) *out = st;
    return HB_OK;
}

int do_iterate(hb_handle* h, hb_iter_stats* out) {
    NvtxRange range("hb_iterate");
    IterPlan p;
    iter_plan(h, p);
    cudaStream_t s = h->stream;
    cudaGraphExec_t exec = iteration_graph(h, p.key, p.a, p.first_systolic);
    if (exec) {
        HB_CUDA(h, cudaGraphLaunch(exec, s));
    } else {
        int r = enqueue_iteration(h, p.a, p.first_systolic, s, false);
        if (r != HB_OK) return r;
    }
    HB_CUDA(h, cudaStreamSynchronize(s));
    return iter_finish(h, p, exec != nullptr, -1.0, out);
}

// ---------------------------------------------------------------------------
// Several handles, one union launch per iteration (no reference
// counterpart). The log2m groups of a batch and the running jobs of a server
// advance together: each handle's pre part (clears, work lists, queue), one
// k_union_jobs launch that drains every handle's window work from one cursor
// (the heavy-node kernels beside it on the handles' side streams), each
// handle's post part, one synchronisation, each handle's bookkeeping. The
// launch sequence of a set of shapes is captured as a CUDA graph the second
// time it comes and replayed afterwards.
// ---------------------------------------------------------------------------
struct MultiCtx {
    int device = 0;
    cudaStream_t s = nullptr;         // every launch of a step (the handles' buffers are ordered before it)
    cudaStream_t cap = nullptr;       // capture stream
    unsigned long long* d_cursor = nullptr;
    // the shared launch's job table (its kernel parameters)
    std::unique_ptr<hbk::JobsArgs> jobs;
    int grid = 1;
    cudaEvent_t u0 = nullptr, u1 = nullptr;  // around the union part (shared launch, heavy kernels)
    cudaEvent_t b0 = nullptr, b1 = nullptr;  // around the whole step
    // a handle with a stream of its own runs its pre and post parts there, so
    // that the small kernels of different handles overlap (steps launched
    // directly, not captured)
    cudaEvent_t fork_ev[64] = {}, join_ev[64] = {};
    bool use_graphs = true;
    struct Shape {
        std::vector<const hb_handle*> hs;
        std::vector<GraphKey> keys;
        bool operator==(const Shape& o) const { return hs == o.hs && keys == o.keys; }
    };
    struct Graph {
        Shape shape;
        cudaGraphExec_t exec;
        uint64_t launches;
    };
    std::vector<Graph> graphs;
    std::vector<Shape> seen;
    uint64_t steps = 0, replays = 0;
    double union_ms = 0.0;
    double pre_ms = 0.0, post_ms = 0.0;   // device time before and after the union part
    double host_ms = 0.0, wait_ms = 0.0;  // planning and launches; waiting for the step's end
    std::string err;
};

static bool job_kernel_log2m(int l) { return l == 4 || l == 6 || l == 8; }
static constexpr uint32_t kMaxJobs = hbk::MAX_JOBS;
static constexpr size_t kMaxMultiGraphs = 64;
// default degree buckets: lane-group nodes up to 64 successors, 8-lane teams up to 4096
static constexpr uint32_t kDefaultSmallMax = 64, kDefaultMediumMax = 4096;

static void multi_free(MultiCtx& mc) {
    cudaSetDevice(mc.device);
    if (mc.s) cudaStreamSynchronize(mc.s);
    for (auto& g : mc.graphs) cudaGraphExecDestroy(g.exec);
    mc.graphs.clear();
    mc.seen.clear();
    if (mc.d_cursor) cudaFree(mc.d_cursor);
    mc.jobs.reset();
    if (mc.u0) cudaEventDestroy(mc.u0);
    if (mc.u1) cudaEventDestroy(mc.u1);
    if (mc.b0) cudaEventDestroy(mc.b0);
    if (mc.b1) cudaEventDestroy(mc.b1);
    for (int j = 0; j < 64; j++) {
        if (mc.fork_ev[j]) cudaEventDestroy(mc.fork_ev[j]);
        if (mc.join_ev[j]) cudaEventDestroy(mc.join_ev[j]);
        mc.fork_ev[j] = mc.join_ev[j] = nullptr;
    }
    if (mc.cap) cudaStreamDestroy(mc.cap);
    mc.d_cursor = nullptr;
    mc.u0 = mc.u1 = mc.b0 = mc.b1 = nullptr;
    mc.cap = nullptr;
}

static int multi_init(MultiCtx& mc, int device, cudaStream_t s) {
    mc.device = device;
    mc.s = s;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaMalloc((void**)&mc.d_cursor, sizeof(unsigned long long));
    mc.jobs.reset(new hbk::JobsArgs());
    if (e == cudaSuccess) e = cudaEventCreate(&mc.u0);
    if (e == cudaSuccess) e = cudaEventCreate(&mc.u1);
    if (e == cudaSuccess) e = cudaEventCreate(&mc.b0);
    if (e == cudaSuccess) e = cudaEventCreate(&mc.b1);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&mc.cap, cudaStreamNonBlocking);
    for (int j = 0; j < 64 && e == cudaSuccess; j++) {
        e = cudaEventCreateWithFlags(&mc.fork_ev[j], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&mc.join_ev[j], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        mc.err = std::string("multi-instance setup: ") + cudaGetErrorString(e);
        multi_free(mc);
        return e == cudaErrorMemoryAllocation ? HB_ERR_OOM : HB_ERR_CUDA;
    }
    mc.grid = hbk::jobs_grid(device);
    return HB_OK;
}

// The launches of one step on stream x (the handles' plans are final).
static int multi_enqueue(std::vector<hb_handle*>& hs, std::vector<IterPlan>& plans, MultiCtx& mc,
                         cudaStream_t x, bool external, uint32_t* njobs) {
    auto rec = [&](cudaEvent_t e) {
        return external ? cudaEventRecordWithFlags(e, x, cudaEventRecordExternal) : cudaEventRecord(e, x);
    };
    int r;
    // the stream a handle's pre and post parts run on, forked from x and joined back
    auto own = [&](size_t j) { return !external && hs[j]->stream && hs[j]->stream != x; };
    auto fork = [&](size_t j) -> cudaError_t {
        cudaError_t e = cudaEventRecord(mc.fork_ev[j], x);
        return e == cudaSuccess ? cudaStreamWaitEvent(hs[j]->stream, mc.fork_ev[j], 0) : e;
    };
    auto join = [&](size_t j) -> cudaError_t {
        cudaError_t e = cudaEventRecord(mc.join_ev[j], hs[j]->stream);
        return e == cudaSuccess ? cudaStreamWaitEvent(x, mc.join_ev[j], 0) : e;
    };
    auto fail = [&](cudaError_t e) {
        mc.err = std::string("multi-instance step: ") + cudaGetErrorString(e);
        return HB_ERR_CUDA;
    };
    if (cudaError_t e = rec(mc.b0); e != cudaSuccess) return fail(e);
    for (size_t j = 0; j < hs.size(); j++) {
        const cudaStream_t y = own(j) ? hs[j]->stream : x;
        if (y != x)
            if (cudaError_t e = fork(j); e != cudaSuccess) return fail(e);
        if ((r = enqueue_pre(hs[j], plans[j].a, plans[j].first_systolic, y, external))) return r;
        if (y != x)
            if (cudaError_t e = join(j); e != cudaSuccess) return fail(e);
    }
    uint32_t J = 0;
    hbk::JobsArgs& p = *mc.jobs;
    for (size_t j = 0; j < hs.size(); j++) {
        hb_handle* h = hs[j];
        if (!h->n_tiles || !job_kernel_log2m(h->log2m) || plans[j].a.far_tma) continue;
        p.job[J] = plans[j].a;
        p.log2m[J] = h->log2m;
        J++;
    }
    p.njobs = J;
    p.cursor = mc.d_cursor;
    *njobs = J;
    if (J) {
        cudaError_t e = cudaMemsetAsync(mc.d_cursor, 0, sizeof(unsigned long long), x);
        if (e != cudaSuccess) {
            mc.err = std::string("multi-instance step: ") + cudaGetErrorString(e);
            return HB_ERR_CUDA;
        }
    }
    if (cudaError_t e = rec(mc.u0); e != cudaSuccess) {
        mc.err = cudaGetErrorString(e);
        return HB_ERR_CUDA;
    }
    for (size_t j = 0; j < hs.size(); j++) {
        hb_handle* h = hs[j];
        // handles outside the shared kernel launch their own window kernel
        const bool own = h->n_tiles && (!job_kernel_log2m(h->log2m) || plans[j].a.far_tma);
        if ((r = enqueue_union(h, plans[j].a, x, own))) return r;
    }
    if (J) {
        const int e = hbk::launch_union_jobs(p, mc.grid, x);
        if (e) {
            mc.err = std::string("k_union_jobs: ") + cudaGetErrorString((cudaError_t)e);
            return HB_ERR_CUDA;
        }
    }
    for (size_t j = 0; j < hs.size(); j++)
        if ((r = enqueue_join(hs[j], x))) return r;
    if (cudaError_t e = rec(mc.u1); e != cudaSuccess) {
        mc.err = cudaGetErrorString(e);
        return HB_ERR_CUDA;
    }
    for (size_t j = 0; j < hs.size(); j++) {
        const cudaStream_t y = own(j) ? hs[j]->stream : x;
        if (y != x)
            if (cudaError_t e = fork(j); e != cudaSuccess) return fail(e);
        if ((r = enqueue_post(hs[j], plans[j].a, y, external))) return r;
        if (y != x)
            if (cudaError_t e = join(j); e != cudaSuccess) return fail(e);
    }
    if (cudaError_t e = rec(mc.b1); e != cudaSuccess) return fail(e);
    return HB_OK;
}

// One iteration of every handle in hs (at most kMaxJobs of them, all on
// mc.device).
static int multi_iterate(std::vector<hb_handle*>& hs, MultiCtx& mc) {
    if (hs.empty()) return HB_OK;
    NvtxRange range("hb_multi_step");
    if (hs.size() > kMaxJobs) {
        mc.err = "more than 48 instances in one step";
        return HB_ERR_INVALID;
    }
    const auto t_start = std::chrono::steady_clock::now();
    std::vector<IterPlan> plans(hs.size());
    MultiCtx::Shape shape;
    for (size_t j = 0; j < hs.size(); j++) {
        iter_plan(hs[j], plans[j]);
        plans[j].a.staged = 0;
        shape.hs.push_back(hs[j]);
        shape.keys.push_back(plans[j].key);
    }
    const uint64_t c0 = hbk::launch_count();
    cudaGraphExec_t exec = nullptr;
    if (mc.use_graphs) {
        for (const auto& g : mc.graphs)
            if (g.shape == shape) {
                exec = g.exec;
                hbk::count_launches((int64_t)g.launches);
                break;
            }
        const bool again = std::find(mc.seen.begin(), mc.seen.end(), shape) != mc.seen.end();
        if (!exec && again && mc.graphs.size() < kMaxMultiGraphs) {
            // capture; a failed capture turns graphs off (they change no result)
            uint32_t J = 0;
            cudaError_t e = cudaStreamBeginCapture(mc.cap, cudaStreamCaptureModeThreadLocal);
            int r = e == cudaSuccess ? multi_enqueue(hs, plans, mc, mc.cap, true, &J) : HB_ERR_CUDA;
            cudaGraph_t graph = nullptr;
            if (e == cudaSuccess) e = cudaStreamEndCapture(mc.cap, &graph);
            const uint64_t launches = hbk::launch_count() - c0;
            hbk::count_launches(-(int64_t)launches);
            if (r == HB_OK && e == cudaSuccess && graph) {
                cudaGraphExec_t x = nullptr;
                if (cudaGraphInstantiate(&x, graph, 0) == cudaSuccess) {
                    mc.graphs.push_back(MultiCtx::Graph{shape, x, launches});
                    exec = x;
                    hbk::count_launches((int64_t)launches);
                }
            }
            if (graph) cudaGraphDestroy(graph);
            if (!exec) {
                cudaGetLastError();
                mc.use_graphs = false;
                for (hb_handle* h : hs) h->err.clear();
                mc.err.clear();
            }
        } else if (!exec && !again) {
            mc.seen.push_back(shape);
        }
    }
    if (exec) {
        cudaError_t e = cudaGraphLaunch(exec, mc.s);
        if (e != cudaSuccess) {
            mc.err = std::string("cudaGraphLaunch: ") + cudaGetErrorString(e);
            return HB_ERR_CUDA;
        }
        mc.replays++;
    } else {
        uint32_t J = 0;
        int r = multi_enqueue(hs, plans, mc, mc.s, false, &J);
        if (r) {
            if (mc.err.empty())
                for (hb_handle* h : hs)
                    if (!h->err.empty()) mc.err = h->err;
            return r;
        }
    }
    const auto t_launched = std::chrono::steady_clock::now();
    cudaError_t e = cudaStreamSynchronize(mc.s);
    if (e != cudaSuccess) {
        mc.err = std::string("multi-instance step: ") + cudaGetErrorString(e);
        return HB_ERR_CUDA;
    }
    const auto t_done = std::chrono::steady_clock::now();
    mc.host_ms += std::chrono::duration<double, std::milli>(t_launched - t_start).count();
    mc.wait_ms += std::chrono::duration<double, std::milli>(t_done - t_launched).count();
    float ms = 0.f, pre = 0.f, post = 0.f;
    cudaEventElapsedTime(&ms, mc.u0, mc.u1);
    cudaEventElapsedTime(&pre, mc.b0, mc.u0);
    cudaEventElapsedTime(&post, mc.u1, mc.b1);
    mc.union_ms += ms;
    mc.pre_ms += pre;
    mc.post_ms += post;
    mc.steps++;
    for (size_t j = 0; j < hs.size(); j++) {
        int r = iter_finish(hs[j], plans[j], exec != nullptr, ms, nullptr);
        if (r) {
            mc.err = hs[j]->err;
            return r;
        }
    }
    return HB_OK;
}

int ensure_iteration(const hb_handle* h) {
    if (!h || h->iteration == 0)
        return set_err(const_cast<hb_handle*>(h), HB_ERR_NOT_RUN,
                       "HyperBall was not run. Please call hb_run before accessing computed fields");
    return HB_OK;
}

int copy_d2h(const hb_handle* h, const void* src, void* dst, size_t bytes) {
    hb_handle* hh = const_cast<hb_handle*>(h);
    HB_CUDA(hh, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
    HB_CUDA(hh, cudaStreamSynchronize(h->stream));
    return HB_OK;
}

// Caller nodes [start, start + count) of a per-node device array (device node
// order) into dst on the host, in caller order.
int copy_nodes_range(const hb_handle* h, const double* src, double* dst, uint64_t start,
                     uint64_t count) {
    hb_handle* hh = const_cast<hb_handle*>(h);
    if (count == 0) return HB_OK;
    HB_CUDA(hh, cudaSetDevice(h->device));
    double* tmp = nullptr;
    cudaError_t e = pool_alloc(h->device, (void**)&tmp, count * 8, h->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_err(hh, e, "cudaMallocFromPoolAsync");
    }
    int r = hbk::launch_gather_f64(src, h->d_inv + start, tmp, count, h->stream);
    if (r == 0) r = copy_d2h(h, tmp, dst, count * 8);
    else r = cuda_err(hh, (cudaError_t)r, "launch_gather_f64");
    cudaFreeAsync(tmp, h->stream);
    cudaStreamSynchronize(h->stream);
    return r;
}

// A per-node device array into caller order on the host.
int copy_nodes_d2h(const hb_handle* h, const double* src, double* dst) {
    return copy_nodes_range(h, src, dst, 0, h->n);
}

// Counters of caller nodes [start, start + count) of one state, packed in the
// reference layout, into dst (count * counter_bytes bytes).
int copy_registers_range(const hb_handle* h, int which, void* dst, uint64_t start, uint64_t count) {
    if (count == 0) return HB_OK;
    const int idx = which == HB_CURRENT_STATE ? h->cur : (h->cur ^ 1);
    hb_handle* hh = const_cast<hb_handle*>(h);
    HB_CUDA(hh, cudaSetDevice(h->device));
    const size_t bytes = count * h->counter_bytes;
    void* packed = nullptr;
    cudaError_t e = pool_alloc(h->device, &packed, bytes, h->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_err(hh, e, "cudaMallocFromPoolAsync");
    }
    int r = hbk::launch_pack_counters(h->log2m, h->d_cnt[idx], h->d_inv + start, (uint8_t*)packed,
                                      count, h->stream);
    if (r == 0) r = copy_d2h(h, packed, dst, bytes);
    else r = cuda_err(hh, (cudaError_t)r, "launch_pack_counters");
    cudaFreeAsync(packed, h->stream);
    cudaStreamSynchronize(h->stream);
    return r;
}

int check_len(const hb_handle* h, size_t len) {
    if (len != h->n)
        return set_err(const_cast<hb_handle*>(h), HB_ERR_INVALID,
                       "output length must equal num_nodes (" + std::to_string(h->n) + ")");
    return HB_OK;
}

}  // namespace

struct hb_multi {
    MultiCtx mc;
};

int hb_multi_create(int device, void* stream, hb_multi** out, std::string& err) {
    hb_multi* m = new hb_multi();
    // a server's set of handles changes as jobs come and go, and a captured
    // graph holds the buffers of the handles it was captured with: no graphs
    m->mc.use_graphs = false;
    int r = multi_init(m->mc, device, (cudaStream_t)stream);
    if (r) {
        err = m->mc.err;
        delete m;
        return r;
    }
    *out = m;
    return HB_OK;
}

void hb_multi_destroy(hb_multi* m) {
    if (!m) return;
    multi_free(m->mc);
    delete m;
}

int hb_multi_start(hb_handle* h) {
    h->tuner.fixed = 0;  // the shared union kernel has one configuration
    HB_CUDA(h, cudaSetDevice(h->device));
    return do_init(h);
}

void hb_multi_reserve_sms(hb_multi* m, uint32_t sms) {
    const int all = hbk::num_sms(m->mc.device);
    const int per_sm = std::max(1, hbk::jobs_grid(m->mc.device) / std::max(all, 1));
    const int used = std::max(1, all - (int)std::min<uint32_t>(sms, (uint32_t)all - 1));
    m->mc.grid = per_sm * used;
}

int hb_multi_set_stream(hb_handle* h, void* stream) {
    HB_CUDA(h, cudaSetDevice(h->device));
    HB_CUDA(h, cudaStreamSynchronize(h->stream));
    h->stream = (cudaStream_t)stream;
    return HB_OK;
}

int hb_multi_step(hb_multi* m, hb_handle* const* hs, uint32_t count, std::string& err) {
    std::vector<hb_handle*> v(hs, hs + count);
    int r = multi_iterate(v, m->mc);
    if (r) err = m->mc.err;
    return r;
}

bool hb_multi_done(const hb_handle* h) {
    return h->n == 0 || (h->iteration > 0 && (h->modified_counters == 0 || h->iteration >= h->n));
}

uint64_t hb_multi_steps(const hb_multi* m, uint64_t* replays, double* union_ms, double* host_ms,
                        double* wait_ms, double* pre_ms, double* post_ms) {
    if (replays) *replays = m->mc.replays;
    if (union_ms) *union_ms = m->mc.union_ms;
    if (pre_ms) *pre_ms = m->mc.pre_ms;
    if (post_ms) *post_ms = m->mc.post_ms;
    if (host_ms) *host_ms = m->mc.host_ms;
    if (wait_ms) *wait_ms = m->mc.wait_ms;
    return m->mc.steps;
}

extern "C" {

void hb_options_default(hb_options* o) {
    std::memset(o, 0, sizeof(*o));
    o->struct_size = sizeof(hb_options);
    o->log2m = 4;
    o->hash_kind = HB_HASH_SIP13;
    o->small_max_degree = HB_AUTO;
    o->medium_max_degree = HB_AUTO;
    o->union_variant = HB_AUTO;
}

// ---- batches ------------------------------------------------------------------
static int create_impl(const hb_graph_view* graph, const hb_graph_view* transpose,
                       const hb_options* opts, const std::vector<uint64_t>* inst, hb_handle** out);

// Instances with the same log2m run as one disjoint union of their graphs
// (instance i's nodes are a contiguous id range; an arc never leaves its
// instance), so every iteration of the union is one pass of the union kernels
// over all of them. The counters, and therefore every output, of an instance
// do not depend on the others; the mode of an iteration (standard, systolic,
// local) changes only which nodes are scanned, not the counters. Each
// instance hashes its own node ids and reports its own neighbourhood function
// and iteration count (the first iteration that modifies none of its
// counters).
struct hb_batch {
    struct Group {
        hb_handle* h = nullptr;
    };
    struct Member {
        uint32_t group = 0, inst = 0;
        uint64_t start = 0, n = 0;
    };
    std::vector<Group> groups;
    std::vector<Member> members;
    int device = 0;
    bool ran = false;
    // every group's launches run on this stream, one step for all groups
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    MultiCtx mc;
};

static void batch_free(hb_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    multi_free(b->mc);
    for (auto& g : b->groups)
        if (g.h) hb_destroy(g.h);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int hb_batch_create(const hb_graph_view* graphs, uint32_t count, const int32_t* log2m,
                    const hb_options* opts, hb_batch** out) {
    if (!out) return set_err(nullptr, HB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!graphs || !log2m || count == 0)
        return set_err(nullptr, HB_ERR_INVALID, "graphs and log2m must hold count > 0 entries");
    hb_options o;
    hb_options_default(&o);
    if (opts) {
        if (opts->struct_size != sizeof(hb_options))
            return set_err(nullptr, HB_ERR_INVALID, "hb_options.struct_size mismatch");
        o = *opts;
    }
    if (o.weights) return set_err(nullptr, HB_ERR_INVALID, "weights are not supported in batches");
    std::string why;
    std::map<int, std::vector<uint32_t>> by_log2m;
    for (uint32_t i = 0; i < count; i++) {
        if (!check_view(&graphs[i], why))
            return set_err(nullptr, HB_ERR_INVALID, "graph " + std::to_string(i) + ": " + why);
        if (log2m[i] < 4 || log2m[i] > 10)
            return set_err(nullptr, HB_ERR_INVALID, "graph " + std::to_string(i) + ": log2m must be in [4, 10]");
        by_log2m[log2m[i]].push_back(i);
    }
    std::unique_ptr<hb_batch, void (*)(hb_batch*)> b(new hb_batch(), batch_free);
    b->device = o.device;
    b->members.resize(count);
    cudaError_t ce = cudaSetDevice(o.device);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, HB_ERR_NO_DEVICE, "no CUDA device available (this library has no CPU path)");
    }
    if (o.stream) {
        b->stream = (cudaStream_t)o.stream;
    } else {
        ce = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (ce != cudaSuccess) {
            cudaGetLastError();
            return set_err(nullptr, HB_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(ce));
        }
        b->own_stream = true;
    }
    for (auto& kv : by_log2m) {
        const std::vector<uint32_t>& idx = kv.second;
        // the disjoint union: instance k's nodes start at inst[k]
        std::vector<uint64_t> inst(idx.size() + 1, 0), arc0(idx.size() + 1, 0);
        for (size_t k = 0; k < idx.size(); k++) {
            inst[k + 1] = inst[k] + graphs[idx[k]].num_nodes;
            arc0[k + 1] = arc0[k] + graphs[idx[k]].num_arcs;
        }
        const uint64_t n = inst.back(), m = arc0.back();
        if (n > 0xffffffffull)
            return set_err(nullptr, HB_ERR_INVALID, "a batch group has more than 2^32 nodes");
        std::vector<uint64_t> off(n + 1);
        std::vector<uint32_t> succ(m);
        {
            const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
            const size_t nt = std::min<size_t>(std::min<size_t>(hw, 64), idx.size());
            std::vector<std::thread> th;
            for (size_t t = 0; t < nt; t++)
                th.emplace_back([&, t] {
                    for (size_t k = idx.size() * t / nt; k < idx.size() * (t + 1) / nt; k++) {
                        const hb_graph_view& gv = graphs[idx[k]];
                        for (uint64_t v = 0; v < gv.num_nodes; v++) off[inst[k] + v] = arc0[k] + gv.offsets[v];
                        for (uint64_t e = 0; e < gv.num_arcs; e++)
                            succ[arc0[k] + e] = (uint32_t)(gv.successors[e] + inst[k]);
                    }
                });
            for (auto& x : th) x.join();
        }
        off[n] = m;
        hb_graph_view uv{n, m, off.data(), succ.data()};
        hb_batch::Group g;
        hb_options go = o;
        go.log2m = kv.first;
        go.stream = b->stream;
        go.num_elements = 0;
        b->groups.push_back(g);
        int r = create_impl(&uv, nullptr, &go, &inst, &b->groups.back().h);
        if (r) return r;
        // the shared union kernel has one configuration (no variant tuning)
        b->groups.back().h->tuner.fixed = 0;
        for (size_t k = 0; k < idx.size(); k++) {
            hb_batch::Member& mb = b->members[idx[k]];
            mb.group = (uint32_t)(b->groups.size() - 1);
            mb.inst = (uint32_t)k;
            mb.start = inst[k];
            mb.n = inst[k + 1] - inst[k];
        }
    }
    *out = b.release();
    return HB_OK;
}

void hb_batch_destroy(hb_batch* b) { batch_free(b); }

// All groups advance together: one step runs one iteration of every group
// whose instances are not all done, with one union launch for all of them
// (multi_iterate). A group stops after an iteration that modified no counter
// (every instance done, HB:559-570) or after num_nodes iterations (HB:541).
int hb_batch_run_until_done(hb_batch* b) {
    if (!b) return set_err(nullptr, HB_ERR_INVALID, "batch is NULL");
    cudaError_t ce = cudaSetDevice(b->device);
    if (ce != cudaSuccess) return set_err(nullptr, HB_ERR_CUDA, cudaGetErrorString(ce));
    if (!b->mc.jobs) {
        int r = multi_init(b->mc, b->device, b->stream);
        if (r) return set_err(nullptr, r, b->mc.err);
    }
    std::vector<hb_handle*> running;
    for (auto& g : b->groups) {
        int r = do_init(g.h);
        if (r) return set_err(nullptr, r, g.h->err);
        if (g.h->n) running.push_back(g.h);
    }
    b->mc.steps = b->mc.replays = 0;
    b->mc.union_ms = 0.0;
    while (!running.empty()) {
        int r = multi_iterate(running, b->mc);
        if (r) return set_err(nullptr, r, b->mc.err);
        std::vector<hb_handle*> still;
        for (hb_handle* h : running)
            if (h->modified_counters != 0 && h->iteration < h->n) still.push_back(h);
        running.swap(still);
    }
    b->ran = true;
    return HB_OK;
}

static int batch_member(const hb_batch* b, uint32_t graph, const hb_batch::Member** mb,
                        const hb_handle** h) {
    if (!b) return set_err(nullptr, HB_ERR_INVALID, "batch is NULL");
    if (graph >= b->members.size()) return set_err(nullptr, HB_ERR_INVALID, "graph index out of range");
    if (!b->ran)
        return set_err(nullptr, HB_ERR_NOT_RUN,
                       "HyperBall was not run. Please call hb_batch_run_until_done before accessing computed fields");
    *mb = &b->members[graph];
    *h = b->groups[(*mb)->group].h;
    return HB_OK;
}

// as ensure_iteration (HB:624-630) for one instance: a graph that ran no
// iteration (no nodes) has no computed fields
static int batch_ran(const hb_handle* h, const hb_batch::Member* mb) {
    if (h->inst_iters[mb->inst] == 0)
        return set_err(nullptr, HB_ERR_NOT_RUN,
                       "HyperBall was not run. Please call hb_batch_run_until_done before accessing computed fields");
    return HB_OK;
}

uint32_t hb_batch_num_graphs(const hb_batch* b) { return b ? (uint32_t)b->members.size() : 0; }

uint64_t hb_batch_num_iterations(const hb_batch* b, uint32_t graph) {
    const hb_batch::Member* mb;
    const hb_handle* h;
    if (batch_member(b, graph, &mb, &h)) return 0;
    return h->inst_iters[mb->inst];
}

int hb_batch_get_neighborhood_function(const hb_batch* b, uint32_t graph, double* dst,
                                       size_t capacity, size_t* len) {
    const hb_batch::Member* mb;
    const hb_handle* h;
    int r = batch_member(b, graph, &mb, &h);
    if (r || (r = batch_ran(h, mb))) return r;
    const std::vector<double>& f = h->inst_nf[mb->inst];
    if (len) *len = f.size();
    if (dst) std::copy(f.begin(), f.begin() + std::min(capacity, f.size()), dst);
    return HB_OK;
}

static int batch_sums(const hb_batch* b, uint32_t graph, double* dst, size_t len, bool harm) {
    const hb_batch::Member* mb;
    const hb_handle* h;
    int r = batch_member(b, graph, &mb, &h);
    if (r || (r = batch_ran(h, mb))) return r;
    const double* src = harm ? h->d_harm : h->d_sod;
    if (!src)
        return set_err(nullptr, HB_ERR_NOT_REQUESTED,
                       harm ? "Sum of inverse distances were not requested. Set HB_SUM_OF_INVERSE_DISTANCES while building the batch"
                            : "Sum of distances were not requested. Set HB_SUM_OF_DISTANCES while building the batch");
    if (!dst || len != mb->n)
        return set_err(nullptr, HB_ERR_INVALID, "output length must equal the graph's num_nodes");
    return copy_nodes_range(h, src, dst, mb->start, mb->n);
}

int hb_batch_get_sum_of_distances(const hb_batch* b, uint32_t graph, double* dst, size_t len) {
    return batch_sums(b, graph, dst, len, false);
}

int hb_batch_get_harmonic_centralities(const hb_batch* b, uint32_t graph, double* dst, size_t len) {
    return batch_sums(b, graph, dst, len, true);
}

int hb_batch_get_registers(const hb_batch* b, uint32_t graph, void* dst, size_t bytes) {
    const hb_batch::Member* mb;
    const hb_handle* h;
    int r = batch_member(b, graph, &mb, &h);
    if (r) return r;
    if (!dst || bytes != mb->n * h->counter_bytes)
        return set_err(nullptr, HB_ERR_INVALID, "bytes must be the graph's num_nodes * counter bytes");
    return copy_registers_range(h, HB_CURRENT_STATE, dst, mb->start, mb->n);
}

int hb_batch_stats(const hb_batch* b, uint64_t* iterations, uint64_t* visited_arcs,
                   uint64_t* register_updates, double* device_ms) {
    if (!b) return set_err(nullptr, HB_ERR_INVALID, "batch is NULL");
    uint64_t it = 0, vis = 0, upd = 0;
    for (const auto& g : b->groups) {
        it = std::max<uint64_t>(it, g.h->iteration);
        for (const auto& s : g.h->stats) {
            vis += s.visited_arcs;
            upd += s.visited_arcs << g.h->log2m;
        }
    }
    const double ms = b->mc.union_ms;
    if (iterations) *iterations = it;
    if (visited_arcs) *visited_arcs = vis;
    if (register_updates) *register_updates = upd;
    if (device_ms) *device_ms = ms;
    return HB_OK;
}

int hb_batch_graph_replays(const hb_batch* b, uint64_t* replayed, uint64_t* iterations) {
    if (!b) return set_err(nullptr, HB_ERR_INVALID, "batch is NULL");
    if (replayed) *replayed = b->mc.replays;
    if (iterations) *iterations = b->mc.steps;
    return HB_OK;
}

// ---- device CSR utilities ----------------------------------------------------
namespace {
// Checks a device CSR before any kernel indexes with it: offsets[0] == 0,
// offsets[n] == m (read back), offsets non-decreasing and successors < n
// (k_validate into the device int `flag`).
int check_device_csr(const uint64_t* off, const uint32_t* succ, uint64_t n, uint64_t m, int* flag,
                     cudaStream_t s) {
    uint64_t ends[2] = {1, 0};
    cudaError_t e = cudaMemcpyAsync(&ends[0], off, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ends[1], off + n, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(flag, 0, sizeof(int), s);
    int r = e == cudaSuccess ? hbk::launch_validate(off, succ, n, m, flag, s) : (int)e;
    int bad = 0;
    if (!r) r = (int)cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (!r) r = (int)cudaStreamSynchronize(s);
    if (r) {
        cudaGetLastError();
        return set_err(nullptr, HB_ERR_CUDA, std::string("device CSR check: ") + cudaGetErrorString((cudaError_t)r));
    }
    if (ends[0] != 0 || ends[1] != m)
        return set_err(nullptr, HB_ERR_INVALID, "offsets[0] must be 0 and offsets[num_nodes] must equal num_arcs");
    if (bad) return set_err(nullptr, HB_ERR_INVALID, "graph has decreasing offsets or successors >= num_nodes");
    return HB_OK;
}

int device_transpose_args(const uint64_t* off, const uint32_t* succ, uint64_t n, uint64_t m,
                          const uint64_t* toff, const uint32_t* tsucc) {
    if (!off || !toff) return set_err(nullptr, HB_ERR_INVALID, "offsets and t_offsets must not be NULL");
    if (m && (!succ || !tsucc))
        return set_err(nullptr, HB_ERR_INVALID, "successors and t_successors must not be NULL");
    if (n > 0xffffffffull) return set_err(nullptr, HB_ERR_INVALID, "more than 2^32 nodes do not fit u32 successors");
    return HB_OK;
}
}  // namespace

int hb_device_transpose(const uint64_t* d_offsets, const uint32_t* d_successors, uint64_t num_nodes,
                        uint64_t num_arcs, uint64_t* d_t_offsets, uint32_t* d_t_successors,
                        void* stream) {
    int r = device_transpose_args(d_offsets, d_successors, num_nodes, num_arcs, d_t_offsets, d_t_successors);
    if (r) return r;
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t n = num_nodes, sl = hbk::scan_scratch_len(n + 1);
    // temporaries: n + 1 cursors, the scan scratch, one flag word
    const size_t bytes = (n + 1 + sl + 1) * 8;
    unsigned long long* tmp = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&tmp, bytes, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, e == cudaErrorMemoryAllocation ? HB_ERR_OOM : HB_ERR_CUDA,
                       std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    }
    r = check_device_csr(d_offsets, d_successors, n, num_arcs, (int*)(tmp + n + 1 + sl), s);
    if (!r) {
        e = transpose_core(d_offsets, d_successors, n, num_arcs, d_t_offsets, d_t_successors, tmp,
                           tmp + n + 1, sl, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            r = set_err(nullptr, HB_ERR_CUDA, std::string("hb_device_transpose: ") + cudaGetErrorString(e));
        }
    }
    cudaFreeAsync(tmp, s);
    cudaStreamSynchronize(s);
    return r;
}

int hb_device_transpose_noalloc(const uint64_t* d_offsets, const uint32_t* d_successors,
                                uint64_t num_nodes, uint64_t num_arcs, uint64_t* d_t_offsets,
                                uint32_t* d_t_successors, void* stream) {
    int r = device_transpose_args(d_offsets, d_successors, num_nodes, num_arcs, d_t_offsets, d_t_successors);
    if (r) return r;
    if (num_nodes > hbk::NOALLOC_MAX_NODES)
        return set_err(nullptr, HB_ERR_INVALID,
                       "hb_device_transpose_noalloc: num_nodes " + std::to_string(num_nodes) +
                           " exceeds its fixed scratch (at most " +
                           std::to_string(hbk::NOALLOC_MAX_NODES) +
                           " nodes); use hb_device_transpose");
    unsigned long long* scratch = nullptr;
    uint64_t words = 0;
    r = hbk::noalloc_scratch(&scratch, &words);
    if (r) {
        cudaGetLastError();
        return set_err(nullptr, HB_ERR_CUDA,
                       std::string("hb_device_transpose_noalloc: cudaGetSymbolAddress: ") +
                           cudaGetErrorString((cudaError_t)r));
    }
    cudaStream_t s = (cudaStream_t)stream;
    // the scratch address is the current device's; a stream of another
    // device would run the kernels on that device's copy of nothing
    if (s != nullptr) {
        int cur = -1, sdev = -1;
        cudaError_t de = cudaGetDevice(&cur);
        if (de == cudaSuccess) de = cudaStreamGetDevice(s, &sdev);
        if (de != cudaSuccess) {
            cudaGetLastError();
            return set_err(nullptr, HB_ERR_CUDA,
                           std::string("hb_device_transpose_noalloc: ") + cudaGetErrorString(de));
        }
        if (sdev != cur)
            return set_err(nullptr, HB_ERR_INVALID,
                           "hb_device_transpose_noalloc: the stream belongs to device " +
                               std::to_string(sdev) + ", the current device is " +
                               std::to_string(cur) + "; make the stream's device current");
    }
    const uint64_t n = num_nodes, sl = hbk::scan_scratch_len(n + 1);
    if (n + 1 + sl + 1 > words)
        return set_err(nullptr, HB_ERR_INVALID, "hb_device_transpose_noalloc: scratch too small");
    // cursors [0, n], scan scratch, then the flag word (all cleared before use)
    r = check_device_csr(d_offsets, d_successors, n, num_arcs, (int*)(scratch + n + 1 + sl), s);
    if (r) return r;
    cudaError_t e = transpose_core(d_offsets, d_successors, n, num_arcs, d_t_offsets, d_t_successors,
                                   scratch, scratch + n + 1, sl, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, HB_ERR_CUDA, std::string("hb_device_transpose_noalloc: ") + cudaGetErrorString(e));
    }
    return HB_OK;
}

int hb_debug_fail_allocations(int64_t after) {
    g_fail_alloc_after.store(after < 0 ? -1 : after);
    return HB_OK;
}

int hb_debug_far_wait(hb_handle* h, uint32_t polls, uint32_t extra_tx_bytes) {
    if (!h) return set_err(nullptr, HB_ERR_INVALID, "null handle");
    if (extra_tx_bytes > (1u << 19))
        return set_err(h, HB_ERR_INVALID, "extra_tx_bytes must be at most 2^19 (the expected count stays below the 2^20 limit of an mbarrier)");
    h->far_polls = polls;
    h->far_extra_tx = extra_tx_bytes;
    // captured iterations hold the old values: capture again
    cudaStreamSynchronize(h->stream);
    for (GraphEntry& g : h->graphs) cudaGraphExecDestroy(g.exec);
    h->graphs.clear();
    return HB_OK;
}

const char* hb_version(void) { return "hyperball_gb300 0.1 sm_103a"; }

uint64_t hb_kernel_launches(const hb_handle* h) { return h ? h->launches : 0; }

int hb_release_cached_memory(int device) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_err(nullptr, HB_ERR_NO_DEVICE, "no CUDA device available (this library has no CPU path)");
    }
    if (device < 0 || device >= ndev) return set_err(nullptr, HB_ERR_INVALID, "no such device");
    cudaMemPool_t pool = nullptr;
    cudaError_t e = lib_pool(device, &pool);
    if (e == cudaSuccess) e = cudaMemPoolTrimTo(pool, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, HB_ERR_CUDA, std::string("cudaMemPoolTrimTo: ") + cudaGetErrorString(e));
    }
    // the page-locked blocks no handle holds
    std::multimap<size_t, void*> blocks;
    {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        blocks.swap(g_pinned_free);
    }
    for (auto& b : blocks) cudaFreeHost(b.second);
    cudaGetLastError();
    return HB_OK;
}
const char* hb_global_last_error(void) { return g_global_err.c_str(); }
const char* hb_last_error(const hb_handle* h) { return h ? h->err.c_str() : g_global_err.c_str(); }

// hb_create, optionally for a batch: `inst` holds the instance starts (caller
// ids, ascending, starting at 0) followed by num_nodes.
// HB_TRACE=1 in the environment prints the duration of each creation phase
// to stderr (the reference's progress-logger role for building).
struct PhaseTrace {
    bool on = std::getenv("HB_TRACE") != nullptr;
    int device = -1;  // once known: the library pool's reserved and used bytes too
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    void mark(const char* phase) {
        if (!on) return;
        const auto now = std::chrono::steady_clock::now();
        uint64_t reserved = 0, used = 0;
        cudaMemPool_t pool = nullptr;
        if (device >= 0 && lib_pool(device, &pool) == cudaSuccess) {
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
        }
        std::fprintf(stderr, "hb_create %-28s %8.2f ms   pool %.2f GB reserved, %.2f GB used\n", phase,
                     std::chrono::duration<double, std::milli>(now - t).count(), reserved / 1e9,
                     used / 1e9);
        t = now;
    }
};

static int create_impl(const hb_graph_view* graph, const hb_graph_view* transpose,
                       const hb_options* opts, const std::vector<uint64_t>* inst, hb_handle** out) {
    NvtxRange range("hb_create");
    if (!out) return set_err(nullptr, HB_ERR_INVALID, "out is NULL");
    PhaseTrace trace;
    *out = nullptr;
    hb_options o;
    hb_options_default(&o);
    if (opts) {
        if (opts->struct_size != sizeof(hb_options))
            return set_err(nullptr, HB_ERR_INVALID, "hb_options.struct_size mismatch");
        o = *opts;
    }
    std::string why;
    if (!check_view(graph, why)) return set_err(nullptr, HB_ERR_INVALID, why);
    if (transpose) {
        if (!check_view(transpose, why)) return set_err(nullptr, HB_ERR_INVALID, "transpose: " + why);
        // HB:230-238
        if (transpose->num_nodes != graph->num_nodes)
            return set_err(nullptr, HB_ERR_INVALID,
                           "the transpose should have same number of nodes of the graph");
        if (transpose->num_arcs != graph->num_arcs)
            return set_err(nullptr, HB_ERR_INVALID,
                           "the transpose should have same number of arcs of the graph");
    }
    // HLL:379-383
    if (o.log2m < 4)
        return set_err(nullptr, HB_ERR_INVALID,
                       "the logarithm of the number of registers per counter should be at least 4; got " +
                           std::to_string(o.log2m));
    if (o.log2m > 10)
        return set_err(nullptr, HB_ERR_INVALID,
                       "log2m above 10 is not supported by the device kernels; got " +
                           std::to_string(o.log2m));
    if (o.hash_kind != HB_HASH_SIP13 && o.hash_kind != HB_HASH_JENKINS)
        return set_err(nullptr, HB_ERR_INVALID, "unknown hash_kind");

    std::unique_ptr<hb_handle> h(new hb_handle());
    if (inst) h->inst_start = *inst;
    h->device = o.device;
    h->stream = (cudaStream_t)o.stream;
    h->n = graph->num_nodes;
    h->m = graph->num_arcs;
    h->log2m = o.log2m;
    h->counter_bytes = ((uint64_t)1 << o.log2m) * 5 / 8;
    h->stride = (uint64_t)1 << o.log2m;
    h->hash_kind = o.hash_kind;
    h->hash_seed = o.hash_seed;
    h->do_sod = o.flags & HB_SUM_OF_DISTANCES;
    h->do_harm = o.flags & HB_SUM_OF_INVERSE_DISTANCES;
    h->quirk = !(o.flags & HB_NO_I32_SHIFT_QUIRK);
    h->arc_granularity = o.arc_granularity ? o.arc_granularity : 16 * 1024;
    h->weight_seed = o.weight_seed;
    h->has_weights = o.weights != nullptr;
    uint64_t ne = o.num_elements;
    if (ne == 0) {
        if (o.weights) {
            for (uint64_t i = 0; i < h->n; i++) ne += o.weights[i];
        } else {
            ne = h->n;
        }
    }
    h->num_elements = ne;
    if (register_size(ne) != 5)
        return set_err(nullptr, HB_ERR_INVALID, "register size other than 5 is not supported");
    {
        // HLL:388-393, 420
        const double mf = (double)(1ull << o.log2m);
        double alpha;
        switch (o.log2m) {
            case 4: alpha = 0.673; break;
            case 5: alpha = 0.697; break;
            case 6: alpha = 0.709; break;
            default: alpha = 0.7213 / (1.0 + 1.079 / mf); break;
        }
        h->alpha_m_m = alpha * (mf * mf);
    }

    hb_handle* hp = h.get();
    LaunchTally tally(hp);
    int r;
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_err(nullptr, HB_ERR_NO_DEVICE, "no CUDA device available (this library has no CPU path)");
    }
    if ((r = cuda_err(hp, cudaSetDevice(h->device), "cudaSetDevice"))) return r;
    for (auto& e : h->ev)
        if ((r = cuda_err(hp, cudaEventCreate(&e), "cudaEventCreate"))) {
            release(hp);
            return r;
        }
    if ((r = cuda_err(hp, cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming), "cudaEventCreate")) ||
        (r = cuda_err(hp, cudaEventCreateWithFlags(&h->join, cudaEventDisableTiming), "cudaEventCreate")) ||
        (r = cuda_err(hp, high_priority_stream(&h->side), "cudaStreamCreate")) ||
        (r = cuda_err(hp, cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking), "cudaStreamCreate")) ||
        (r = cuda_err(hp, pinned_alloc((void**)&h->h_ic, sizeof(hbk::IterConsts)), "cudaMallocHost")) ||
        (r = cuda_err(hp, pinned_alloc((void**)&h->h_tot, sizeof(hbk::TilePartial)), "cudaMallocHost"))) {
        release(hp);
        return r;
    }
    std::memset(h->h_ic, 0, sizeof(hbk::IterConsts));
    std::memset(h->h_tot, 0, sizeof(hbk::TilePartial));
    if (!h->inst_start.empty()) {
        const size_t ni = h->inst_start.size() - 1;
        if ((r = cuda_err(hp, pinned_alloc((void**)&h->h_inst_mod, std::max<size_t>(ni, 1) * 8), "cudaMallocHost")) ||
            (r = cuda_err(hp, pinned_alloc((void**)&h->h_inst_sum, std::max<size_t>(ni, 1) * 8), "cudaMallocHost"))) {
            release(hp);
            return r;
        }
    }
    h->use_graphs = !(o.flags & HB_NO_GRAPHS);
    h->capture_in_run = !h->inst_start.empty();

    auto fail = [&](int code) {
        g_global_err = hp->err;
        release(hp);
        return code;
    };
    // Work partition and renumbering (host), then the CSR (and the transpose
    // when given) uploaded, validated and renumbered on the device.
    h->small_max = o.small_max_degree != HB_AUTO ? o.small_max_degree : kDefaultSmallMax;
    h->medium_max = o.medium_max_degree != HB_AUTO ? o.medium_max_degree : kDefaultMediumMax;
    if (h->medium_max < h->small_max) h->medium_max = h->small_max;
    const bool device_transpose = !transpose && (o.flags & HB_TRANSPOSE_ON_DEVICE);
    unsigned long long* trows = nullptr;
    {
        uint32_t win_nodes = 0, win_arcs = 0, per_light = 0, per_medium = 0;
        hbk::tile_capacity(h->log2m, &win_nodes, &win_arcs);
        hbk::chunk_nodes(h->log2m, &per_light, &per_medium);
        uint64_t* off0 = nullptr;
        uint32_t* succ0 = nullptr;
        trace.device = h->device;
        trace.mark("setup");
        if ((r = upload_csr(hp, graph, &off0, &succ0))) return fail(r);
        trace.mark("CSR upload + check");
        if ((r = device_partition(hp, off0, win_nodes, per_light, per_medium))) return fail(r);
        trace.mark("work partition");
        const uint64_t words = (h->n + 31) / 32;
        if ((r = dalloc(hp, &h->d_word_cnt, words + 1))) return fail(r);
        if ((r = dalloc(hp, &h->d_word_off, words + 1))) return fail(r);
        h->list_scratch_len = hbk::scan_scratch_len(words + 1);
        if ((r = dalloc(hp, &h->d_list_scratch, h->list_scratch_len))) return fail(r);
        if ((r = dalloc(hp, &h->d_light_list, h->n + 1))) return fail(r);
        if ((r = dalloc(hp, &h->d_medium_list, h->n + 1))) return fail(r);
        if (!h->inst_start.empty()) {
            // batch: per-instance bookkeeping (the hashed ids came with the partition)
            const size_t ni = h->inst_start.size() - 1;
            if ((r = dalloc(hp, &h->d_inst_start, h->inst_start.size()))) return fail(r);
            if ((r = cuda_err(hp, cudaMemcpyAsync(h->d_inst_start, h->inst_start.data(),
                                                  h->inst_start.size() * 8, cudaMemcpyHostToDevice,
                                                  h->stream),
                              "cudaMemcpyAsync")))
                return fail(r);
            if ((r = dalloc(hp, &h->d_inst_mod, ni))) return fail(r);
            if ((r = dalloc(hp, &h->d_inst_nf, ni))) return fail(r);
            // the chunks of each instance, for the queue of running instances
            if (h->n_chunks && ni && h->n_chunks < (1ull << 32)) {
                if ((r = dalloc(hp, &h->d_inst_chunk, ni + 1))) return fail(r);
                if ((r = dalloc(hp, &h->d_queue, h->n_chunks))) return fail(r);
                if ((r = dalloc(hp, &h->d_queue_len, 1))) return fail(r);
                if ((r = dalloc(hp, &h->d_q_cnt, ni + 1))) return fail(r);
                if ((r = dalloc(hp, &h->d_q_at, ni + 1))) return fail(r);
                h->q_scratch_len = hbk::scan_scratch_len(ni + 1);
                if ((r = dalloc(hp, &h->d_q_scratch, h->q_scratch_len))) return fail(r);
                if ((r = cuda_err(hp, (cudaError_t)hbk::launch_inst_first_chunk(
                                          h->d_chunks, h->n_chunks, h->d_inst_start, (uint32_t)ni,
                                          h->d_inst_chunk, h->stream),
                                  "k_inst_first_chunk")))
                    return fail(r);
            }
        }
        // renumbering; the same pass counts in-degrees without self-loops and,
        // with a transpose to build, each node's self-loops (its row lengths
        // are in-degree + self-loops)
        unsigned long long* loops = nullptr;
        if ((r = dalloc(hp, &h->d_indeg, h->n))) return fail(r);
        if ((r = dalloc(hp, &loops, 1))) return fail(r);
        if (device_transpose && (r = dalloc(hp, &trows, h->n + 1))) return fail(r);
        if ((r = cuda_err(hp, cudaMemsetAsync(h->d_indeg, 0, h->n * 4, h->stream), "cudaMemsetAsync")))
            return fail(r);
        if ((r = cuda_err(hp, cudaMemsetAsync(loops, 0, 8, h->stream), "cudaMemsetAsync"))) return fail(r);
        if (trows &&
            (r = cuda_err(hp, cudaMemsetAsync(trows, 0, (h->n + 1) * 8, h->stream), "cudaMemsetAsync")))
            return fail(r);
        if ((r = relabel_csr(hp, off0, succ0, &h->d_off, &h->d_succ, h->d_indeg, loops, trows,
                             device_transpose ? &h->d_arc_tiles : nullptr)))
            return fail(r);
        trace.mark("renumbering + in-degrees");
        dfree(hp, off0);
        dfree(hp, succ0);
        unsigned long long nl = 0;
        if ((r = cuda_err(hp, cudaMemcpyAsync(&nl, loops, 8, cudaMemcpyDeviceToHost, h->stream), "cudaMemcpy")))
            return fail(r);
        if ((r = cuda_err(hp, cudaStreamSynchronize(h->stream), "cudaStreamSynchronize"))) return fail(r);
        h->self_loops = nl;
        dfree(hp, loops);
    }
    if (transpose) {
        uint64_t* off0 = nullptr;
        uint32_t* succ0 = nullptr;
        if ((r = upload_csr(hp, transpose, &off0, &succ0))) return fail(r);
        if ((r = relabel_csr(hp, off0, succ0, &h->d_toff, &h->d_tsucc, nullptr, nullptr, nullptr,
                             nullptr)))
            return fail(r);
        dfree(hp, off0);
        dfree(hp, succ0);
        h->has_transpose = true;
    } else if (device_transpose) {
        if ((r = build_transpose_on_device(hp, trows))) return fail(r);
        dfree(hp, h->d_arc_tiles);
        h->d_arc_tiles = nullptr;
        trace.mark("transpose");
    }
    const uint64_t n = h->n;
    if ((r = dalloc(hp, &h->d_cnt[0], n * h->stride))) return fail(r);
    if ((r = dalloc(hp, &h->d_cnt[1], n * h->stride))) return fail(r);
    if (o.far_rows) h->far_rows = std::min<uint32_t>(o.far_rows, 0x7fffffffu);
    if (o.flags & HB_TMA_GATHER)
        h->far_ok = hbk::encode_far_map(h->log2m, h->d_cnt[0], n, &h->far_map[0]) == 0 &&
                    hbk::encode_far_map(h->log2m, h->d_cnt[1], n, &h->far_map[1]) == 0;
    const uint64_t words = (n + 31) / 32;
    for (int b = 0; b < 4; b++)
        if ((r = dalloc(hp, &h->d_bits[b], words))) return fail(r);
    if ((r = dalloc(hp, &h->d_est, n))) return fail(r);
    if (h->do_sod && (r = dalloc(hp, &h->d_sod, n))) return fail(r);
    if (h->do_harm && (r = dalloc(hp, &h->d_harm, n))) return fail(r);
    {
        const uint64_t mm = 1ull << o.log2m;
        std::vector<double> lnt(mm + 1, 0.0);
        const double mf = (double)mm;
        for (uint64_t z = 1; z <= mm; z++) lnt[z] = mf * std::log(mf / (double)z);
        // Host-to-device copies of the handle go on its own stream: a plain
        // cudaMemcpy from pageable memory may return before its DMA lands and
        // orders nothing on the handle's non-blocking streams (the init
        // kernel once read a table that was still on its way: every initial
        // estimate 0 in a served job). A pageable source is staged before
        // cudaMemcpyAsync returns, so it may go out of scope right after.
        if ((r = dalloc(hp, &h->d_lnt, mm + 1))) return fail(r);
        if ((r = cuda_err(hp, cudaMemcpyAsync(h->d_lnt, lnt.data(), (mm + 1) * 8, cudaMemcpyHostToDevice,
                                              h->stream),
                          "cudaMemcpyAsync")))
            return fail(r);
    }
    if (o.weights) {
        if ((r = dalloc(hp, &h->d_weights, n))) return fail(r);
        if ((r = cuda_err(hp, cudaMemcpyAsync(h->d_weights, o.weights, n * 8, cudaMemcpyHostToDevice,
                                              h->stream),
                          "cudaMemcpyAsync")))
            return fail(r);
    }
    trace.mark("state arrays");
    h->grid_tile = hbk::tile_grid(h->log2m, h->device, 0);
    h->grid_tile_occ = hbk::tile_grid(h->log2m, h->device, 1);
    h->grid_tile_two = hbk::tile_grid(h->log2m, h->device, 2);
    h->grid_staged = hbk::staged_grid(h->log2m, h->device, 0);
    h->grid_staged_occ = hbk::staged_grid(h->log2m, h->device, 1);
    {
        // one warp per chunk, 8 warps per block
        const uint64_t need = (h->n_chunks + 7) / 8 + 1;
        if ((uint64_t)h->grid_tile > need) h->grid_tile = (int)need;
        if ((uint64_t)h->grid_tile_occ > need) h->grid_tile_occ = (int)need;
        if ((uint64_t)h->grid_tile_two > need) h->grid_tile_two = (int)need;
        if ((uint64_t)h->grid_staged > need) h->grid_staged = (int)need;
        if ((uint64_t)h->grid_staged_occ > need) h->grid_staged_occ = (int)need;
    }
    // the staged kernel's item table (arc positions are u32 there)
    if (h->n_chunks && h->m + 64 < (1ull << 32)) {
        if ((r = dalloc(hp, &h->d_items, h->n_chunks))) return fail(r);
        if ((r = cuda_err(hp, (cudaError_t)hbk::launch_chunk_items(h->d_chunks, h->n_chunks, h->d_off,
                                                                   h->d_items, h->stream),
                          "k_chunk_items")))
            return fail(r);
    }
    if (o.union_variant != HB_AUTO) {
        if (o.union_variant >= (uint32_t)kNumVariants)
            return fail(set_err(hp, HB_ERR_INVALID, "union_variant out of range"));
        h->tuner.fixed = (int)o.union_variant;
    } else {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(TuneKey{h->device, h->log2m, h->n, h->m});
        if (it != g_tune_cache.end())
            for (int c = 0; c < kTunedClasses; c++) h->tuner.chosen[c] = it->second[c];
    }
    h->grid_heavy = hbk::heavy_grid(h->log2m, h->device);
    if ((uint64_t)h->grid_heavy > h->n_heavy_items + 1) h->grid_heavy = (int)(h->n_heavy_items + 1);
    h->grid_mark = 8 * hbk::num_sms(h->device);
    // integer totals of the union kernels (atomics) and the summed
    // neighbourhood function
    h->n_partials = 1;
    if ((r = dalloc(hp, &h->d_partials, h->n_partials))) return fail(r);
    if ((r = dalloc(hp, &h->d_nf_items, h->n_chunks + h->n_heavy + 1))) return fail(r);
    if ((r = dalloc(hp, &h->d_nf_scratch, 256))) return fail(r);
    if ((r = dalloc(hp, &h->d_any31, 1))) return fail(r);
    if ((r = dalloc(hp, &h->d_ic, 1))) return fail(r);
    if ((r = dalloc(hp, &h->d_cursor, 1))) return fail(r);
    if ((r = cuda_err(hp, cudaStreamSynchronize(h->stream), "cudaStreamSynchronize"))) return fail(r);
    trace.mark("launch setup");
    *out = h.release();
    return HB_OK;
}

int hb_create(const hb_graph_view* graph, const hb_graph_view* transpose, const hb_options* opts,
              hb_handle** out) {
    return create_impl(graph, transpose, opts, nullptr, out);
}

int hb_add_discount_function(hb_handle* h, hb_discount_fn fn, void* ctx) {
    if (!h || !fn) return set_err(h, HB_ERR_INVALID, "handle or function is NULL");
    if ((int)h->disc_fn.size() >= hbk::MAX_DISCOUNT)
        return set_err(h, HB_ERR_INVALID, "at most 8 discount functions");
    double* d = nullptr;
    int r = dalloc(h, &d, h->n);
    if (r) return r;
    h->disc_fn.push_back(fn);
    h->disc_ctx.push_back(ctx);
    h->d_disc.push_back(d);
    return HB_OK;
}

void hb_destroy(hb_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    release(h);
    delete h;
}

int hb_init(hb_handle* h) {
    if (!h) return set_err(nullptr, HB_ERR_INVALID, "handle is NULL");
    LaunchTally tally(h);
    HB_CUDA(h, cudaSetDevice(h->device));
    return do_init(h);
}

int hb_iterate(hb_handle* h, hb_iter_stats* out) {
    if (!h) return set_err(nullptr, HB_ERR_INVALID, "handle is NULL");
    LaunchTally tally(h);
    if (!h->initialised) return set_err(h, HB_ERR_NOT_RUN, "hb_init must precede hb_iterate");
    HB_CUDA(h, cudaSetDevice(h->device));
    return do_iterate(h, out);
}

int hb_run(hb_handle* h, uint64_t upper_bound, double threshold) {
    if (!h) return set_err(nullptr, HB_ERR_INVALID, "handle is NULL");
    LaunchTally tally(h);
    HB_CUDA(h, cudaSetDevice(h->device));
    upper_bound = std::min<uint64_t>(upper_bound, h->n);  // HB:541
    int r = do_init(h);
    if (r) return r;
    for (uint64_t i = 0; i < upper_bound; i++) {
        if ((r = do_iterate(h, nullptr))) return r;
        if (h->modified_counters == 0) break;  // HB:559-570
        if (!std::isnan(threshold) && i > 3 && h->relative_increment < 1.0 + threshold) break;
    }
    return HB_OK;
}

int hb_run_until_stable(hb_handle* h, uint64_t upper_bound) { return hb_run(h, upper_bound, NAN); }
int hb_run_until_done(hb_handle* h) { return hb_run(h, UINT64_MAX, NAN); }

int hb_tune_degree_buckets(const hb_graph_view* graph, const hb_options* opts, uint32_t iterations,
                           uint32_t* small_max, uint32_t* medium_max, double* union_ms) {
    if (!graph || !opts || !small_max || !medium_max)
        return set_err(nullptr, HB_ERR_INVALID, "NULL argument");
    if (opts->struct_size != sizeof(hb_options))
        return set_err(nullptr, HB_ERR_INVALID, "hb_options.struct_size mismatch");
    iterations = std::max<uint32_t>(iterations, 2);
    // lane-group nodes up to 32..1024 successors; 8-lane teams up to 4096..65536
    static const uint32_t kSmall[] = {32, 64, 128, 256, 512, 1024};
    static const uint32_t kMedium[] = {4096, 16384, 65536};
    double best = INFINITY, dflt = INFINITY;
    uint32_t bs = 32, bm = 4096;
    for (uint32_t sm : kSmall)
        for (uint32_t mm : kMedium) {
            hb_options o = *opts;
            o.small_max_degree = sm;
            o.medium_max_degree = mm;
            // standard iterations only (they carry the union work), on one
            // fixed kernel variant so that only the buckets differ
            o.flags &= ~HB_TRANSPOSE_ON_DEVICE;
            o.flags |= HB_NO_GRAPHS;
            if (o.union_variant == HB_AUTO) o.union_variant = 0;
            hb_handle* h = nullptr;
            int r = hb_create(graph, nullptr, &o, &h);
            if (r) return r;
            r = hb_init(h);
            double t = 0.0;
            for (uint32_t i = 0; r == HB_OK && i < iterations; i++) {
                hb_iter_stats st{};
                r = hb_iterate(h, &st);
                if (r == HB_OK && i > 0) t += st.union_ms;  // the first iteration warms up
                if (r == HB_OK && st.modified_counters == 0) break;
            }
            if (r) {
                g_global_err = h->err;
                hb_destroy(h);
                return r;
            }
            hb_destroy(h);
            if (sm == kDefaultSmallMax && mm == kDefaultMediumMax) dflt = t;
            if (t < best) {
                best = t;
                bs = sm;
                bm = mm;
            }
        }
    // one sample each: another pair must beat the default by a clear margin
    // (the same graph gave 64 or 128 from run to run, 9.1 against 9.5 ms per
    // standard iteration at 2^26)
    if (best > 0.98 * dflt) {
        bs = kDefaultSmallMax;
        bm = kDefaultMediumMax;
        best = dflt;
    }
    *small_max = bs;
    *medium_max = bm;
    if (union_ms) *union_ms = best;
    return HB_OK;
}

uint64_t hb_num_iterations(const hb_handle* h) { return h ? h->iteration : 0; }

int hb_get_iteration_stats(const hb_handle* h, uint64_t i, hb_iter_stats* out) {
    if (!h || !out) return set_err(nullptr, HB_ERR_INVALID, "NULL argument");
    if (i >= h->stats.size()) return set_err(const_cast<hb_handle*>(h), HB_ERR_INVALID, "no such iteration");
    *out = h->stats[i];
    return HB_OK;
}

int hb_get_neighborhood_function(const hb_handle* h, double* dst, size_t capacity, size_t* len) {
    int r = ensure_iteration(h);
    if (r) return r;
    if (len) *len = h->nf.size();
    if (dst) std::memcpy(dst, h->nf.data(), std::min(capacity, h->nf.size()) * sizeof(double));
    return HB_OK;
}

int hb_get_sum_of_distances(const hb_handle* h, double* dst, size_t len) {
    int r = ensure_iteration(h);
    if (r) return r;
    if (!h->d_sod)
        return set_err(const_cast<hb_handle*>(h), HB_ERR_NOT_REQUESTED,
                       "Sum of distances were not requested. Set HB_SUM_OF_DISTANCES while building HyperBall to compute them");
    if ((r = check_len(h, len))) return r;
    return copy_nodes_d2h(h, h->d_sod, dst);
}

int hb_get_harmonic_centralities(const hb_handle* h, double* dst, size_t len) {
    int r = ensure_iteration(h);
    if (r) return r;
    if (!h->d_harm)
        return set_err(const_cast<hb_handle*>(h), HB_ERR_NOT_REQUESTED,
                       "Sum of inverse distances were not requested. Set HB_SUM_OF_INVERSE_DISTANCES while building HyperBall to compute them");
    if ((r = check_len(h, len))) return r;
    return copy_nodes_d2h(h, h->d_harm, dst);
}

int hb_get_discounted_centrality(const hb_handle* h, size_t index, double* dst, size_t len) {
    int r = ensure_iteration(h);
    if (r) return r;
    if (index >= h->d_disc.size())
        return set_err(const_cast<hb_handle*>(h), HB_ERR_NOT_REQUESTED,
                       "Discount centrality of index " + std::to_string(index) + " does not exist");
    if ((r = check_len(h, len))) return r;
    return copy_nodes_d2h(h, h->d_disc[index], dst);
}

int hb_get_closeness_centrality(const hb_handle* h, double* dst, size_t len) {
    int r = hb_get_sum_of_distances(h, dst, len);
    if (r) {
        if (r == HB_ERR_NOT_REQUESTED)
            const_cast<hb_handle*>(h)->err =
                "Sum of distances were not requested. Set HB_SUM_OF_DISTANCES while building HyperBall to compute closeness centrality";
        return r;
    }
    for (size_t i = 0; i < len; i++) dst[i] = dst[i] == 0.0 ? 0.0 : 1.0 / dst[i];
    return HB_OK;
}

int hb_get_reachable_nodes(const hb_handle* h, double* dst, size_t len) {
    int r = ensure_iteration(h);
    if (r) return r;
    if ((r = check_len(h, len))) return r;
    return copy_nodes_d2h(h, h->d_est, dst);
}

int hb_reachable_nodes_from(const hb_handle* h, uint64_t node, double* out) {
    int r = ensure_iteration(h);
    if (r) return r;
    if (node >= h->n || !out) return set_err(const_cast<hb_handle*>(h), HB_ERR_INVALID, "node out of range");
    uint32_t dev_node = 0;
    if ((r = copy_d2h(h, h->d_inv + node, &dev_node, 4))) return r;
    return copy_d2h(h, h->d_est + dev_node, out, 8);
}

static int lin_or_nieminen(const hb_handle* h, double* dst, size_t len, bool lin) {
    int r = hb_get_sum_of_distances(h, dst, len);
    if (r) {
        if (r == HB_ERR_NOT_REQUESTED)
            const_cast<hb_handle*>(h)->err =
                lin ? "Sum of distances were not requested. Set HB_SUM_OF_DISTANCES while building HyperBall to compute lin centrality"
                    : "Sum of distances were not requested. Set HB_SUM_OF_DISTANCES while building HyperBall to compute nieminen centrality";
        return r;
    }
    std::vector<double> cnt(len);
    if ((r = copy_nodes_d2h(h, h->d_est, cnt.data()))) return r;
    for (size_t i = 0; i < len; i++) {
        const double d = dst[i];
        if (lin) {
            dst[i] = d == 0.0 ? 1.0 : cnt[i] * cnt[i] / d;
        } else {
            dst[i] = (cnt[i] * cnt[i]) - d;
        }
    }
    return HB_OK;
}

int hb_get_lin_centrality(const hb_handle* h, double* dst, size_t len) {
    return lin_or_nieminen(h, dst, len, true);
}
int hb_get_nieminen_centrality(const hb_handle* h, double* dst, size_t len) {
    return lin_or_nieminen(h, dst, len, false);
}

int hb_get_registers(const hb_handle* h, int which, void* dst, size_t bytes) {
    if (!h || !dst) return set_err(nullptr, HB_ERR_INVALID, "NULL argument");
    if (bytes != h->n * h->counter_bytes)
        return set_err(const_cast<hb_handle*>(h), HB_ERR_INVALID, "bytes must be num_nodes * counter bytes");
    if (which != HB_CURRENT_STATE && which != HB_NEXT_STATE)
        return set_err(const_cast<hb_handle*>(h), HB_ERR_INVALID, "which must be HB_CURRENT_STATE or HB_NEXT_STATE");
    // the device keeps a byte per register; pack into the reference's layout
    return copy_registers_range(h, which, dst, 0, h->n);
}

int hb_union_variant_count(void) { return kNumVariants; }

int hb_union_variant_chosen(const hb_handle* h, int32_t chosen[3]) {
    if (!h || !chosen) return set_err(const_cast<hb_handle*>(h), HB_ERR_INVALID, "null argument");
    const Tuner& t = h->tuner;
    for (int c = 0; c < kTunedClasses; c++) chosen[c] = t.fixed >= 0 ? t.fixed : t.chosen[c];
    chosen[2] = t.fixed >= 0 ? t.fixed : 0;
    return HB_OK;
}

int hb_counter_layout(const hb_handle* h, uint64_t* counter_bytes, int* reg_size) {
    if (!h) return set_err(nullptr, HB_ERR_INVALID, "handle is NULL");
    if (counter_bytes) *counter_bytes = h->counter_bytes;
    if (reg_size) *reg_size = register_size(h->num_elements);
    return HB_OK;
}

// ---- graphs -----------------------------------------------------------------
int hb_graph_load_bvgraph(const char* basename, hb_graph** out) {
    if (!basename || !out) return set_err(nullptr, HB_ERR_INVALID, "NULL argument");
    std::unique_ptr<hb_graph> g(new hb_graph());
    std::string err;
    uint64_t checked = 0;
    int r = hbg::load_bvgraph(basename, g->g, err, &checked);
    if (r) return set_err(nullptr, r, err);
    *out = g.release();
    return HB_OK;
}

int hb_graph_generate_er(uint64_t n, uint32_t d, uint64_t seed, hb_graph** out) {
    if (!out) return set_err(nullptr, HB_ERR_INVALID, "NULL argument");
    if (n > 0xffffffffull) return set_err(nullptr, HB_ERR_INVALID, "too many nodes");
    std::unique_ptr<hb_graph> g(new hb_graph());
    hbg::gen_er(n, d, seed, g->g);
    *out = g.release();
    return HB_OK;
}

int hb_graph_generate_rmat(int scale, uint64_t epn, double a, double b, double c, uint64_t seed,
                           hb_graph** out) {
    if (!out || scale < 1 || scale > 31 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
        return set_err(nullptr, HB_ERR_INVALID, "invalid R-MAT parameters");
    std::unique_ptr<hb_graph> g(new hb_graph());
    hbg::gen_rmat(scale, epn, a, b, c, seed, g->g);
    *out = g.release();
    return HB_OK;
}

int hb_graph_generate_weblike(uint64_t n, uint64_t cap, double shift, uint64_t window, uint64_t seed,
                              hb_graph** out) {
    if (!out || n == 0 || n > 0xffffffffull || cap == 0 || !(shift >= 0.0))
        return set_err(nullptr, HB_ERR_INVALID, "invalid web-like parameters");
    std::unique_ptr<hb_graph> g(new hb_graph());
    hbg::gen_weblike(n, cap, shift, window, seed, g->g);
    *out = g.release();
    return HB_OK;
}

int hb_graph_transpose(const hb_graph* g, hb_graph** out) {
    if (!g || !out) return set_err(nullptr, HB_ERR_INVALID, "NULL argument");
    std::unique_ptr<hb_graph> t(new hb_graph());
    hbg::transpose(g->g, t->g);
    *out = t.release();
    return HB_OK;
}

int hb_graph_from_csr(const hb_graph_view* v, hb_graph** out) {
    std::string why;
    if (!out) return set_err(nullptr, HB_ERR_INVALID, "NULL argument");
    if (!check_view(v, why)) return set_err(nullptr, HB_ERR_INVALID, why);
    std::unique_ptr<hb_graph> g(new hb_graph());
    g->g.n = v->num_nodes;
    g->g.m = v->num_arcs;
    g->g.offsets.assign(v->offsets, v->offsets + v->num_nodes + 1);
    g->g.successors.assign(v->successors, v->successors + v->num_arcs);
    *out = g.release();
    return HB_OK;
}

hb_graph_view hb_graph_get_view(const hb_graph* g) {
    hb_graph_view v{};
    if (!g) return v;
    v.num_nodes = g->g.n;
    v.num_arcs = g->g.m;
    v.offsets = g->g.offsets.data();
    v.successors = g->g.successors.data();
    return v;
}

void hb_graph_free(hb_graph* g) { delete g; }

}  // extern "C"
