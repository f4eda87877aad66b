// Breadth-first visits on the device: the GB300 counterpart of the
// reference's fair parallel breadth-first visit (ParFair,
// src/algo/visits/breadth_first/par_fair.rs:92-330) and, run root by root,
// of the sequential one (seq.rs:113-224).
//
// State: the graph in device CSR, a visited bitmap that persists across
// visits until hb_visit_reset (par_fair.rs:101, 322-324), and a queue that
// holds every node visited since the last reset in visit order, with its
// predecessor. A visit is level-synchronous like the reference's frontier
// loop (par_fair.rs:169-213):
//   k_visit_roots   roots not yet visited are marked and form level 0;
//   k_visit_expand  one warp per frontier node walks its successors 32 at a
//                   time; a successor whose visited bit a lane sets first
//                   (atomicOr, after a plain read that skips the common
//                   already-visited case) is staged with its predecessor
//                   in the warp's run in shared memory, and a run goes to
//                   the next level with one atomicAdd on the tail per up to
//                   RUN nodes; nodes with more than HEAVY_MIN successors
//                   are deferred to
//   k_visit_heavy   one block per node.
// The Unknown events of the reference (node, pred, distance) are the queue
// slots of the visit with the level of each slot; Known events are counted.
// Within a level the order is unspecified, as in the reference's parallel
// visit; distances are exact, and the predecessor of a node is a node of
// the previous level with an arc to it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "hb_internal.h"

namespace hbv {

constexpr uint32_t HEAVY_MIN = 4096;

__device__ __forceinline__ bool claim(uint32_t* visited, uint32_t s) {
    const uint32_t w = s >> 5, bit = 1u << (s & 31);
    if (*(volatile uint32_t*)(visited + w) & bit) return false;
    return !(atomicOr(visited + w, bit) & bit);
}

// appends the lanes' claimed nodes (warp-aggregated), with predecessor p
__device__ __forceinline__ void append(bool c, uint32_t s, uint32_t p, uint32_t* queue, uint32_t* pred,
                                       unsigned long long* tail) {
    const unsigned mask = __ballot_sync(0xffffffffu, c);
    if (!mask) return;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == __ffs(mask) - 1) base = atomicAdd(tail, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
    if (c) {
        const unsigned long long slot = base + __popc(mask & ((1u << lane) - 1u));
        queue[slot] = s;
        pred[slot] = p;
    }
}

// A warp's claimed nodes and their predecessors wait in shared memory and
// go to the queue in runs of up to RUN slots: a per-chunk append puts one
// same-address atomic on the tail in the chain of almost every frontier
// node of a level of many small-degree nodes.
constexpr int RUN = 128;
constexpr int EXPAND_THREADS = 256;

// writes the warp's run [0, fill) to the queue (every lane of the warp)
__device__ __forceinline__ void write_run(const uint32_t* rn, const uint32_t* rp, int fill, uint32_t* queue,
                                          uint32_t* pred, unsigned long long* tail) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(tail, (unsigned long long)fill);
    base = __shfl_sync(0xffffffffu, base, 0);
    for (int k = lane; k < fill; k += 32) {
        queue[base + k] = rn[k];
        pred[base + k] = rp[k];
    }
    __syncwarp();
}

// adds the lanes' claimed nodes (predecessor p) to the warp's run, writing
// the run out when another chunk might not fit (every lane of the warp)
__device__ __forceinline__ void stage(bool c, uint32_t s, uint32_t p, uint32_t* rn, uint32_t* rp, int& fill,
                                      uint32_t* queue, uint32_t* pred, unsigned long long* tail) {
    const unsigned mask = __ballot_sync(0xffffffffu, c);
    if (c) {
        const int k = fill + __popc(mask & ((1u << (threadIdx.x & 31)) - 1u));
        rn[k] = s;
        rp[k] = p;
    }
    fill += __popc(mask);
    if (fill > RUN - 32) {
        write_run(rn, rp, fill, queue, pred, tail);
        fill = 0;
    }
}

__global__ void k_visit_roots(const uint32_t* __restrict__ roots, uint64_t nroots, uint32_t* visited,
                              uint32_t* queue, uint32_t* pred, unsigned long long* tail) {
    // whole warps iterate together (the limit is a multiple of 32) so that
    // every lane of a warp takes part in the append
    const uint64_t limit = (nroots + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < limit;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const bool in = i < nroots;
        const uint32_t r = in ? roots[i] : 0u;
        const bool c = in && claim(visited, r);
        append(c, r, r, queue, pred, tail);
    }
}

// level [b, e) of the queue -> the next level, appended at *tail
__global__ void k_visit_expand(const uint64_t* __restrict__ off, const uint32_t* __restrict__ succ,
                               uint32_t* visited, uint32_t* queue, uint32_t* pred, uint64_t b,
                               uint64_t e, unsigned long long* tail, uint32_t* heavy,
                               unsigned long long* heavy_n, unsigned long long* known) {
    __shared__ uint32_t run_node[EXPAND_THREADS / 32][RUN], run_pred[EXPAND_THREADS / 32][RUN];
    uint32_t* rn = run_node[threadIdx.x >> 5];
    uint32_t* rp = run_pred[threadIdx.x >> 5];
    int fill = 0;  // the same in every lane of the warp
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long kn = 0;
    for (uint64_t i = b + warp; i < e; i += warps) {
        const uint32_t v = queue[i];
        const uint64_t s0 = off[v], s1 = off[v + 1];
        if (s1 - s0 > HEAVY_MIN) {
            if (lane == 0) heavy[atomicAdd(heavy_n, 1ull)] = v;
            continue;
        }
        for (uint64_t a = s0; a < s1; a += 32) {
            const uint64_t x = a + lane;
            uint32_t s = 0;
            bool c = false;
            if (x < s1) {
                s = __ldg(succ + x);
                c = claim(visited, s);
                kn += !c;
            }
            stage(c, s, v, rn, rp, fill, queue, pred, tail);
        }
    }
    if (fill) write_run(rn, rp, fill, queue, pred, tail);
    if (kn) atomicAdd(known, kn);
}

// the deferred nodes of a level, one block each
__global__ void k_visit_heavy(const uint64_t* __restrict__ off, const uint32_t* __restrict__ succ,
                              uint32_t* visited, uint32_t* queue, uint32_t* pred,
                              unsigned long long* tail, const uint32_t* heavy,
                              const unsigned long long* heavy_n, unsigned long long* known) {
    const uint64_t count = *heavy_n;
    unsigned long long kn = 0;
    for (uint64_t h = blockIdx.x; h < count; h += gridDim.x) {
        const uint32_t v = heavy[h];
        const uint64_t s0 = off[v], s1 = off[v + 1];
        for (uint64_t a = s0; a < s1; a += blockDim.x) {
            const uint64_t x = a + threadIdx.x;
            uint32_t s = 0;
            bool c = false;
            if (x < s1) {
                s = __ldg(succ + x);
                c = claim(visited, s);
                kn += !c;
            }
            append(c, s, v, queue, pred, tail);
        }
    }
    if (kn) atomicAdd(known, kn);
}

__global__ void k_visit_validate(const uint64_t* __restrict__ off, const uint32_t* __restrict__ succ,
                                 uint64_t n, uint64_t m, int* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint64_t v = t0; v < n; v += stride)
        if (off[v] > off[v + 1]) *bad = 1;
    for (uint64_t x = t0; x < m; x += stride)
        if (succ[x] >= n) *bad = 1;
}

}  // namespace hbv

struct hb_visit {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint64_t n = 0, m = 0;
    uint64_t* d_off = nullptr;
    uint32_t* d_succ = nullptr;
    uint32_t* d_visited = nullptr;
    uint32_t* d_queue = nullptr;   // every node visited since the last reset, in visit order
    uint32_t* d_pred = nullptr;
    uint32_t* d_heavy = nullptr;
    uint32_t* d_roots = nullptr;   // roots of the current visit (capacity n)
    unsigned long long* d_cnt = nullptr;   // [0] tail, [1] deferred nodes, [2] known arcs
    unsigned long long* h_cnt = nullptr;   // page-locked copy
    uint64_t tail = 0;
    int sms = 1;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<uint32_t> host_visited;    // copy of d_visited (visit_each)
    std::string err;
};

static thread_local std::string t_visit_err;

static int visit_err(hb_visit* v, int code, const std::string& msg) {
    if (v) v->err = msg;
    t_visit_err = msg;
    return code;
}

static int visit_cuda(hb_visit* v, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return HB_OK;
    cudaGetLastError();
    const int code = e == cudaErrorMemoryAllocation ? HB_ERR_OOM
                     : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? HB_ERR_NO_DEVICE
                                                                                     : HB_ERR_CUDA;
    return visit_err(v, code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define VC(v, call, what)                               \
    do {                                                \
        int _r = visit_cuda((v), (call), (what));       \
        if (_r) return _r;                              \
    } while (0)

static void visit_free(hb_visit* v) {
    if (!v) return;
    cudaSetDevice(v->device);
    if (v->stream) cudaStreamSynchronize(v->stream);
    cudaFree(v->d_off);
    cudaFree(v->d_succ);
    cudaFree(v->d_visited);
    cudaFree(v->d_queue);
    cudaFree(v->d_pred);
    cudaFree(v->d_heavy);
    cudaFree(v->d_roots);
    cudaFree(v->d_cnt);
    if (v->h_cnt) cudaFreeHost(v->h_cnt);
    if (v->ev0) cudaEventDestroy(v->ev0);
    if (v->ev1) cudaEventDestroy(v->ev1);
    if (v->own_stream && v->stream) cudaStreamDestroy(v->stream);
    delete v;
}

extern "C" {

int hb_visit_create(const hb_graph_view* g, int device, void* stream, hb_visit** out) {
    if (!out) return visit_err(nullptr, HB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!g || !g->offsets || (g->num_arcs && !g->successors))
        return visit_err(nullptr, HB_ERR_INVALID, "graph arrays must not be NULL");
    if (g->num_nodes >= 0xffffffffull)
        return visit_err(nullptr, HB_ERR_INVALID, "node ids must fit u32");
    if (g->offsets[0] != 0 || g->offsets[g->num_nodes] != g->num_arcs)
        return visit_err(nullptr, HB_ERR_INVALID,
                         "offsets[0] must be 0 and offsets[num_nodes] must equal num_arcs");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return visit_err(nullptr, HB_ERR_NO_DEVICE, "no CUDA device available (this library has no CPU path)");
    }
    hb_visit* v = new hb_visit();
    v->device = device;
    v->n = g->num_nodes;
    v->m = g->num_arcs;
    const uint64_t n = v->n, m = v->m, words = (n + 31) / 32;
    auto fail = [&](int r) {
        visit_free(v);
        return r;
    };
    int r;
    if ((r = visit_cuda(v, cudaSetDevice(device), "cudaSetDevice"))) return fail(r);
    if (stream) {
        v->stream = (cudaStream_t)stream;
    } else {
        if ((r = visit_cuda(v, cudaStreamCreateWithFlags(&v->stream, cudaStreamNonBlocking),
                            "cudaStreamCreate")))
            return fail(r);
        v->own_stream = true;
    }
    cudaDeviceGetAttribute(&v->sms, cudaDevAttrMultiProcessorCount, device);
    const size_t nn = std::max<uint64_t>(n, 1);
    if ((r = visit_cuda(v, cudaMalloc((void**)&v->d_off, (n + 1) * 8), "cudaMalloc")) ||
        (r = visit_cuda(v, cudaMalloc((void**)&v->d_succ, std::max<uint64_t>(m, 1) * 4), "cudaMalloc")) ||
        (r = visit_cuda(v, cudaMalloc((void**)&v->d_visited, std::max<uint64_t>(words, 1) * 4), "cudaMalloc")) ||
        (r = visit_cuda(v, cudaMalloc((void**)&v->d_queue, nn * 4), "cudaMalloc")) ||
        (r = visit_cuda(v, cudaMalloc((void**)&v->d_pred, nn * 4), "cudaMalloc")) ||
        (r = visit_cuda(v, cudaMalloc((void**)&v->d_heavy, nn * 4), "cudaMalloc")) ||
        (r = visit_cuda(v, cudaMalloc((void**)&v->d_roots, nn * 4), "cudaMalloc")) ||
        (r = visit_cuda(v, cudaMalloc((void**)&v->d_cnt, 4 * 8), "cudaMalloc")) ||
        (r = visit_cuda(v, cudaMallocHost((void**)&v->h_cnt, 4 * 8), "cudaMallocHost")))
        return fail(r);
    if ((r = visit_cuda(v, cudaMemcpyAsync(v->d_off, g->offsets, (n + 1) * 8, cudaMemcpyHostToDevice, v->stream),
                        "cudaMemcpyAsync")))
        return fail(r);
    if (m && (r = visit_cuda(v, cudaMemcpyAsync(v->d_succ, g->successors, m * 4, cudaMemcpyHostToDevice,
                                                v->stream),
                             "cudaMemcpyAsync")))
        return fail(r);
    // the CSR is checked before any kernel indexes with it
    int* d_bad = (int*)(v->d_cnt + 3);
    int bad = 0;
    if ((r = visit_cuda(v, cudaMemsetAsync(d_bad, 0, sizeof(int), v->stream), "cudaMemsetAsync"))) return fail(r);
    const int grid = (int)std::min<uint64_t>((std::max(n, m) + 255) / 256 + 1, 8192);
    hbv::k_visit_validate<<<grid, 256, 0, v->stream>>>(v->d_off, v->d_succ, n, m, d_bad);
    if ((r = visit_cuda(v, cudaGetLastError(), "k_visit_validate")) ||
        (r = visit_cuda(v, cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, v->stream),
                        "cudaMemcpyAsync")) ||
        (r = visit_cuda(v, cudaStreamSynchronize(v->stream), "cudaStreamSynchronize")))
        return fail(r);
    if (bad) return fail(visit_err(v, HB_ERR_INVALID, "graph has decreasing offsets or successors >= num_nodes"));
    v->host_visited.assign(std::max<uint64_t>(words, 1), 0);
    if ((r = visit_cuda(v, cudaEventCreate(&v->ev0), "cudaEventCreate")) ||
        (r = visit_cuda(v, cudaEventCreate(&v->ev1), "cudaEventCreate")))
        return fail(r);
    if ((r = visit_cuda(v, cudaMemsetAsync(v->d_visited, 0, std::max<uint64_t>(words, 1) * 4, v->stream),
                        "cudaMemsetAsync")) ||
        (r = visit_cuda(v, cudaStreamSynchronize(v->stream), "cudaStreamSynchronize")))
        return fail(r);
    *out = v;
    return HB_OK;
}

void hb_visit_destroy(hb_visit* v) { visit_free(v); }

int hb_visit_reset(hb_visit* v) {
    if (!v) return visit_err(nullptr, HB_ERR_INVALID, "visit is NULL");
    VC(v, cudaSetDevice(v->device), "cudaSetDevice");
    const uint64_t words = (v->n + 31) / 32;
    VC(v, cudaMemsetAsync(v->d_visited, 0, std::max<uint64_t>(words, 1) * 4, v->stream), "cudaMemsetAsync");
    VC(v, cudaStreamSynchronize(v->stream), "cudaStreamSynchronize");
    v->tail = 0;
    return HB_OK;
}

int hb_visit_run(hb_visit* v, const uint64_t* roots, size_t nroots, uint64_t max_distance,
                 uint32_t* nodes, uint32_t* preds, uint32_t* dists, size_t capacity,
                 hb_visit_stats* stats) {
    if (!v) return visit_err(nullptr, HB_ERR_INVALID, "visit is NULL");
    if (nroots && !roots) return visit_err(v, HB_ERR_INVALID, "roots is NULL");
    for (size_t i = 0; i < nroots; i++)
        if (roots[i] >= v->n) return visit_err(v, HB_ERR_INVALID, "root " + std::to_string(roots[i]) + " >= num_nodes");
    VC(v, cudaSetDevice(v->device), "cudaSetDevice");
    cudaStream_t s = v->stream;
    hb_visit_stats st{};
    const uint64_t q0 = v->tail;
    std::vector<uint64_t> level_end;
    if (nroots) {
        std::vector<uint32_t> r32(nroots);
        for (size_t i = 0; i < nroots; i++) r32[i] = (uint32_t)roots[i];
        // d_roots holds n roots: longer lists (repeated roots) go in pieces
        const uint64_t nr = std::min<uint64_t>(nroots, std::max<uint64_t>(v->n, 1));
        unsigned long long zero2[3] = {q0, 0, 0};
        VC(v, cudaMemcpyAsync(v->d_cnt, zero2, 3 * 8, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        VC(v, cudaEventRecord(v->ev0, s), "cudaEventRecord");
        for (size_t at = 0; at < nroots; at += nr) {
            const uint64_t k = std::min<uint64_t>(nr, nroots - at);
            VC(v, cudaMemcpyAsync(v->d_roots, r32.data() + at, k * 4, cudaMemcpyHostToDevice, s),
               "cudaMemcpyAsync");
            const int grid = (int)std::min<uint64_t>((k + 31 + 255) / 256, 4096);
            hbv::k_visit_roots<<<grid, 256, 0, s>>>(v->d_roots, k, v->d_visited, v->d_queue, v->d_pred,
                                                    v->d_cnt);
            VC(v, cudaGetLastError(), "k_visit_roots");
            // the next piece's copy must not overwrite roots still being read
            VC(v, cudaStreamSynchronize(s), "cudaStreamSynchronize");
        }
        VC(v, cudaMemcpyAsync(v->h_cnt, v->d_cnt, 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        VC(v, cudaStreamSynchronize(s), "cudaStreamSynchronize");
        uint64_t b = q0, e = v->h_cnt[0];
        if (e > b) level_end.push_back(e);
        const int egrid = v->sms * 8, hgrid = v->sms * 2;
        uint64_t d = 0;
        while (e > b && d < max_distance) {
            VC(v, cudaMemsetAsync(v->d_cnt + 1, 0, 8, s), "cudaMemsetAsync");
            const int g1 = (int)std::min<uint64_t>(((e - b) * 32 + hbv::EXPAND_THREADS - 1) / hbv::EXPAND_THREADS,
                                                   (uint64_t)egrid);
            hbv::k_visit_expand<<<g1, hbv::EXPAND_THREADS, 0, s>>>(v->d_off, v->d_succ, v->d_visited, v->d_queue, v->d_pred,
                                                   b, e, v->d_cnt, v->d_heavy, v->d_cnt + 1, v->d_cnt + 2);
            VC(v, cudaGetLastError(), "k_visit_expand");
            hbv::k_visit_heavy<<<hgrid, 256, 0, s>>>(v->d_off, v->d_succ, v->d_visited, v->d_queue, v->d_pred,
                                                     v->d_cnt, v->d_heavy, v->d_cnt + 1, v->d_cnt + 2);
            VC(v, cudaGetLastError(), "k_visit_heavy");
            VC(v, cudaMemcpyAsync(v->h_cnt, v->d_cnt, 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
            VC(v, cudaStreamSynchronize(s), "cudaStreamSynchronize");
            b = e;
            e = v->h_cnt[0];
            if (e > b) level_end.push_back(e);
            d++;
        }
        VC(v, cudaEventRecord(v->ev1, s), "cudaEventRecord");
        VC(v, cudaMemcpyAsync(v->h_cnt, v->d_cnt, 3 * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        VC(v, cudaStreamSynchronize(s), "cudaStreamSynchronize");
        v->tail = v->h_cnt[0];
        st.known_arcs = v->h_cnt[2];
        float ms = 0.f;
        cudaEventElapsedTime(&ms, v->ev0, v->ev1);
        st.device_ms = ms;
    }
    const uint64_t count = v->tail - q0;
    st.visited = count;
    st.levels = level_end.size();
    // the events into the caller's buffers
    if (count && (nodes || preds || dists)) {
        const size_t k = std::min<uint64_t>(capacity, count);
        if (nodes)
            VC(v, cudaMemcpyAsync(nodes, v->d_queue + q0, k * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        if (preds)
            VC(v, cudaMemcpyAsync(preds, v->d_pred + q0, k * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        VC(v, cudaStreamSynchronize(s), "cudaStreamSynchronize");
        if (dists) {
            uint64_t lvl = 0;
            for (uint64_t i = 0; i < k; i++) {
                while (lvl < level_end.size() && q0 + i >= level_end[lvl]) lvl++;
                dists[i] = (uint32_t)lvl;
            }
        }
    }
    if (stats) *stats = st;
    if (capacity < count)
        return visit_err(v, HB_ERR_INVALID, "capacity holds fewer than the " + std::to_string(count) +
                                                " events of the visit (the first ones were written)");
    return HB_OK;
}

int hb_visit_each(hb_visit* v, const uint64_t* roots, size_t nroots, uint32_t* dist, uint32_t* pred,
                  size_t len) {
    if (!v) return visit_err(nullptr, HB_ERR_INVALID, "visit is NULL");
    if ((dist && len != v->n) || (pred && len != v->n))
        return visit_err(v, HB_ERR_INVALID, "dist and pred must hold num_nodes entries");
    std::vector<uint32_t> nodes(v->n), preds(pred ? v->n : 0), ds(v->n);
    const uint64_t words = (v->n + 31) / 32;
    if (words) {
        VC(v, cudaSetDevice(v->device), "cudaSetDevice");
        VC(v, cudaMemcpyAsync(v->host_visited.data(), v->d_visited, words * 4, cudaMemcpyDeviceToHost,
                              v->stream),
           "cudaMemcpyAsync");
        VC(v, cudaStreamSynchronize(v->stream), "cudaStreamSynchronize");
    }
    for (size_t i = 0; i < nroots; i++) {
        const uint64_t r = roots[i];
        if (r >= v->n) return visit_err(v, HB_ERR_INVALID, "root " + std::to_string(r) + " >= num_nodes");
        if ((v->host_visited[r >> 5] >> (r & 31)) & 1) continue;  // seq.rs:130: already visited
        hb_visit_stats st{};
        int rc = hb_visit_run(v, &r, 1, UINT64_MAX, nodes.data(), pred ? preds.data() : nullptr, ds.data(),
                              v->n, &st);
        if (rc) return rc;
        for (uint64_t k = 0; k < st.visited; k++) {
            if (dist) dist[nodes[k]] = ds[k];
            if (pred) pred[nodes[k]] = preds[k];
            v->host_visited[nodes[k] >> 5] |= 1u << (nodes[k] & 31);
        }
    }
    return HB_OK;
}

const char* hb_visit_last_error(const hb_visit* v) { return v ? v->err.c_str() : t_visit_err.c_str(); }

}  // extern "C"
