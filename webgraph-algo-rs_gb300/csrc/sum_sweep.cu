// ExactSumSweep on the device: the GB300 counterpart of the reference's
// ExactSumSweep (src/algo/exact_sum_sweep/computer.rs, scc_graph.rs,
// output_level.rs; Borassi et al., "Fast diameter and radius BFS-based
// computation in (weakly connected) real-world graphs", TCS 586, 2015).
//
// The work of the algorithm is its breadth-first visits (forward on the
// graph, backward on the transpose) and, after each, an update of per-node
// bounds; between visits it picks the next start node with a filtered
// argmax / argmin over all nodes. All of that runs on the device:
//   k_sw_expand / k_sw_heavy  level-synchronous visit: one warp per frontier
//                             node (a block for nodes above SW_HEAVY arcs);
//                             a successor is claimed by an atomicCAS on its
//                             distance word and appended to the next level
//                             through a per-warp run in shared memory (one
//                             atomicAdd per run of up to 128 nodes); an optional
//                             component array keeps a visit inside each
//                             start node's strongly connected component
//                             (computer.rs:745-800: all pivots at once);
//   k_sw_fwd_update, k_sw_bwd_update
//                             the per-node bound updates of a forward /
//                             backward visit (computer.rs:572-693) over the
//                             visited nodes; a new minimal radius is an
//                             atomicMin of (eccentricity << 32 | node);
//   k_sw_select               filtered argmax / argmin per block, with the
//                             reference's tie rules (larger / smaller value,
//                             then tie value, then smaller node), finished on
//                             the host over the block results;
//   k_sw_missing              the five counts of find_missing_nodes;
//   k_sw_pivot_*              the best pivot of every component
//                             (computer.rs:418-475) by three atomicMin passes;
//   k_sw_refine               the node pass of all_cc_upper_bound.
// The strongly connected component of the largest out-degree node comes from
// two device visits (one for a symmetric graph); the host runs Tarjan's
// algorithm (sccs/tarjan.rs) or the symmetric labelling (sccs/symm_seq.rs) on
// the nodes outside it (see directed_components, symmetric_components), and
// finds the arcs between components (scc_graph.rs) and the two passes over
// the component DAG of all_cc_upper_bound (computer.rs:829-873), which touch
// one value per component and per DAG arc.
//
// Where the reference's parallel visits leave a choice open (which of the
// nodes reaching a new minimal radius in one step becomes the radial vertex)
// this takes the smallest node; everything else follows the reference's
// sequence of steps exactly, so the iteration counts match too.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "hb_internal.h"

namespace hbs {

constexpr uint32_t INF = 0xffffffffu;
constexpr uint32_t SW_HEAVY = 4096;
constexpr int SW_THREADS = 256;

__device__ __forceinline__ bool sw_claim(uint32_t* dist, uint32_t s, uint32_t d) {
    if (*(volatile uint32_t*)(dist + s) != INF) return false;
    return atomicCAS(dist + s, INF, d) == INF;
}

__device__ __forceinline__ void sw_append(bool c, uint32_t s, uint32_t* queue, unsigned long long* tail) {
    const unsigned mask = __ballot_sync(0xffffffffu, c);
    if (!mask) return;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == __ffs(mask) - 1) base = atomicAdd(tail, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
    if (c) queue[base + __popc(mask & ((1u << lane) - 1u))] = s;
}

// A warp's claimed nodes wait in shared memory and go to the queue in runs
// of up to SW_RUN slots, one atomicAdd on the tail per run: on a level of
// many small-degree nodes a per-chunk append puts one same-address atomic
// in the chain of almost every frontier node.
constexpr int SW_RUN = 128;

// adds the lanes' claimed nodes to the warp's run, writing the run out when
// another chunk might not fit (every lane of the warp calls it)
__device__ __forceinline__ void sw_stage(bool c, uint32_t s, uint32_t* run, int& fill, uint32_t* queue,
                                         unsigned long long* tail) {
    const unsigned mask = __ballot_sync(0xffffffffu, c);
    const int lane = threadIdx.x & 31;
    if (c) run[fill + __popc(mask & ((1u << lane) - 1u))] = s;
    fill += __popc(mask);
    if (fill > SW_RUN - 32) {
        __syncwarp();
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(tail, (unsigned long long)fill);
        base = __shfl_sync(0xffffffffu, base, 0);
        for (int k = lane; k < fill; k += 32) queue[base + k] = run[k];
        __syncwarp();
        fill = 0;
    }
}

// writes out what is left of the warp's run
__device__ __forceinline__ void sw_flush(const uint32_t* run, int fill, uint32_t* queue, unsigned long long* tail) {
    if (fill == 0) return;
    __syncwarp();
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(tail, (unsigned long long)fill);
    base = __shfl_sync(0xffffffffu, base, 0);
    for (int k = lane; k < fill; k += 32) queue[base + k] = run[k];
}

// The level state of a visit in device memory, so that the host enqueues
// several levels before it looks: queue slots [b, e) are the frontier (at
// distance d - 1), d the distance its successors get, last the largest
// distance that reached a node.
struct Level {
    unsigned long long b, e, d, last;
};

// level [b, e) of the queue (distance d - 1) -> distance d, appended at *tail
__global__ void k_sw_expand(const uint64_t* __restrict__ off, const uint32_t* __restrict__ succ,
                            const uint32_t* __restrict__ comp, uint32_t* dist, uint32_t* queue,
                            const Level* lev, unsigned long long* tail, uint32_t* heavy,
                            unsigned long long* heavy_n) {
    __shared__ uint32_t runs[SW_THREADS / 32][SW_RUN];
    uint32_t* run = runs[threadIdx.x >> 5];
    int fill = 0;  // the same in every lane of the warp
    const uint64_t b = lev->b, e = lev->e;
    const uint32_t d = (uint32_t)lev->d;
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = b + warp; i < e; i += warps) {
        const uint32_t v = queue[i];
        const uint64_t s0 = off[v], s1 = off[v + 1];
        if (s1 - s0 > SW_HEAVY) {
            if (lane == 0) heavy[atomicAdd(heavy_n, 1ull)] = v;
            continue;
        }
        const uint32_t cv = comp ? comp[v] : 0u;
        for (uint64_t a = s0; a < s1; a += 32) {
            const uint64_t x = a + lane;
            uint32_t s = 0;
            bool c = false;
            if (x < s1) {
                s = __ldg(succ + x);
                c = (!comp || __ldg(comp + s) == cv) && sw_claim(dist, s, d);
            }
            sw_stage(c, s, run, fill, queue, tail);
        }
    }
    sw_flush(run, fill, queue, tail);
}

// the deferred nodes of a level, one block each
__global__ void k_sw_heavy(const uint64_t* __restrict__ off, const uint32_t* __restrict__ succ,
                           const uint32_t* __restrict__ comp, uint32_t* dist, uint32_t* queue, const Level* lev,
                           unsigned long long* tail, const uint32_t* heavy, const unsigned long long* heavy_n) {
    const uint64_t count = *heavy_n;
    const uint32_t d = (uint32_t)lev->d;
    for (uint64_t h = blockIdx.x; h < count; h += gridDim.x) {
        const uint32_t v = heavy[h];
        const uint64_t s0 = off[v], s1 = off[v + 1];
        const uint32_t cv = comp ? comp[v] : 0u;
        for (uint64_t a = s0; a < s1; a += blockDim.x) {
            const uint64_t x = a + threadIdx.x;
            uint32_t s = 0;
            bool c = false;
            if (x < s1) {
                s = __ldg(succ + x);
                c = (!comp || __ldg(comp + s) == cv) && sw_claim(dist, s, d);
            }
            sw_append(c, s, queue, tail);
        }
    }
}

// the next level: the nodes just appended become the frontier
__global__ void k_sw_advance(Level* lev, const unsigned long long* tail, unsigned long long* heavy_n) {
    const unsigned long long t = *tail;
    if (t > lev->e) lev->last = lev->d;
    lev->b = lev->e;
    lev->e = t;
    lev->d++;
    *heavy_n = 0;
}

// the start nodes of a visit at distance 0 (each start is distinct)
__global__ void k_sw_roots(const uint32_t* __restrict__ roots, uint64_t count, uint32_t* dist, uint32_t* queue) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r = roots[i];
        dist[r] = 0;
        queue[i] = r;
    }
}

// computer.rs:652-678 (forward visit): backward totals and lower bounds
__global__ void k_sw_fwd_update(const uint32_t* __restrict__ queue, uint64_t count, const uint32_t* __restrict__ dist,
                                uint64_t* bt, uint64_t* bl, const uint64_t* __restrict__ bh) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = queue[i];
        const uint64_t d = dist[v];
        bt[v] += d;
        if (bl[v] != bh[v] && bl[v] < d) bl[v] = d;
    }
}

// computer.rs:586-626 (backward visit): forward totals and lower bounds; a
// node whose bounds meet becomes a radius candidate
__global__ void k_sw_bwd_update(const uint32_t* __restrict__ queue, uint64_t count, const uint32_t* __restrict__ dist,
                                uint64_t* ft, uint64_t* fl, const uint64_t* __restrict__ fh,
                                const uint8_t* __restrict__ radial, unsigned long long* key) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = queue[i];
        const uint64_t d = dist[v];
        ft[v] += d;
        if (fl[v] != fh[v] && fl[v] < d) {
            fl[v] = d;
            if (d == fh[v] && radial[v]) atomicMin(key, (d << 32) | v);
        }
    }
}

__global__ void k_sw_mark(const uint32_t* __restrict__ queue, uint64_t count, uint8_t* radial) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x)
        radial[queue[i]] = 1;
}

// a pivot's eccentricity inside its component: the largest distance there
__global__ void k_sw_pivot_ecc(const uint32_t* __restrict__ queue, uint64_t count, const uint32_t* __restrict__ dist,
                               const uint32_t* __restrict__ comp, unsigned long long* ecc) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = queue[i];
        atomicMax(ecc + comp[v], (unsigned long long)dist[v]);
    }
}

struct Best {
    uint64_t val, tie;
    uint64_t idx;  // ~0: none
};

// a better than b: larger (val, tie) when maximizing, smaller when
// minimizing, then the smaller node (argmax.rs, argmin.rs)
__device__ __host__ __forceinline__ bool better(const Best& a, const Best& b, bool maximize) {
    if (a.idx == ~0ull) return false;
    if (b.idx == ~0ull) return true;
    if (a.val != b.val) return maximize ? a.val > b.val : a.val < b.val;
    if (a.tie != b.tie) return maximize ? a.tie > b.tie : a.tie < b.tie;
    return a.idx < b.idx;
}

// filter: 0 fa[i] != fb[i] (bounds not met), 1 radial[i]; val == nullptr:
// the out-degree from off (the start of the SumSweep heuristic)
__global__ void k_sw_select(uint64_t n, const uint64_t* __restrict__ val, const uint64_t* __restrict__ tie,
                            const uint64_t* __restrict__ off, int maximize, int filter,
                            const uint64_t* __restrict__ fa, const uint64_t* __restrict__ fb,
                            const uint8_t* __restrict__ radial, Best* out) {
    __shared__ Best s[SW_THREADS];
    Best b{0, 0, ~0ull};
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        bool keep = true;
        if (filter == 0) keep = fa[i] != fb[i];
        else if (filter == 1) keep = radial[i] != 0;
        if (!keep) continue;
        Best c;
        c.val = val ? val[i] : off[i + 1] - off[i];
        c.tie = tie ? tie[i] : 0;
        c.idx = i;
        if (better(c, b, maximize)) b = c;
    }
    s[threadIdx.x] = b;
    __syncthreads();
    for (int w = SW_THREADS / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w && better(s[threadIdx.x + w], s[threadIdx.x], maximize))
            s[threadIdx.x] = s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = s[0];
}

// computer.rs:929-973: incomplete forward, of them above the diameter bound
// and radial below the radius bound; incomplete backward, of them above the
// diameter bound
__global__ void k_sw_missing(uint64_t n, const uint64_t* __restrict__ fl, const uint64_t* __restrict__ fh,
                             const uint64_t* __restrict__ bl, const uint64_t* __restrict__ bh,
                             const uint8_t* __restrict__ radial, uint64_t diameter_low, uint64_t radius_high,
                             unsigned long long* cnt) {
    unsigned long long r = 0, df = 0, db = 0, af = 0, ab = 0;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        if (fl[v] != fh[v]) {
            af++;
            if (fh[v] > diameter_low) df++;
            if (radial[v] && fl[v] < radius_high) r++;
        }
        if (bl[v] != bh[v]) {
            ab++;
            if (bh[v] > diameter_low) db++;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_xor_sync(0xffffffffu, r, o);
        df += __shfl_xor_sync(0xffffffffu, df, o);
        db += __shfl_xor_sync(0xffffffffu, db, o);
        af += __shfl_xor_sync(0xffffffffu, af, o);
        ab += __shfl_xor_sync(0xffffffffu, ab, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (r) atomicAdd(cnt + 0, r);
        if (df) atomicAdd(cnt + 1, df);
        if (db) atomicAdd(cnt + 2, db);
        if (af) atomicAdd(cnt + 3, af);
        if (ab) atomicAdd(cnt + 4, ab);
    }
}

// computer.rs:424-466: per component the node of the smallest
// (bl + fl + n [forward bounds met] + n [backward bounds met], ft + bt, node)
__device__ __forceinline__ uint64_t pivot_score(uint64_t v, uint64_t n, const uint64_t* fl, const uint64_t* fh,
                                                const uint64_t* bl, const uint64_t* bh) {
    return bl[v] + fl[v] + (fl[v] != fh[v] ? 0 : n) + (bl[v] != bh[v] ? 0 : n);
}
__global__ void k_sw_pivot_pass(int pass, uint64_t n, const uint32_t* __restrict__ comp,
                                const uint64_t* __restrict__ fl, const uint64_t* __restrict__ fh,
                                const uint64_t* __restrict__ bl, const uint64_t* __restrict__ bh,
                                const uint64_t* __restrict__ ft, const uint64_t* __restrict__ bt,
                                unsigned long long* best_score, unsigned long long* best_tot, uint32_t* pivot) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = comp[v];
        const uint64_t sc = pivot_score(v, n, fl, fh, bl, bh);
        if (pass == 0) {
            atomicMin(best_score + c, (unsigned long long)sc);
            continue;
        }
        if (sc != best_score[c]) continue;
        const uint64_t tot = ft[v] + bt[v];
        if (pass == 1) atomicMin(best_tot + c, (unsigned long long)tot);
        else if (tot == best_tot[c]) atomicMin(pivot + c, (uint32_t)v);
    }
}

// gathers: out[k] = src[idx[k]]
__global__ void k_sw_gather(const uint32_t* __restrict__ idx, uint64_t count, const uint32_t* __restrict__ src,
                            uint32_t* out) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (uint64_t)gridDim.x * blockDim.x)
        out[k] = src[idx[k]];
}
__global__ void k_sw_gather64(const uint32_t* __restrict__ idx, uint64_t count, const uint64_t* __restrict__ src,
                              uint64_t* out) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (uint64_t)gridDim.x * blockDim.x)
        out[k] = src[idx[k]];
}

// computer.rs:879-915: the node pass of all_cc_upper_bound
__global__ void k_sw_refine(uint64_t n, const uint32_t* __restrict__ comp, const uint32_t* __restrict__ df,
                            const uint32_t* __restrict__ db, const uint64_t* __restrict__ ef,
                            const uint64_t* __restrict__ eb, const uint64_t* __restrict__ fl, uint64_t* fh,
                            uint64_t* bh, const uint8_t* __restrict__ radial, unsigned long long* key) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = comp[v];
        uint64_t h = fh[v];
        const uint64_t pv = (uint64_t)db[v] + ef[c];
        if (pv < h) {
            fh[v] = pv;
            h = pv;
        }
        if (h == fl[v] && radial[v]) atomicMin(key, (h << 32) | v);
        const uint64_t pb = (uint64_t)df[v] + eb[c];
        if (pb < bh[v]) bh[v] = pb;
    }
}

// a[i] = b[i] = value (the start node's bounds after its own visit)
__global__ void k_sw_set2(uint64_t* a, uint64_t* b, uint64_t i, uint64_t value) {
    a[i] = value;
    b[i] = value;
}

__global__ void k_sw_fill64(uint64_t* p, uint64_t count, uint64_t value) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = value;
}

__global__ void k_sw_validate(const uint64_t* __restrict__ off, const uint32_t* __restrict__ succ, uint64_t n,
                              uint64_t m, int* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint64_t v = t0; v < n; v += stride)
        if (off[v] > off[v + 1]) *bad = 1;
    for (uint64_t x = t0; x < m; x += stride)
        if (succ[x] >= n) *bad = 1;
}

}  // namespace hbs

namespace {

using u64 = uint64_t;
constexpr u64 NONE = ~0ull;

thread_local std::string t_sweep_err;

struct SweepError {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg) { throw SweepError{code, msg}; }

void ck(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    cudaGetLastError();
    const int code = e == cudaErrorMemoryAllocation ? HB_ERR_OOM : HB_ERR_CUDA;
    fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

struct HostCsr {
    u64 n;
    const u64* off;
    const uint32_t* succ;
    u64 deg(u64 v) const { return off[v + 1] - off[v]; }
};

// sccs/tarjan.rs: components numbered as they are emitted (reverse
// topological order), roots in node order, successors in arc order
// With `group` given, only the nodes v with group[v] == want and the arcs
// between them take part (the other entries of comp are left as they are),
// and the components are numbered from ncomp on.
void tarjan_into(const HostCsr& g, std::vector<uint32_t>& comp, u64& ncomp, const uint8_t* group = nullptr,
                 uint8_t want = 0) {
    const u64 n = g.n;
    auto in = [&](u64 v) { return !group || group[v] == want; };
    std::vector<uint32_t> index(n, 0xffffffffu), low(n, 0);
    std::vector<uint8_t> on_stack(n, 0);
    std::vector<uint32_t> stack;
    std::vector<std::pair<uint32_t, u64>> call;
    uint32_t counter = 0;
    for (u64 r = 0; r < n; r++) {
        if (index[r] != 0xffffffffu || !in(r)) continue;
        index[r] = low[r] = counter++;
        stack.push_back((uint32_t)r);
        on_stack[r] = 1;
        call.push_back({(uint32_t)r, g.off[r]});
        while (!call.empty()) {
            const uint32_t v = call.back().first;
            u64& e = call.back().second;
            if (e < g.off[v + 1]) {
                const uint32_t w = g.succ[e++];
                if (!in(w)) continue;
                if (index[w] == 0xffffffffu) {
                    index[w] = low[w] = counter++;
                    stack.push_back(w);
                    on_stack[w] = 1;
                    call.push_back({w, g.off[w]});
                } else if (on_stack[w] && index[w] < low[v]) {
                    low[v] = index[w];
                }
                continue;
            }
            if (low[v] == index[v]) {
                for (;;) {
                    const uint32_t w = stack.back();
                    stack.pop_back();
                    on_stack[w] = 0;
                    comp[w] = (uint32_t)ncomp;
                    if (w == v) break;
                }
                ncomp++;
            }
            call.pop_back();
            if (!call.empty() && low[v] < low[call.back().first]) low[call.back().first] = low[v];
        }
    }
}

std::vector<uint32_t> tarjan(const HostCsr& g, u64& ncomp) {
    std::vector<uint32_t> comp(g.n, 0);
    ncomp = 0;
    tarjan_into(g, comp, ncomp);
    return comp;
}

// sccs/symm_seq.rs: components of a symmetric graph in order of their
// smallest node (nodes already labelled are skipped, the others numbered
// from ncomp on)
void symm_into(const HostCsr& g, std::vector<uint32_t>& comp, u64& ncomp) {
    std::vector<uint32_t> st;
    for (u64 r = 0; r < g.n; r++) {
        if (comp[r] != 0xffffffffu) continue;
        comp[r] = (uint32_t)ncomp;
        st.push_back((uint32_t)r);
        while (!st.empty()) {
            const uint32_t v = st.back();
            st.pop_back();
            for (u64 e = g.off[v]; e < g.off[v + 1]; e++)
                if (comp[g.succ[e]] == 0xffffffffu) {
                    comp[g.succ[e]] = (uint32_t)ncomp;
                    st.push_back(g.succ[e]);
                }
        }
        ncomp++;
    }
}

std::vector<uint32_t> symm_components(const HostCsr& g, u64& ncomp) {
    std::vector<uint32_t> comp(g.n, 0xffffffffu);
    ncomp = 0;
    symm_into(g, comp, ncomp);
    return comp;
}

struct Sweeper {
    int device = 0;
    cudaStream_t s = nullptr;
    bool own_stream = false;
    u64 n = 0, m = 0;
    bool undirected = false;
    int level = 0;
    int sms = 1;
    // device state
    u64 *d_off = nullptr, *d_toff = nullptr;
    uint32_t *d_succ = nullptr, *d_tsucc = nullptr;
    uint32_t *d_dist = nullptr, *d_queue = nullptr, *d_heavy = nullptr, *d_comp = nullptr;
    uint32_t *d_roots = nullptr, *d_df = nullptr, *d_db = nullptr;
    u64 *d_fl = nullptr, *d_fh = nullptr, *d_bl = nullptr, *d_bh = nullptr, *d_ft = nullptr, *d_bt = nullptr;
    uint8_t* d_radial = nullptr;
    unsigned long long* d_cnt = nullptr;  // [2] radius key [3..7] missing counts
    hbs::Level* d_lev = nullptr;          // a visit's level, then its tail and deferred-node count
    unsigned long long *d_ecc_f = nullptr, *d_ecc_b = nullptr, *d_best_score = nullptr, *d_best_tot = nullptr;
    uint32_t* d_pivot = nullptr;
    u64 *d_ef = nullptr, *d_eb = nullptr;
    uint32_t *d_cstart = nullptr, *d_cend = nullptr, *d_gather = nullptr;
    u64* d_gather64 = nullptr;
    hbs::Best* d_best = nullptr;
    unsigned long long* h_cnt = nullptr;  // page-locked: [0, 6) a visit's level, 6 root, 7 key, [8, 13) counts
    hbs::Best* h_best = nullptr;          // page-locked copy of the selection's block results
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    static constexpr int LEVELS_AHEAD = 8;
    cudaGraphExec_t group_graph[2][2] = {};  // [backward][inside components]: LEVELS_AHEAD levels
    cudaStream_t cap = nullptr;              // capture stream of the groups
    float device_ms = 0.f;
    u64 sweeps = 0;
    // host state (computer.rs:38-89)
    std::vector<uint32_t> comp;
    u64 ncomp = 0;
    std::vector<u64> seg;
    std::vector<uint32_t> cstart, cend, ctarget;
    u64 diameter_low = 0, radius_high = NONE, diameter_vertex = 0, radius_vertex = 0, iterations = 0;
    u64 radius_it = NONE, diameter_it = NONE, forward_it = NONE, all_it = NONE;
    bool compute_radial = true;
    std::vector<uint8_t> radial_host;  // the radial vertices (read on the host by forward steps)
    int grid = 1;

    ~Sweeper() {
        cudaSetDevice(device);
        if (s) cudaStreamSynchronize(s);
        // a symmetric graph is its own transpose: each block once
        std::vector<void*> ps = {d_off, d_toff, d_succ, d_tsucc, d_dist, d_queue, d_heavy, d_comp,
                                 d_roots, d_df, d_db, d_fl, d_fh, d_bl, d_bh, d_ft, d_bt, d_radial,
                                 d_cnt, d_lev, d_ecc_f, d_ecc_b, d_best_score, d_best_tot, d_pivot, d_ef,
                                 d_eb, d_cstart, d_cend, d_gather, d_gather64, d_best};
        std::sort(ps.begin(), ps.end());
        ps.erase(std::unique(ps.begin(), ps.end()), ps.end());
        for (void* p : ps)
            if (p) cudaFree(p);
        if (h_cnt) cudaFreeHost(h_cnt);
        if (h_best) cudaFreeHost(h_best);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        for (auto& row : group_graph)
            for (cudaGraphExec_t g : row)
                if (g) cudaGraphExecDestroy(g);
        if (cap) cudaStreamDestroy(cap);
        if (own_stream && s) cudaStreamDestroy(s);
    }

    template <class T>
    void alloc(T** p, u64 count) {
        ck(cudaMalloc((void**)p, std::max<u64>(count, 1) * sizeof(T)), "cudaMalloc");
    }
    int blocks(u64 work) const { return (int)std::min<u64>((work + hbs::SW_THREADS - 1) / hbs::SW_THREADS + 1, (u64)grid); }
    void sync() { ck(cudaStreamSynchronize(s), "cudaStreamSynchronize"); }

    // One visit from the `count` start nodes in d_roots on the graph or its
    // transpose (inside components when `in_comp`); returns the number of
    // visited nodes (d_queue[0, visited), distances in d_dist) and the
    // largest distance in *ecc. Levels are enqueued LEVELS_AHEAD at a time
    // with their bounds in device memory (a level past the last is empty);
    // the host looks only between groups. A group is one CUDA graph per kind
    // of visit (forward or backward, inside components or not), captured
    // the first time on a private stream and launched on the call's stream.
    u64 visit(u64 count, bool backward, bool in_comp, u64* ecc) {
        const u64* off = backward ? d_toff : d_off;
        const uint32_t* succ = backward ? d_tsucc : d_succ;
        const uint32_t* cp = in_comp ? d_comp : nullptr;
        ck(cudaMemsetAsync(d_dist, 0xff, n * 4, s), "cudaMemsetAsync");
        hbs::k_sw_roots<<<blocks(count), hbs::SW_THREADS, 0, s>>>(d_roots, count, d_dist, d_queue);
        ck(cudaGetLastError(), "k_sw_roots");
        hbs::Level* h = reinterpret_cast<hbs::Level*>(h_cnt);
        *h = hbs::Level{0, count, 1, 0};
        h_cnt[4] = count;  // tail
        h_cnt[5] = 0;      // deferred nodes
        ck(cudaMemcpyAsync(d_lev, h_cnt, 6 * 8, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        unsigned long long* tail = reinterpret_cast<unsigned long long*>(d_lev) + 4;
        unsigned long long* heavy_n = tail + 1;
        auto enqueue = [&](cudaStream_t x) {
            for (int k = 0; k < LEVELS_AHEAD; k++) {
                hbs::k_sw_expand<<<grid, hbs::SW_THREADS, 0, x>>>(off, succ, cp, d_dist, d_queue, d_lev, tail,
                                                                 d_heavy, heavy_n);
                hbs::k_sw_heavy<<<sms * 4, hbs::SW_THREADS, 0, x>>>(off, succ, cp, d_dist, d_queue, d_lev, tail,
                                                                  d_heavy, heavy_n);
                hbs::k_sw_advance<<<1, 1, 0, x>>>(d_lev, tail, heavy_n);
            }
        };
        cudaGraphExec_t& ge = group_graph[backward ? 1 : 0][in_comp ? 1 : 0];
        if (!ge) {
            if (!cap) ck(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "cudaStreamCreate");
            ck(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
            enqueue(cap);
            cudaGraph_t graph = nullptr;
            const cudaError_t e = cudaStreamEndCapture(cap, &graph);
            if (e == cudaSuccess) ck(cudaGraphInstantiate(&ge, graph, 0), "cudaGraphInstantiate");
            if (graph) cudaGraphDestroy(graph);
            ck(e, "cudaStreamEndCapture");
        }
        for (;;) {
            ck(cudaGraphLaunch(ge, s), "cudaGraphLaunch");
            ck(cudaMemcpyAsync(h_cnt, d_lev, 6 * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
            sync();
            if (h->b == h->e) break;
        }
        if (ecc) *ecc = h->last;
        return h_cnt[4];
    }

    // small transfers go through page-locked words (a pageable copy would
    // wait for the stream each time): h_cnt[6] the start node, h_cnt[7]
    // the radius key
    void set_root(u64 r) {
        reinterpret_cast<uint32_t*>(h_cnt + 6)[0] = (uint32_t)r;
        ck(cudaMemcpyAsync(d_roots, h_cnt + 6, 4, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    }

    unsigned long long read_key() {
        ck(cudaMemcpyAsync(h_cnt + 7, d_cnt + 2, 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        sync();
        return h_cnt[7];
    }
    void reset_key() { ck(cudaMemsetAsync(d_cnt + 2, 0xff, 8, s), "cudaMemsetAsync"); }

    // argmax / argmin over nodes (filter 0: bounds fa, fb not met; 1 radial)
    u64 select(const u64* val, const u64* tie, bool maximize, int filter, const u64* fa, const u64* fb) {
        const int g = blocks(n);
        hbs::k_sw_select<<<g, hbs::SW_THREADS, 0, s>>>(n, val, tie, d_off, maximize ? 1 : 0, filter, fa, fb,
                                                       d_radial, d_best);
        ck(cudaGetLastError(), "k_sw_select");
        ck(cudaMemcpyAsync(h_best, d_best, g * sizeof(hbs::Best), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        sync();
        hbs::Best b{0, 0, NONE};
        for (int k = 0; k < g; k++)
            if (hbs::better(h_best[k], b, maximize)) b = h_best[k];
        return b.idx;
    }

    // The strongly connected components of a directed graph, numbered in a
    // reverse topological order (sccs/tarjan.rs numbers them as Tarjan's
    // algorithm emits them). The component of the largest out-degree node
    // is found on the device, as the nodes that both reach it and are reached
    // from it (two visits). The other nodes are split into those reached from it
    // (their components can only lead to components reached from it) and the
    // rest (whose components can lead to everything). Tarjan's algorithm runs
    // on each part alone, on the host, the first part numbered first, then the
    // pivot's component, then the rest: every arc between components goes
    // from a higher number to a lower one, as in Tarjan's numbering. The
    // numbering of the reference matters only when two components share the
    // largest size (computer.rs:498-506 takes the first); then the whole
    // graph goes through Tarjan's algorithm in node order instead.
    std::vector<uint32_t> directed_components(const HostCsr& hg) {
        const u64 p = select(nullptr, nullptr, true, 2, nullptr, nullptr);
        std::vector<uint32_t> fw(n), bw(n);
        set_root(p);
        visit(1, false, false, nullptr);
        ck(cudaMemcpyAsync(fw.data(), d_dist, n * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        set_root(p);
        visit(1, true, false, nullptr);
        ck(cudaMemcpyAsync(bw.data(), d_dist, n * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        sync();
        // group 0: reached from p only; 1: the component of p; 2: the rest
        std::vector<uint8_t> group(n);
        for (u64 v = 0; v < n; v++) {
            const bool f = fw[v] != hbs::INF, b = bw[v] != hbs::INF;
            group[v] = f && b ? 1 : f ? 0 : 2;
        }
        std::vector<uint32_t> comp(n, 0);
        u64 nc = 0;
        tarjan_into(hg, comp, nc, group.data(), 0);
        const uint32_t pc = (uint32_t)nc++;
        for (u64 v = 0; v < n; v++)
            if (group[v] == 1) comp[v] = pc;
        tarjan_into(hg, comp, nc, group.data(), 2);
        std::vector<u64> sizes(nc, 0);
        for (u64 v = 0; v < n; v++) sizes[comp[v]]++;
        const u64 big = *std::max_element(sizes.begin(), sizes.end());
        if (std::count(sizes.begin(), sizes.end(), big) > 1) return tarjan(hg, ncomp);
        ncomp = nc;
        return comp;
    }

    // The components of a symmetric graph: the one of the largest-degree
    // node from one device visit, the others on the host (symm_seq.rs). The
    // numbering (symm_seq.rs numbers by smallest node) matters only when two
    // components share the largest size; then all of them come from the host
    // in the reference's order.
    std::vector<uint32_t> symmetric_components(const HostCsr& hg) {
        const u64 p = select(nullptr, nullptr, true, 2, nullptr, nullptr);
        std::vector<uint32_t> d(n);
        set_root(p);
        visit(1, false, false, nullptr);
        ck(cudaMemcpyAsync(d.data(), d_dist, n * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        sync();
        std::vector<uint32_t> comp(n, 0xffffffffu);
        u64 nc = 0;
        for (u64 v = 0; v < n; v++)
            if (d[v] != hbs::INF) comp[v] = 0;
        nc = 1;
        symm_into(hg, comp, nc);
        std::vector<u64> sizes(nc, 0);
        for (u64 v = 0; v < n; v++) sizes[comp[v]]++;
        const u64 big = *std::max_element(sizes.begin(), sizes.end());
        if (std::count(sizes.begin(), sizes.end(), big) > 1) return symm_components(hg, ncomp);
        ncomp = nc;
        return comp;
    }

    // computer.rs:487-542
    void compute_radial_vertices() {
        std::vector<u64> sizes(ncomp, 0);
        for (u64 v = 0; v < n; v++) sizes[comp[v]]++;
        u64 big = 0;
        for (u64 c = 1; c < ncomp; c++)
            if (sizes[c] > sizes[big]) big = c;
        u64 v = n;
        while (v > 0) {
            v--;
            if (comp[v] == big) break;
        }
        set_root(v);
        const u64 cnt = visit(1, true, false, nullptr);
        hbs::k_sw_mark<<<blocks(cnt), hbs::SW_THREADS, 0, s>>>(d_queue, cnt, d_radial);
        ck(cudaGetLastError(), "k_sw_mark");
        sweeps++;
    }

    // computer.rs:644-693
    void forward_step(u64 start) {
        set_root(start);
        u64 ecc = 0;
        const u64 cnt = visit(1, false, false, &ecc);
        sweeps++;
        hbs::k_sw_fwd_update<<<blocks(cnt), hbs::SW_THREADS, 0, s>>>(d_queue, cnt, d_dist, d_bt, d_bl, d_bh);
        hbs::k_sw_set2<<<1, 1, 0, s>>>(d_fl, d_fh, start, ecc);
        ck(cudaGetLastError(), "k_sw_fwd_update");
        const bool rad = radial_host[start] != 0;
        if (diameter_low < ecc) {
            diameter_low = ecc;
            diameter_vertex = start;
        }
        if (rad && radius_high > ecc) {
            radius_high = ecc;
            radius_vertex = start;
        }
    }

    // computer.rs:572-642
    void backward_step(u64 start) {
        set_root(start);
        u64 ecc = 0;
        const u64 cnt = visit(1, true, false, &ecc);
        sweeps++;
        reset_key();
        hbs::k_sw_bwd_update<<<blocks(cnt), hbs::SW_THREADS, 0, s>>>(d_queue, cnt, d_dist, d_ft, d_fl, d_fh,
                                                                    d_radial, d_cnt + 2);
        hbs::k_sw_set2<<<1, 1, 0, s>>>(d_bl, d_bh, start, ecc);
        ck(cudaGetLastError(), "k_sw_bwd_update");
        const unsigned long long key = read_key();
        if (key != ~0ull && (key >> 32) < radius_high) {
            radius_high = key >> 32;
            radius_vertex = key & 0xffffffffull;
        }
        if (diameter_low < ecc) {
            diameter_low = ecc;
            diameter_vertex = start;
        }
    }

    // computer.rs:554-570
    void step(u64 start, bool forward) {
        if (start == NONE) return;
        if (forward) forward_step(start);
        else backward_step(start);
        iterations++;
    }

    // computer.rs:818-921
    void all_cc_upper_bound() {
        const u64 nc = ncomp;
        ck(cudaMemsetAsync(d_best_score, 0xff, nc * 8, s), "cudaMemsetAsync");
        ck(cudaMemsetAsync(d_best_tot, 0xff, nc * 8, s), "cudaMemsetAsync");
        ck(cudaMemsetAsync(d_pivot, 0xff, nc * 4, s), "cudaMemsetAsync");
        for (int pass = 0; pass < 3; pass++) {
            hbs::k_sw_pivot_pass<<<blocks(n), hbs::SW_THREADS, 0, s>>>(pass, n, d_comp, d_fl, d_fh, d_bl, d_bh, d_ft,
                                                                      d_bt, d_best_score, d_best_tot, d_pivot);
            ck(cudaGetLastError(), "k_sw_pivot_pass");
        }
        // distances from the pivots inside each component, both directions
        ck(cudaMemcpyAsync(d_roots, d_pivot, nc * 4, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
        u64 cnt = visit(nc, false, true, nullptr);
        ck(cudaMemsetAsync(d_ecc_f, 0, nc * 8, s), "cudaMemsetAsync");
        hbs::k_sw_pivot_ecc<<<blocks(cnt), hbs::SW_THREADS, 0, s>>>(d_queue, cnt, d_dist, d_comp, d_ecc_f);
        ck(cudaGetLastError(), "k_sw_pivot_ecc");
        ck(cudaMemcpyAsync(d_df, d_dist, n * 4, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
        ck(cudaMemcpyAsync(d_roots, d_pivot, nc * 4, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
        cnt = visit(nc, true, true, nullptr);
        ck(cudaMemsetAsync(d_ecc_b, 0, nc * 8, s), "cudaMemsetAsync");
        hbs::k_sw_pivot_ecc<<<blocks(cnt), hbs::SW_THREADS, 0, s>>>(d_queue, cnt, d_dist, d_comp, d_ecc_b);
        ck(cudaGetLastError(), "k_sw_pivot_ecc");
        ck(cudaMemcpyAsync(d_db, d_dist, n * 4, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
        sweeps += 2;
        // what the passes over the component DAG read, to the host
        const u64 nconn = ctarget.size();
        std::vector<u64> ef(nc), eb(nc), fhp(nc), bhp(nc);
        std::vector<uint32_t> dfs(nconn), dbe(nconn);
        ck(cudaMemcpyAsync(ef.data(), d_ecc_f, nc * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        ck(cudaMemcpyAsync(eb.data(), d_ecc_b, nc * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        hbs::k_sw_gather64<<<blocks(nc), hbs::SW_THREADS, 0, s>>>(d_pivot, nc, d_fh, d_gather64);
        ck(cudaMemcpyAsync(fhp.data(), d_gather64, nc * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        hbs::k_sw_gather64<<<blocks(nc), hbs::SW_THREADS, 0, s>>>(d_pivot, nc, d_bh, d_gather64);
        ck(cudaMemcpyAsync(bhp.data(), d_gather64, nc * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        if (nconn) {
            hbs::k_sw_gather<<<blocks(nconn), hbs::SW_THREADS, 0, s>>>(d_cstart, nconn, d_df, d_gather);
            ck(cudaMemcpyAsync(dfs.data(), d_gather, nconn * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
            sync();
            hbs::k_sw_gather<<<blocks(nconn), hbs::SW_THREADS, 0, s>>>(d_cend, nconn, d_db, d_gather);
            ck(cudaMemcpyAsync(dbe.data(), d_gather, nconn * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        }
        ck(cudaGetLastError(), "k_sw_gather");
        sync();
        // computer.rs:829-873: forward bounds in component order (children
        // first), backward bounds in reverse order (parents first)
        for (u64 c = 0; c < nc; c++) {
            const u64 e1 = c + 1 < nc ? seg[c + 1] : nconn;
            for (u64 k = seg[c]; k < e1; k++) {
                ef[c] = std::max(ef[c], (u64)dfs[k] + 1 + dbe[k] + ef[ctarget[k]]);
                if (ef[c] >= fhp[c]) {
                    ef[c] = fhp[c];
                    break;
                }
            }
        }
        for (u64 c = nc; c-- > 0;) {
            const u64 e1 = c + 1 < nc ? seg[c + 1] : nconn;
            for (u64 k = seg[c]; k < e1; k++) {
                const u64 t = ctarget[k];
                eb[t] = std::max(eb[t], (u64)dfs[k] + 1 + dbe[k] + eb[c]);
                if (eb[t] >= bhp[t]) eb[t] = bhp[t];
            }
        }
        ck(cudaMemcpyAsync(d_ef, ef.data(), nc * 8, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        ck(cudaMemcpyAsync(d_eb, eb.data(), nc * 8, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        reset_key();
        hbs::k_sw_refine<<<blocks(n), hbs::SW_THREADS, 0, s>>>(n, d_comp, d_df, d_db, d_ef, d_eb, d_fl, d_fh, d_bh,
                                                              d_radial, d_cnt + 2);
        ck(cudaGetLastError(), "k_sw_refine");
        const unsigned long long key = read_key();
        if (key != ~0ull && (key >> 32) < radius_high) {
            radius_high = key >> 32;
            radius_vertex = key & 0xffffffffull;
        }
        iterations += 3;
    }

    // computer.rs:929-1015
    u64 missing() {
        ck(cudaMemsetAsync(d_cnt + 3, 0, 5 * 8, s), "cudaMemsetAsync");
        hbs::k_sw_missing<<<blocks(n), hbs::SW_THREADS, 0, s>>>(n, d_fl, d_fh, d_bl, d_bh, d_radial, diameter_low,
                                                               radius_high, d_cnt + 3);
        ck(cudaGetLastError(), "k_sw_missing");
        unsigned long long* c = h_cnt + 8;
        ck(cudaMemcpyAsync(c, d_cnt + 3, 5 * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        sync();
        const u64 mr = c[0], mdf = c[1], mdb = c[2], maf = c[3], mab = c[4];
        if (mr == 0 && radius_it == NONE) radius_it = iterations;
        if ((mdf == 0 || mdb == 0) && diameter_it == NONE) diameter_it = iterations;
        if (maf == 0 && forward_it == NONE) forward_it = iterations;
        if (maf == 0 && mab == 0) all_it = iterations;
        switch (level) {
            case HB_SWEEP_RADIUS: return mr;
            case HB_SWEEP_DIAMETER: return std::min(mdf, mdb);
            case HB_SWEEP_RADIUS_DIAMETER: return mr + std::min(mdf, mdb);
            case HB_SWEEP_ALL_FORWARD: return maf;
            default: return mab + maf;
        }
    }

    // computer.rs:282-409
    void compute() {
        if (compute_radial) compute_radial_vertices();
        radial_host.resize(n);
        ck(cudaMemcpyAsync(radial_host.data(), d_radial, n, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        sync();
        step(select(nullptr, nullptr, true, 2, nullptr, nullptr), true);
        for (int i = 2; i <= 6; i++) {
            if (i % 2 == 0)
                step(select(d_bt, d_bl, true, 0, d_bl, d_bh), false);
            else
                step(select(d_ft, d_fl, true, 0, d_fl, d_fh), true);
        }
        double points[5];
        for (double& p : points) p = (double)n;
        u64 miss = missing();
        while (miss > 0) {
            int st = 0;
            for (int i = 1; i < 5; i++)
                if (points[i] > points[st]) st = i;
            switch (st) {
                case 0: all_cc_upper_bound(); break;
                case 1: step(select(d_fh, d_ft, true, 0, d_fl, d_fh), true); break;
                case 2: step(select(d_fl, d_ft, false, 1, nullptr, nullptr), true); break;
                case 3: step(select(d_bh, d_bt, true, 0, d_bl, d_bh), false); break;
                default: step(select(d_bt, d_bh, true, 0, d_bl, d_bh), false); break;
            }
            const u64 old = miss;
            miss = missing();
            if (miss > old) fail(HB_ERR_CUDA, "ExactSumSweep: the number of missing nodes grew");
            points[st] = (double)(old - miss);
            for (int i = 0; i < 5; i++)
                if (i != st && points[i] >= 0.0) points[i] += 2.0 / (double)iterations;
        }
    }
};

int run(const hb_graph_view* g, const hb_graph_view* t, int level, const uint8_t* radial, int device,
        void* stream, uint64_t* fecc, uint64_t* becc, hb_sweep_result* out) {
    if (!g || !out) fail(HB_ERR_INVALID, "graph and out must not be NULL");
    if (level < HB_SWEEP_ALL || level > HB_SWEEP_RADIUS) fail(HB_ERR_INVALID, "level must be 0..4");
    const u64 n = g->num_nodes, m = g->num_arcs;
    if (!g->offsets || (m && !g->successors)) fail(HB_ERR_INVALID, "graph arrays must not be NULL");
    if (n >= 0xffffffffull) fail(HB_ERR_INVALID, "node ids must fit u32");
    if (g->offsets[0] != 0 || g->offsets[n] != m)
        fail(HB_ERR_INVALID, "offsets[0] must be 0 and offsets[num_nodes] must equal num_arcs");
    if (t) {
        if (t->num_nodes != n || t->num_arcs != m) fail(HB_ERR_INVALID, "the transpose must have the graph's nodes and arcs");
        if (!t->offsets || (m && !t->successors)) fail(HB_ERR_INVALID, "transpose arrays must not be NULL");
        if (t->offsets[0] != 0 || t->offsets[n] != m)
            fail(HB_ERR_INVALID, "offsets[0] must be 0 and offsets[num_nodes] must equal num_arcs");
    }
    Sweeper w;
    w.undirected = t == nullptr;
    // computer.rs:109-114: a symmetric graph has only forward eccentricities
    w.level = (w.undirected && level == HB_SWEEP_ALL) ? HB_SWEEP_ALL_FORWARD : level;
    std::memset(out, 0, sizeof *out);
    static const char* kNames[] = {"All", "AllForward", "RadiusDiameter", "Diameter", "Radius"};
    if (n == 0) {
        // output_level.rs: the output builders assert that their fields were
        // computed; the first assert of each level fails on an empty graph
        const char* what = w.level == HB_SWEEP_RADIUS           ? "the radius computed"
                           : w.level == HB_SWEEP_ALL            ? "all eccentricities computed"
                           : w.level == HB_SWEEP_ALL_FORWARD    ? "all forward eccentricities computed"
                                                                : "the diameter computed";
        fail(HB_ERR_INVALID, std::string("Trying to build ") + kNames[level] + " without " + what);
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        fail(HB_ERR_NO_DEVICE, "no CUDA device available (this library has no CPU path)");
    }
    w.device = device;
    w.n = n;
    w.m = m;
    ck(cudaSetDevice(device), "cudaSetDevice");
    if (stream) {
        w.s = (cudaStream_t)stream;
    } else {
        ck(cudaStreamCreateWithFlags(&w.s, cudaStreamNonBlocking), "cudaStreamCreate");
        w.own_stream = true;
    }
    cudaDeviceGetAttribute(&w.sms, cudaDevAttrMultiProcessorCount, device);
    w.grid = w.sms * 8;
    ck(cudaEventCreate(&w.ev0), "cudaEventCreate");
    ck(cudaEventCreate(&w.ev1), "cudaEventCreate");
    // HB_TRACE=1: the phases' host time on stderr
    const bool trace = std::getenv("HB_TRACE") != nullptr;
    auto t_mark = std::chrono::steady_clock::now();
    auto mark = [&](const char* what) {
        if (!trace) return;
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "hb_exact_sum_sweep %-22s %9.2f ms\n", what,
                     std::chrono::duration<double, std::milli>(now - t_mark).count());
        t_mark = now;
    };
    HostCsr hg{n, g->offsets, g->successors};
    HostCsr ht = t ? HostCsr{n, t->offsets, t->successors} : hg;
    // the graph on the device first: the components use its visits
    w.alloc(&w.d_off, n + 1);
    w.alloc(&w.d_succ, m);
    if (t) {
        w.alloc(&w.d_toff, n + 1);
        w.alloc(&w.d_tsucc, m);
    } else {
        w.d_toff = w.d_off;
        w.d_tsucc = w.d_succ;
    }
    for (uint32_t** p : {&w.d_dist, &w.d_queue, &w.d_heavy, &w.d_comp, &w.d_roots, &w.d_df, &w.d_db}) w.alloc(p, n);
    for (u64** p : {&w.d_fl, &w.d_fh, &w.d_bl, &w.d_bh, &w.d_ft, &w.d_bt}) w.alloc(p, n);
    w.alloc(&w.d_radial, n);
    w.alloc(&w.d_cnt, 8);
    ck(cudaMalloc((void**)&w.d_lev, 6 * 8), "cudaMalloc");
    w.alloc(&w.d_best, (u64)w.grid);
    ck(cudaMallocHost((void**)&w.h_cnt, 16 * 8), "cudaMallocHost");
    ck(cudaMallocHost((void**)&w.h_best, (size_t)w.grid * sizeof(hbs::Best)), "cudaMallocHost");
    cudaStream_t s = w.s;
    ck(cudaMemcpyAsync(w.d_off, g->offsets, (n + 1) * 8, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    if (m) ck(cudaMemcpyAsync(w.d_succ, g->successors, m * 4, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    if (t) {
        ck(cudaMemcpyAsync(w.d_toff, t->offsets, (n + 1) * 8, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        if (m) ck(cudaMemcpyAsync(w.d_tsucc, t->successors, m * 4, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    }
    // the CSR is checked before any kernel indexes with it
    {
        int bad = 0;
        int* d_bad = (int*)(w.d_cnt + 7);
        ck(cudaMemsetAsync(d_bad, 0, 4, s), "cudaMemsetAsync");
        hbs::k_sw_validate<<<w.blocks(std::max(n, m)), hbs::SW_THREADS, 0, s>>>(w.d_off, w.d_succ, n, m, d_bad);
        if (t) hbs::k_sw_validate<<<w.blocks(std::max(n, m)), hbs::SW_THREADS, 0, s>>>(w.d_toff, w.d_tsucc, n, m, d_bad);
        ck(cudaGetLastError(), "k_sw_validate");
        ck(cudaMemcpyAsync(&bad, d_bad, 4, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        w.sync();
        if (bad) fail(HB_ERR_INVALID, "graph has decreasing offsets or successors >= num_nodes");
    }
    mark("device graph");
    // components and the arcs between them
    if (w.undirected) w.comp = w.symmetric_components(hg);
    else w.comp = w.directed_components(hg);
    w.seg.assign(w.ncomp, 0);
    mark("components");
    if (!w.undirected) {
        // scc_graph.rs:118-227; the nodes of each component in increasing
        // order by a counting sort
        std::vector<u64> first(w.ncomp + 1, 0);
        for (u64 v = 0; v < n; v++) first[w.comp[v] + 1]++;
        for (u64 c = 0; c < w.ncomp; c++) first[c + 1] += first[c];
        std::vector<uint32_t> members(n);
        {
            std::vector<u64> at(first.begin(), first.end() - 1);
            for (u64 v = 0; v < n; v++) members[at[w.comp[v]]++] = (uint32_t)v;
        }
        std::vector<uint32_t> bs(w.ncomp, 0xffffffffu), be(w.ncomp, 0);
        std::vector<uint32_t> children;
        auto value = [&](u64 a, u64 b) { return ht.deg(a) + hg.deg(b); };
        for (u64 c = 0; c < w.ncomp; c++) {
            for (u64 k = first[c]; k < first[c + 1]; k++) {
                const uint32_t v = members[k];
                for (u64 e = hg.off[v]; e < hg.off[v + 1]; e++) {
                    const uint32_t x = hg.succ[e];
                    const uint32_t xc = w.comp[x];
                    if (xc == c) continue;
                    if (bs[xc] == 0xffffffffu) {
                        bs[xc] = v;
                        be[xc] = x;
                        children.push_back(xc);
                    }
                    if (value(v, x) > value(bs[xc], be[xc])) {
                        bs[xc] = v;
                        be[xc] = x;
                    }
                }
            }
            w.seg[c] = w.ctarget.size();
            for (uint32_t ch : children) {
                w.ctarget.push_back(ch);
                w.cstart.push_back(bs[ch]);
                w.cend.push_back(be[ch]);
                bs[ch] = 0xffffffffu;
            }
            children.clear();
        }
    }
    mark("component arcs");
    const u64 nc = w.ncomp, nconn = w.ctarget.size();
    w.alloc(&w.d_ecc_f, nc);
    w.alloc(&w.d_ecc_b, nc);
    w.alloc(&w.d_best_score, nc);
    w.alloc(&w.d_best_tot, nc);
    w.alloc(&w.d_pivot, nc);
    w.alloc(&w.d_ef, nc);
    w.alloc(&w.d_eb, nc);
    w.alloc(&w.d_gather64, nc);
    w.alloc(&w.d_cstart, nconn);
    w.alloc(&w.d_cend, nconn);
    w.alloc(&w.d_gather, nconn);
    ck(cudaMemcpyAsync(w.d_comp, w.comp.data(), n * 4, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    if (nconn) {
        ck(cudaMemcpyAsync(w.d_cstart, w.cstart.data(), nconn * 4, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        ck(cudaMemcpyAsync(w.d_cend, w.cend.data(), nconn * 4, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    }
    // computer.rs:213-240: lower bounds 0, upper bounds n, totals 0
    ck(cudaMemsetAsync(w.d_fl, 0, n * 8, s), "cudaMemsetAsync");
    ck(cudaMemsetAsync(w.d_bl, 0, n * 8, s), "cudaMemsetAsync");
    ck(cudaMemsetAsync(w.d_ft, 0, n * 8, s), "cudaMemsetAsync");
    ck(cudaMemsetAsync(w.d_bt, 0, n * 8, s), "cudaMemsetAsync");
    hbs::k_sw_fill64<<<w.blocks(n), hbs::SW_THREADS, 0, s>>>(w.d_fh, n, n);
    hbs::k_sw_fill64<<<w.blocks(n), hbs::SW_THREADS, 0, s>>>(w.d_bh, n, n);
    ck(cudaGetLastError(), "k_sw_fill64");
    if (radial) {
        ck(cudaMemcpyAsync(w.d_radial, radial, n, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        w.compute_radial = false;
    } else {
        ck(cudaMemsetAsync(w.d_radial, 0, n, s), "cudaMemsetAsync");
    }
    w.sync();
    mark("device state");
    ck(cudaEventRecord(w.ev0, s), "cudaEventRecord");
    w.compute();
    ck(cudaEventRecord(w.ev1, s), "cudaEventRecord");
    w.sync();
    mark("visits and bounds");
    cudaEventElapsedTime(&w.device_ms, w.ev0, w.ev1);
    // output_level.rs: what each level reports, and its asserts
    out->diameter = w.diameter_low;
    out->radius = w.radius_high;
    out->diametral_vertex = w.diameter_vertex;
    out->radial_vertex = w.radius_vertex;
    out->radius_iterations = w.radius_it;
    out->diameter_iterations = w.diameter_it;
    out->forward_iterations = w.forward_it;
    out->all_iterations = w.all_it;
    out->sweeps = w.sweeps;
    out->device_ms = w.device_ms;
    const int lv = w.level;
    auto need = [&](bool ok, const char* what) {
        if (!ok) fail(HB_ERR_INVALID, std::string("Trying to build ") + kNames[level] + " without " + what);
    };
    if (lv == HB_SWEEP_ALL) need(w.all_it != NONE, "all eccentricities computed");
    if (lv == HB_SWEEP_ALL || lv == HB_SWEEP_ALL_FORWARD) need(w.forward_it != NONE, "all forward eccentricities computed");
    if (lv != HB_SWEEP_RADIUS) need(w.diameter_it != NONE, "the diameter computed");
    if (lv != HB_SWEEP_DIAMETER) need(w.radius_it != NONE, "the radius computed");
    if (fecc && (lv == HB_SWEEP_ALL || lv == HB_SWEEP_ALL_FORWARD))
        ck(cudaMemcpyAsync(fecc, w.d_fl, n * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    if (becc && lv == HB_SWEEP_ALL)
        ck(cudaMemcpyAsync(becc, w.d_bh, n * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    w.sync();
    return HB_OK;
}

}  // namespace

extern "C" {

int hb_exact_sum_sweep(const hb_graph_view* graph, const hb_graph_view* transpose, int level,
                       const uint8_t* radial_vertices, int device, void* stream, uint64_t* forward_eccentricities,
                       uint64_t* backward_eccentricities, hb_sweep_result* out) {
    nvtxRangePushA("hb_exact_sum_sweep");
    struct Pop {
        ~Pop() { nvtxRangePop(); }
    } pop;
    try {
        return run(graph, transpose, level, radial_vertices, device, stream, forward_eccentricities,
                   backward_eccentricities, out);
    } catch (const SweepError& e) {
        t_sweep_err = e.msg;
        return e.code;
    } catch (const std::bad_alloc&) {
        t_sweep_err = "host allocation failed";
        return HB_ERR_OOM;
    }
}

const char* hb_sweep_last_error(void) { return t_sweep_err.c_str(); }

}  // extern "C"
