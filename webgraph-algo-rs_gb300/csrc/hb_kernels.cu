// HyperBall kernels for sm_103a.
//
// One HyperBall iteration (reference: HyperBall::iterate / parallel_task,
// src/algo/hyperball/hyperball_impl.rs:775-1152) runs as
//   1. k_list_count,     — systolic iterations only: the light and medium
//      k_list_fill         nodes to check or to copy, in node order;
//   2. k_union_window    — one warp per chunk of nodes, chunks taken in node
//                          order from a global cursor; every node of
//                          out-degree up to tile_max_degree: merge of the
//                          successors' counters, modified test, next-state
//                          store, and for changed counters the exact count,
//                          neighbourhood-function part and per-node f64 sums
//                          (finish_node) while the counter is in registers;
//   3. k_union_heavy     — the same for the heavy nodes, one CTA per node;
//   4. k_sum_f64         — the neighbourhood-function parts summed in a fixed
//                          order (reproducible);
//   5. k_mark_preds      — systolic iterations: predecessors of modified nodes
//                          (through the transpose) into next-must-be-checked.
// Only successors flagged in the previous iteration's modified bitmap are
// merged (HB:1038), or all of them where that gives the same counters. The
// count of an unchanged counter is the cached estimate of the previous
// iteration, so only changed counters are counted.
//
// GB300's f64 pipe issues 2 lane-operations per cycle per SM (1/64 of fp32),
// so the epilogue keeps f64 instructions to the reference's own operations:
// one division for the estimate, the subtraction, the per-node sums, and a
// three-instruction correctly rounded division by the iteration number.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "hb_internal.h"
#include "hll_device.cuh"

using namespace hbd;

namespace hbk {

// kernels launched by this host thread (diagnostics: launches per iteration)
static thread_local uint64_t t_launches = 0;
uint64_t launch_count() { return t_launches; }
void count_launches(int64_t delta) { t_launches += (uint64_t)delta; }

// ---------------------------------------------------------------------------
// block-level publish of per-thread statistics into one partial slot
// ---------------------------------------------------------------------------
__device__ __forceinline__ void publish(double nf, unsigned long long vis, unsigned long long modc,
                                        unsigned long long scanned, TilePartial* slot) {
    __shared__ double s_nf[32];
    __shared__ unsigned long long s_v[32], s_m[32], s_s[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        nf = __dadd_rn(nf, __shfl_xor_sync(0xffffffffu, nf, off));
        vis += __shfl_xor_sync(0xffffffffu, vis, off);
        modc += __shfl_xor_sync(0xffffffffu, modc, off);
        scanned += __shfl_xor_sync(0xffffffffu, scanned, off);
    }
    if (lane == 0) {
        s_nf[warp] = nf;
        s_v[warp] = vis;
        s_m[warp] = modc;
        s_s[warp] = scanned;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned long long tv = 0, tm = 0, ts = 0;
        const int nwarps = (blockDim.x + 31) >> 5;
        for (int w = 0; w < nwarps; w++) {
            t = __dadd_rn(t, s_nf[w]);
            tv += s_v[w];
            tm += s_m[w];
            ts += s_s[w];
        }
        *slot = TilePartial{t, tv, tm, ts};
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// end of a node's union, run by the G lanes (one per chunk) of a team: store
// the merged counter into the next state; true when it differs from the
// previous one (HB:1052).
// ---------------------------------------------------------------------------
template <int LOG2M>
__device__ __forceinline__ bool commit_node(const UnionArgs& a, uint64_t v, int c,
                                            unsigned team_mask,
                                            const uint32_t (&prev)[Geo<LOG2M>::NW],
                                            const uint32_t (&acc)[Geo<LOG2M>::NW]) {
    using Gm = Geo<LOG2M>;
    constexpr int G = Gm::CHUNKS, NW = Gm::NW;
    uint32_t diff = 0;
#pragma unroll
    for (int i = 0; i < NW; i++) diff |= prev[i] ^ acc[i];
    bool changed = diff != 0u;
    if constexpr (G > 1) changed = __any_sync(team_mask, changed);
    store_chunk<LOG2M>(a.next, v, c, acc);
    return changed;
}

// ---------------------------------------------------------------------------
// End of a node's union, for the nodes whose counter changed: the per-node
// arithmetic of HB:1052-1093, run by the G lanes that hold the new counter
// (lane c == 0 does the f64 part), while it is still in registers:
//   post = count(new counter)   (exact integer harmonic sum, one division)
//   pre  = cached count of the previous counter
//   NF  += post (standard) or post - pre (systolic); unchanged nodes add
//          their cached count in standard iterations
//   delta = post - pre; if delta > 0: sod += delta*(t+1), harm += delta/(t+1),
//   discounted sums += delta*f(t+1)
// and the in-degree of a changed node is added to the arcs the next
// iteration visits.
// ---------------------------------------------------------------------------
// The per-node values finish_node reads (measured: loading them before the
// gather instead gains nothing and costs registers).
struct NodeSums {
    double pre, sod, harm;
    uint32_t indeg;
};

__device__ __forceinline__ NodeSums load_sums(const UnionArgs& a, uint32_t v) {
    NodeSums s;
    s.pre = a.est[v];
    s.sod = a.sod ? a.sod[v] : 0.0;
    s.harm = a.harm ? a.harm[v] : 0.0;
    s.indeg = __ldg(a.indeg + v);
    return s;
}

template <int LOG2M>
__device__ __forceinline__ void finish_node(const UnionArgs& a, uint32_t v, int c, unsigned gmask,
                                            const uint32_t (&acc)[Geo<LOG2M>::NW], bool changed,
                                            const NodeSums& ns, double& nf, uint32_t& vis) {
    using Gm = Geo<LOG2M>;
    constexpr int G = Gm::CHUNKS, REGS = Gm::CHUNK_REGS;
    if (changed) {
        uint64_t hs = 0;
        uint32_t z = 0, c31 = 0;
        count_chunk<REGS>(acc, hs, z, c31, a.any31 != 0);
        if constexpr (G > 1) {
#pragma unroll
            for (int off = 1; off < G; off <<= 1) {
                hs += __shfl_xor_sync(gmask, hs, off);
                z += __shfl_xor_sync(gmask, z, off);
                c31 += __shfl_xor_sync(gmask, c31, off);
            }
        }
        if (c == 0) {
            const double pre = ns.pre;
            const double post = estimate_fast(signed_hsum(hs, c31, a.quirk), z, a.alpha_m_m,
                                              a.a_scaled, a.small_bits, (double)Gm::M, a.ln_table);
            a.est[v] = post;
            if (a.systolic) {
                nf = __dadd_rn(nf, -pre);
                nf = __dadd_rn(nf, post);
            } else {
                nf = __dadd_rn(nf, post);
            }
            const double delta = __dsub_rn(post, pre);
            // delta > 0.0 as an integer test: positive, not NaN
            const long long db = __double_as_longlong(delta);
            if (db > 0 && db <= 0x7ff0000000000000ll) {
                const double d1 = __ldg(&a.ic->d1);
                if (a.sod) a.sod[v] = __dadd_rn(ns.sod, __dmul_rn(delta, d1));
                if (a.harm) a.harm[v] = __dadd_rn(ns.harm, div_by_small_int(delta, d1, __ldg(&a.ic->rd1)));
                for (int k = 0; k < a.ndisc; k++)
                    a.disc[k][v] = __dadd_rn(a.disc[k][v], __dmul_rn(delta, __ldg(&a.ic->disc_factor[k])));
            }
            vis += ns.indeg;
        }
    } else if (!a.systolic && c == 0) {
        nf = __dadd_rn(nf, ns.pre);
    }
}

// fixed-order warp sum (lane 0 gets it)
__device__ __forceinline__ double warp_sum_f64(double x) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x = __dadd_rn(x, __shfl_xor_sync(0xffffffffu, x, off));
    return x;
}

// ---------------------------------------------------------------------------
// windows and chunks: every node up to tile_max_degree
//
// The graph never changes, so the work order is fixed once at build time and
// the nodes are renumbered to follow it: nodes are cut into windows of WINDOW
// consecutive ids, and inside a window the heavy nodes, then the medium nodes
// (out-degree above the light bound, up to tile_max_degree), then the light
// nodes take the window's ids by decreasing out-degree. Renumbering moves a
// node by less than WINDOW, so URL-order locality survives, and a run of
// nodes of one kind is a run of consecutive ids: their offsets, counters and
// per-node sums are read and written coalesced. The runs are cut into chunks
// of one warp-step each (32/G light nodes, one lane-group each, or 32/TB_MED
// medium nodes, one team each); the chunk table follows node order. Heavy
// nodes run in k_union_heavy.
//
// k_union_window hands out the chunk table in order through a global cursor,
// so the warps in flight at any moment work on a narrow band of consecutive
// node ids; with URL-order locality their successors cluster around that band
// and its counters stay L2-resident while the band passes (a static
// assignment lets warps drift apart and the band outgrows L2). Systolic iterations
// walk node lists instead (k_list_fill): runs of the light list, then of the
// medium list; list order is node order, so locality and the degree order
// inside each kind survive. Neighbouring lanes walk successor lists of equal
// length; each lane keeps PIPE counter gathers in flight while the ids and
// modified bits of the next PIPE successors load.
//
// In iterations where nearly every counter changed before (`gather_all`), a
// successor's counter is merged without its modified bit: an unmodified
// successor's counter is already contained in the node's own
// (c_{t-1}(u) = c_{t-2}(u) <= c_{t-1}(v)), and so is the node's own counter,
// so merging them changes nothing and no dependent bitmap load stands before
// the gather. Visited arcs are not counted per arc at all: every predecessor
// of a node modified in t-1 is scanned in t, in every mode, so
// visited_t = sum over u modified in t-1 of (in-degree of u without
// self-loops), which finish_node accumulates for the next iteration.
// ---------------------------------------------------------------------------
constexpr int WINDOW = 1024;
// lanes of the team that runs one medium node: 8 arc lanes of G chunk lanes
// (measured at 2^26 web-like: 4 arc lanes 8% slower, 16 the same)
template <int LOG2M>
__host__ __device__ constexpr int team_lanes() {
    return 8 * Geo<LOG2M>::CHUNKS < 32 ? 8 * Geo<LOG2M>::CHUNKS : 32;
}
// counter loads in flight per lane: 64 bytes, within the register budget of
// three 256-thread blocks per SM (measured: more resident warps beat deeper
// per-lane pipelines)
template <int NW>
__host__ __device__ constexpr int pipe_depth() { return NW >= 16 ? 1 : NW >= 8 ? 2 : 4; }

template <int LOG2M>
struct TileGeo {
    static constexpr int NODES = WINDOW;
    static constexpr int ARCS = 1 << 30;  // no per-window arc limit
};

// Far successors: more than far_rows ids away from the node (mostly not in
// L2). The first FAR_SLOTS far successors of an arc lane that pass the filter
// come by one TMA gather (see collect_far); gather_rolling then skips them.
constexpr int FAR_SLOTS = 4;
__device__ __forceinline__ bool is_far(uint32_t s, uint32_t v, uint32_t far_rows) {
    return s - v + far_rows > 2 * far_rows;
}

template <int LOG2M, int FK>
__device__ __forceinline__ void filtered_gather(const UnionArgs& a, uint32_t v, int c, uint64_t e0,
                                                uint64_t e1, uint32_t stride,
                                                uint32_t (&acc)[Geo<LOG2M>::NW], int skip) {
    using Gm = Geo<LOG2M>;
    constexpr int NW = Gm::NW, REGS = Gm::CHUNK_REGS;
    for (uint64_t e = e0; e < e1; e += (uint64_t)FK * stride) {
        uint32_t ids[FK];
#pragma unroll
        for (int k = 0; k < FK; k++) {
            const uint64_t ek = e + (uint64_t)k * stride;
            ids[k] = ek < e1 ? __ldg(a.succ + ek) : v;
        }
        uint32_t want = 0;
#pragma unroll
        for (int k = 0; k < FK; k++)
            want |= (uint32_t)(ids[k] != v && test_bit(a.curr_mod, ids[k])) << k;
        if (!want) continue;
        if (a.pf) {
            // every wanted counter but the first is requested now, so the
            // loads below find them on chip
            const int first = __ffs(want) - 1;
#pragma unroll
            for (int k = 0; k < FK; k++)
                if (k != first && ((want >> k) & 1u)) prefetch_chunk<LOG2M>(a.curr, ids[k], c, a.pf);
        }
#pragma unroll
        for (int k = 0; k < FK; k++) {
            if (!((want >> k) & 1u)) continue;
            if (skip > 0 && is_far(ids[k], v, a.far_rows)) {
                skip--;
                continue;
            }
            uint32_t y[NW];
            load_chunk<LOG2M>(a.curr, ids[k], c, y);
            merge_chunk<REGS>(acc, y);
        }
    }
}

// Merges into acc (chunk c) the counters of the successors e0, e0+stride, ...
// (< e1) of node v: all of them, or (filter) only the non-loop ones modified
// in the previous iteration; the first `skip` far ones that qualify are left
// out (they arrive by TMA). PIPE counter loads stay in flight per lane.
// PIPEX: counter loads in flight per lane (0: pipe_depth)
template <int LOG2M, int PIPEX = 0>
__device__ __forceinline__ void gather_rolling(const UnionArgs& a, uint32_t v, int c, uint64_t e0,
                                               uint64_t e1, uint32_t stride, bool filter,
                                               uint32_t (&acc)[Geo<LOG2M>::NW], int skip) {
    using Gm = Geo<LOG2M>;
    constexpr int NW = Gm::NW, REGS = Gm::CHUNK_REGS, PIPE = PIPEX ? PIPEX : pipe_depth<NW>();
    auto wanted = [&](uint32_t s) {
        bool w = !filter || (s != v && test_bit(a.curr_mod, s));
        if (skip > 0 && w && is_far(s, v, a.far_rows)) {
            skip--;
            w = false;
        }
        return w;
    };
    if (filter) {
        // Filtered: the ids and modified bits of FK arcs load together, so
        // their latencies overlap; then the counters of the modified ones, in
        // arc order. Systolic iterations (few successors modified) take 16
        // arcs at a time, filtered standard iterations (many modified) 4.
        if (a.systolic)
            filtered_gather<LOG2M, 16>(a, v, c, e0, e1, stride, acc, skip);
        else
            filtered_gather<LOG2M, 4>(a, v, c, e0, e1, stride, acc, skip);
        return;
    }
    if constexpr (PIPE == 1) {
        // one counter in flight: the next successor id loads while the current
        // counter is merged
        if (e0 >= e1) return;
        const uint32_t* sp = a.succ + e0;
        const uint32_t cnt = (uint32_t)((e1 - e0 + stride - 1) / stride);
        uint32_t s = __ldg(sp);
        bool have = wanted(s);
        uint32_t y[NW];
        if (have) load_chunk<LOG2M>(a.curr, s, c, y);
        if (a.pf) {
            // the same with the counter `pd` arcs ahead requested early
            const uint32_t pd = a.pd;
            for (uint32_t k = 1; k <= pd && k < cnt; k++)
                prefetch_chunk<LOG2M>(a.curr, __ldg(sp + (uint64_t)k * stride), c, a.pf);
            for (uint32_t i = 1; i < cnt; i++) {
                const uint32_t ns = __ldg(sp + (uint64_t)i * stride);
                if (i + pd < cnt)
                    prefetch_chunk<LOG2M>(a.curr, __ldg(sp + (uint64_t)(i + pd) * stride), c, a.pf);
                const bool nh = wanted(ns);
                if (have) merge_chunk<REGS>(acc, y);
                if (nh) load_chunk<LOG2M>(a.curr, ns, c, y);
                have = nh;
            }
        } else {
            for (uint32_t i = 1; i < cnt; i++) {
                const uint32_t ns = __ldg(sp + (uint64_t)i * stride);
                const bool nh = wanted(ns);
                if (have) merge_chunk<REGS>(acc, y);
                if (nh) load_chunk<LOG2M>(a.curr, ns, c, y);
                have = nh;
            }
        }
        if (have) merge_chunk<REGS>(acc, y);
    } else {
        uint32_t y[PIPE][NW];
        bool have[PIPE];
        uint32_t nid[PIPE];
#pragma unroll
        for (int k = 0; k < PIPE; k++) {
            const uint64_t e = e0 + (uint64_t)k * stride;
            const uint32_t sid = e < e1 ? __ldg(a.succ + e) : v;
            const uint64_t en = e + (uint64_t)PIPE * stride;
            nid[k] = en < e1 ? __ldg(a.succ + en) : v;
            have[k] = e < e1 && wanted(sid);
            if (have[k]) load_chunk<LOG2M>(a.curr, sid, c, y[k]);
        }
        for (uint64_t e = e0 + (uint64_t)PIPE * stride; e < e1 + (uint64_t)PIPE * stride;
             e += (uint64_t)PIPE * stride) {
#pragma unroll
            for (int k = 0; k < PIPE; k++) {
                if (have[k]) merge_chunk<REGS>(acc, y[k]);
                const uint64_t ek = e + (uint64_t)k * stride;
                const uint32_t sid = nid[k];
                const uint64_t en = ek + (uint64_t)PIPE * stride;
                nid[k] = en < e1 ? __ldg(a.succ + en) : v;
                have[k] = ek < e1 && wanted(sid);
                if (have[k]) load_chunk<LOG2M>(a.curr, sid, c, y[k]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// TMA gathers of far successors. Every lane group (the G lanes of one counter)
// owns FAR_SLOTS counter rows of its warp's shared memory; one
// cp.async.bulk.tensor tile::gather4 copy fills them from the tensor map of
// the current counters (rows of 2^log2m bytes), and the warp's mbarrier
// counts the bytes in. The copies run while the lanes gather their near
// successors with plain loads.
// ---------------------------------------------------------------------------
template <int LOG2M>
struct FarGeo {
    static constexpr bool ON = LOG2M <= 8;  // a box row is at most 256 bytes
    static constexpr int ROW = Geo<LOG2M>::COUNTER_BYTES;
    static constexpr int GROUPS = 32 / Geo<LOG2M>::CHUNKS;
    // a group's rows start on a 128-byte boundary
    static constexpr int REGION = FAR_SLOTS * ROW < 128 ? 128 : FAR_SLOTS * ROW;
    static constexpr int WARP_BYTES = ON ? GROUPS * REGION : 0;
};

// the bounded wait gives up after this many polls (each poll may suspend the
// thread for a while); the kernel then reports a timeout
constexpr int MBAR_POLLS = 1 << 20;

__device__ __forceinline__ void mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, uint32_t polls) {
    const uint32_t limit = polls ? polls : (uint32_t)MBAR_POLLS;
    uint32_t done = 0;
    for (uint32_t i = 0; i < limit && !done; i++)
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
    return done != 0;
}
// counts `bytes` in as if a copy had delivered them (releases the bytes a
// test added to the expected count)
__device__ __forceinline__ void mbar_complete_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// orders this thread's earlier shared-memory reads before later TMA writes
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tma_gather4(uint32_t dst, const CUtensorMap* map, uint32_t r0,
                                            uint32_t r1, uint32_t r2, uint32_t r3, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(map), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(bar)
        : "memory");
}

// The first FAR_SLOTS far successors among e0, e0+stride, ... (< e1) that
// pass the filter, in arc order; unused slots repeat v. Returns how many.
__device__ __forceinline__ int collect_far(const UnionArgs& a, uint32_t v, uint64_t e0, uint64_t e1,
                                           uint32_t stride, bool filter, uint32_t (&f)[FAR_SLOTS]) {
    int nf = 0;
#pragma unroll
    for (int k = 0; k < FAR_SLOTS; k++) f[k] = v;
    for (uint64_t e = e0; e < e1 && nf < FAR_SLOTS; e += stride) {
        const uint32_t s = __ldg(a.succ + e);
        if (is_far(s, v, a.far_rows) && (!filter || test_bit(a.curr_mod, s))) {
#pragma unroll
            for (int k = 0; k < FAR_SLOTS; k++)
                if (k == nf) f[k] = s;
            nf++;
        }
    }
    return nf;
}

// Merges rows [0, nf) of the group's slots (chunk c of each) into acc.
template <int LOG2M>
__device__ __forceinline__ void merge_far(uint32_t region, int c, int nf,
                                          uint32_t (&acc)[Geo<LOG2M>::NW]) {
    using Gm = Geo<LOG2M>;
    constexpr int NW = Gm::NW;
    for (int j = 0; j < nf; j++) {
        const uint32_t p = region + (uint32_t)(j * FarGeo<LOG2M>::ROW + c * Gm::CHUNK_BYTES);
        uint32_t y[NW];
#pragma unroll
        for (int q = 0; q < NW / 4; q++)
            asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(y[4 * q]), "=r"(y[4 * q + 1]), "=r"(y[4 * q + 2]), "=r"(y[4 * q + 3])
                         : "r"(p + 16 * q));
        merge_chunk<Gm::CHUNK_REGS>(acc, y);
    }
}

// A warp's far-gather slots and mbarrier (dynamic and static shared memory of
// the union kernel), and its state: bit 0 the barrier's phase, bit 1 set when
// a wait gave up (the warp then issues no more TMA copies).
extern __shared__ __align__(128) uint8_t far_smem[];
__shared__ __align__(8) unsigned long long far_bar[8];
template <int LOG2M>
__device__ __forceinline__ uint32_t far_region(int lane) {
    return (uint32_t)__cvta_generic_to_shared(far_smem) +
           (threadIdx.x >> 5) * (uint32_t)FarGeo<LOG2M>::WARP_BYTES +
           (uint32_t)((lane / Geo<LOG2M>::CHUNKS) * FarGeo<LOG2M>::REGION);
}
__device__ __forceinline__ uint32_t far_barrier() {
    return (uint32_t)__cvta_generic_to_shared(&far_bar[threadIdx.x >> 5]);
}
struct FarState {
    uint32_t bits;
};

// true when chunk c of counter v in `base` differs from w (read 32 bytes at a
// time, so few registers are live)
template <int LOG2M>
__device__ __forceinline__ bool differs_from(const uint8_t* __restrict__ base, uint64_t v, int c,
                                             const uint32_t (&w)[Geo<LOG2M>::NW]) {
    using Gm = Geo<LOG2M>;
    constexpr int NW = Gm::NW;
    const uint8_t* p = base + v * (uint64_t)Gm::COUNTER_BYTES + (uint64_t)c * Gm::CHUNK_BYTES;
    uint32_t diff = 0;
    if constexpr (NW >= 8) {
#pragma unroll
        for (int i = 0; i < NW / 8; i++) {
            uint32_t x[8];
            ld_nc_256(p + 32 * i, x);
#pragma unroll
            for (int k = 0; k < 8; k++) diff |= x[k] ^ w[8 * i + k];
        }
    } else {
        const uint4 t = __ldg(reinterpret_cast<const uint4*>(p));
        diff = (t.x ^ w[0]) | (t.y ^ w[1]) | (t.z ^ w[2]) | (t.w ^ w[3]);
    }
    return diff != 0u;
}

// One warp-step over up to 32/TB nodes: the consecutive nodes [b, e), or
// list[b .. e) when a list is given. Scan, copy or nothing; sets the modified
// bits and counts scanned nodes, their arcs and the changed counters.
template <int LOG2M, int TB, bool FAR, int PIPEX = 0>
__device__ __forceinline__ void run_nodes(const UnionArgs& a, const uint32_t* __restrict__ list,
                                          uint32_t b, uint32_t e, uint32_t& modc, uint32_t& scanned,
                                          uint32_t& sarcs, uint32_t& vis, double& nf, FarState& fs) {
    using Gm = Geo<LOG2M>;
    constexpr int G = Gm::CHUNKS, NW = Gm::NW;
    constexpr int PB = TB / G;   // arc lanes per node
    constexpr int NPW = 32 / TB; // nodes per warp-step
    const int lane = threadIdx.x & 31;
    const int slot = lane / TB, tl = lane % TB, p = tl / G, c = tl % G;
    const unsigned tmask = TB == 32 ? 0xffffffffu : (((1u << TB) - 1u) << (slot * TB));
    const unsigned lmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (slot * TB));
    const bool filter = !a.gather_all;
    for (uint32_t base = b; base < e; base += NPW) {
        const uint32_t idx = base + slot;
        const uint32_t v = list ? (idx < e ? __ldg(list + idx) : 0u) : idx;
        bool scan = false, copy = false;
        if (idx < e) {
            if (!a.systolic || test_bit(a.mbc, v))
                scan = true;
            else if (test_bit(a.curr_mod, v))
                copy = true;
        }
        uint64_t s0 = 0, s1 = 0;
        if (scan) {
            s0 = __ldg(a.off + v);
            s1 = __ldg(a.off + v + 1);
        }
        // far successors: one TMA gather per lane group, in flight during the
        // plain loads below
        int nfar = 0;
        bool far_used = false, gave_up = false;
        if constexpr (FAR && FarGeo<LOG2M>::ON) {
            if (!(fs.bits & 2u)) {
                uint32_t f[FAR_SLOTS];
                if (scan) nfar = collect_far(a, v, s0 + p, s1, PB, filter, f);
                const bool issue = nfar > 0 && c == 0;
                const unsigned im = __ballot_sync(0xffffffffu, issue);
                if (im) {
                    far_used = true;
                    if (lane == 0)
                        mbar_arrive_expect(far_barrier(),
                                           (uint32_t)__popc(im) * FAR_SLOTS * FarGeo<LOG2M>::ROW +
                                               a.test_extra_tx);
                    __syncwarp();
                    if (issue)
                        tma_gather4(far_region<LOG2M>(lane), &a.far_map, f[0], f[1], f[2], f[3],
                                    far_barrier());
                }
            }
        }
        bool changed = false;
        if (scan) {
            uint32_t acc[NW];
            if (PB == 1 || p == 0) {
                load_chunk<LOG2M>(a.curr, v, c, acc);
            } else {
#pragma unroll
                for (int k = 0; k < NW; k++) acc[k] = 0u;
            }
            gather_rolling<LOG2M, PIPEX>(a, v, c, s0 + p, s1, PB, filter, acc, nfar);
            if (nfar > 0) {
                if (mbar_wait(far_barrier(), fs.bits & 1u, a.mbar_polls)) {
                    merge_far<LOG2M>(far_region<LOG2M>(lane), c, nfar, acc);
                    fence_proxy_async();
                } else {
                    gave_up = true;
                }
            }
            if constexpr (PB > 1) {
                __syncwarp(tmask);
#pragma unroll
                for (int off = G; off < TB; off <<= 1) {
                    // four words at a time keeps few registers live
#pragma unroll
                    for (int k = 0; k < NW; k += 4) {
                        uint32_t x4[4], y4[4];
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            x4[j] = acc[k + j];
                            y4[j] = __shfl_xor_sync(tmask, acc[k + j], off);
                        }
                        merge_chunk<16>(x4, y4);
#pragma unroll
                        for (int j = 0; j < 4; j++) acc[k + j] = x4[j];
                    }
                }
            }
            if (p == 0) {
                // the previous counter, read again (L1/L2) rather than kept in registers
                changed = differs_from<LOG2M>(a.curr, v, c, acc);
                if constexpr (G > 1) changed = __any_sync(lmask, changed);
                store_chunk<LOG2M>(a.next, v, c, acc);
                if (c == 0) {
                    scanned++;
                    sarcs += (uint32_t)(s1 - s0);
                }
                NodeSums ns{};
                if (c == 0) ns = load_sums(a, v);
                finish_node<LOG2M>(a, v, c, lmask, acc, changed, ns, nf, vis);
            }
        } else if (copy && p == 0) {
            uint32_t w[NW];
            load_chunk<LOG2M>(a.curr, v, c, w);
            store_chunk<LOG2M>(a.next, v, c, w);
        }
        if constexpr (FAR && FarGeo<LOG2M>::ON) {
            if (__any_sync(0xffffffffu, gave_up)) {
                // A wait gave up: the iteration fails (HB_ERR_TIMEOUT). Drain
                // this warp's copies before going on without the far path:
                // release any bytes a test added to the expected count, then
                // wait once more, again bounded, for the phase to complete.
                if (lane == 0 && a.test_extra_tx) mbar_complete_tx(far_barrier(), a.test_extra_tx);
                __syncwarp();
                mbar_wait(far_barrier(), fs.bits & 1u, a.mbar_polls);
                fs.bits |= 2u;
            }
        }
        if (far_used) fs.bits ^= 1u;
        // modified bits, aggregated over the lanes that hit the same word
        const bool flag = changed && p == 0 && c == 0;
        const unsigned want = __ballot_sync(0xffffffffu, flag);
        if (want) {
            const uint32_t word = flag ? (v >> 5) : 0xffffffffu;
            const unsigned peers = __match_any_sync(0xffffffffu, word);
            // each group of lanes on one word reduces with its own mask
            const uint32_t bits = __reduce_or_sync(peers, flag ? (1u << (v & 31)) : 0u);
            if (flag && lane == __ffs(peers) - 1) atomicOr(a.next_mod + word, bits);
            modc += flag;
        }
    }
}

// The medium path (measured: inlining it beats a separate call frame).
template <int LOG2M, int TB, bool FAR>
__device__ __forceinline__ void run_medium(const UnionArgs& a, uint32_t b, uint32_t e,
                                        uint32_t& modc, uint32_t& scanned, uint32_t& sarcs,
                                        uint32_t& vis, double& nf, FarState& fs) {
    run_nodes<LOG2M, TB, FAR>(a, a.medium_list, b, e, modc, scanned, sarcs, vis, nf, fs);
}

// Work item k: a chunk of the table, or (systolic) a run of the light list
// followed by runs of the medium list; {first, count | medium << 31}.
struct WorkItems {
    uint32_t n_work, light_items;
    uint32_t n_light, n_medium;
};

template <int NPW_L, int NPW_M>
__device__ __forceinline__ WorkItems work_items(const UnionArgs& a) {
    WorkItems w{};
    if (a.queue) {
        // a batch's standard iteration: the chunks of its running instances
        w.n_work = *a.queue_len;
    } else if (a.light_list) {
        const uint64_t c = *a.list_counts;
        w.n_light = (uint32_t)c;
        w.n_medium = (uint32_t)(c >> 32);
        w.light_items = (w.n_light + NPW_L - 1) / NPW_L;
        w.n_work = w.light_items + (w.n_medium + NPW_M - 1) / NPW_M;
    } else {
        w.n_work = (uint32_t)a.n_chunks;
    }
    return w;
}

template <int NPW_L, int NPW_M>
__device__ __forceinline__ uint2 item_at(const UnionArgs& a, const WorkItems& w,
                                         uint32_t k) {
    if (k >= w.n_work) return make_uint2(0u, 0u);
    if (a.queue) return __ldg(a.chunks + __ldg(a.queue + k));
    if (!a.light_list) return __ldg(a.chunks + k);
    if (k < w.light_items) {
        const uint32_t f = (uint32_t)(k * NPW_L);
        return make_uint2(f, min((uint32_t)NPW_L, w.n_light - f));
    }
    const uint32_t f = (uint32_t)((k - w.light_items) * NPW_M);
    return make_uint2(f, min((uint32_t)NPW_M, w.n_medium - f) | 0x80000000u);
}

// FAR: far successors by TMA gathers (an option: measured slower than plain
// loads on the web-like and R-MAT workloads)
// MINB: resident blocks per SM the registers are sized for (3: 80 registers
// a thread, 4: 64; the autotuner picks one per graph)
// PIPEX: counter loads in flight per light lane (0: pipe_depth; the 2-block
// build has the registers for 2 at 16 words per lane)
template <int LOG2M, bool FAR, int MINB, int PIPEX = 0>
__global__ void __launch_bounds__(256, MINB) k_union_window(const __grid_constant__ UnionArgs a) {
    using Gm = Geo<LOG2M>;
    constexpr int G = Gm::CHUNKS;
    constexpr int TB_MED = team_lanes<LOG2M>();
    const int lane = threadIdx.x & 31;
    // per warp: the mbarrier of its far-successor TMA copies
    FarState fs{0u};
    if constexpr (FAR && FarGeo<LOG2M>::ON) {
        if (lane == 0) mbar_init(far_barrier());
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        __syncwarp();
    }
    constexpr int NPW_L = 32 / G, NPW_M = 32 / TB_MED;
    // per-warp totals: at most one warp's share of the nodes and arcs of one
    // iteration, far below 2^32
    uint32_t modc = 0, scanned = 0, sarcs = 0, vis = 0;
    const WorkItems wi = work_items<NPW_L, NPW_M>(a);
    const uint32_t n_work = wi.n_work;
    // Work items come GRAB at a time from the cursor (one atomic per GRAB
    // chunks; measured fastest at 1). Handing out consecutive items keeps the
    // band of nodes in flight narrow.
    constexpr unsigned GRAB = 1;
    uint32_t k = 0, kend = 0;
    for (;;) {
        if (k == kend) {
            uint32_t first = 0;
            if (lane == 0) first = (uint32_t)atomicAdd(a.cursor, (unsigned long long)GRAB);
            k = __shfl_sync(0xffffffffu, first, 0);
            kend = k + GRAB;
        }
        if (k >= n_work) break;
        const uint2 d = item_at<NPW_L, NPW_M>(a, wi, k);
        k++;
        const uint32_t cnt = d.y & 0x7fffffffu;
        double nf = 0.0;
        if (d.y >> 31)
            run_medium<LOG2M, TB_MED, FAR>(a, d.x, d.x + cnt, modc, scanned, sarcs, vis, nf, fs);
        else
            run_nodes<LOG2M, G, FAR, PIPEX>(a, a.light_list, d.x, d.x + cnt, modc, scanned, sarcs, vis, nf, fs);
        // the item's neighbourhood-function part: fixed lanes, fixed order
        nf = warp_sum_f64(nf);
        if (lane == 0) a.nf_items[k - 1] = nf;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        modc += __shfl_xor_sync(0xffffffffu, modc, off);
        scanned += __shfl_xor_sync(0xffffffffu, scanned, off);
        sarcs += __shfl_xor_sync(0xffffffffu, sarcs, off);
        vis += __shfl_xor_sync(0xffffffffu, vis, off);
    }
    if (lane == 0) {
        // integer totals are order independent
        TilePartial* t = a.partials + a.acc_slot;
        if (modc) atomicAdd(&t->mod, (unsigned long long)modc);
        if (scanned) atomicAdd(&t->scanned, (unsigned long long)scanned);
        if (sarcs) atomicAdd(&t->sarcs, (unsigned long long)sarcs);
        if (vis) atomicAdd(&t->vis, (unsigned long long)vis);
    }
    if (__any_sync(0xffffffffu, (fs.bits & 2u) != 0) && lane == 0)
        atomicAdd(&a.partials[a.acc_slot].timeouts, 1ull);
}

// ---------------------------------------------------------------------------
// Several HyperBall instances in one launch: the window work of up to
// MAX_JOBS handles (the log2m groups of a batch, the running jobs of a
// server), each with its own arguments and log2m in {4, 6, 8}, drained from
// one cursor. A block first turns the jobs' work-item counts into a prefix
// in shared memory; a warp maps each item it takes to its job and runs it
// exactly as k_union_window would (same items, lanes and order, so every
// counter and per-item neighbourhood-function part is that job's alone).
// Integer totals go to each job's partial slot when the warp moves to
// another job.
// ---------------------------------------------------------------------------

template <int LOG2M>
__device__ __forceinline__ WorkItems job_items(const UnionArgs& a) {
    constexpr int G = Geo<LOG2M>::CHUNKS, TB_MED = team_lanes<LOG2M>();
    return work_items<32 / G, 32 / TB_MED>(a);
}

template <int LOG2M>
__device__ __forceinline__ void job_item(const UnionArgs& a, const WorkItems& wi, uint32_t k,
                                         uint32_t& modc, uint32_t& scanned, uint32_t& sarcs,
                                         uint32_t& vis) {
    using Gm = Geo<LOG2M>;
    constexpr int G = Gm::CHUNKS;
    constexpr int TB_MED = team_lanes<LOG2M>();
    constexpr int NPW_L = 32 / G, NPW_M = 32 / TB_MED;
    const uint2 d = item_at<NPW_L, NPW_M>(a, wi, k);
    const uint32_t cnt = d.y & 0x7fffffffu;
    FarState fs{0u};
    double nf = 0.0;
    if (d.y >> 31)
        run_medium<LOG2M, TB_MED, false>(a, d.x, d.x + cnt, modc, scanned, sarcs, vis, nf, fs);
    else
        run_nodes<LOG2M, G, false>(a, a.light_list, d.x, d.x + cnt, modc, scanned, sarcs, vis, nf, fs);
    nf = warp_sum_f64(nf);
    if ((threadIdx.x & 31) == 0) a.nf_items[k] = nf;
}

__device__ __forceinline__ void flush_totals(const UnionArgs& a, uint32_t& modc, uint32_t& scanned,
                                             uint32_t& sarcs, uint32_t& vis) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        modc += __shfl_xor_sync(0xffffffffu, modc, off);
        scanned += __shfl_xor_sync(0xffffffffu, scanned, off);
        sarcs += __shfl_xor_sync(0xffffffffu, sarcs, off);
        vis += __shfl_xor_sync(0xffffffffu, vis, off);
    }
    if ((threadIdx.x & 31) == 0) {
        TilePartial* t = a.partials + a.acc_slot;
        if (modc) atomicAdd(&t->mod, (unsigned long long)modc);
        if (scanned) atomicAdd(&t->scanned, (unsigned long long)scanned);
        if (sarcs) atomicAdd(&t->sarcs, (unsigned long long)sarcs);
        if (vis) atomicAdd(&t->vis, (unsigned long long)vis);
    }
    modc = scanned = sarcs = vis = 0;
}

template <int MINB>
__global__ void __launch_bounds__(256, MINB) k_union_jobs(const __grid_constant__ JobsArgs p) {
    __shared__ uint32_t s_first[MAX_JOBS + 1];
    __shared__ WorkItems s_wi[MAX_JOBS];
    const uint32_t njobs = p.njobs;
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t j = 0; j < njobs; j++) {
            s_first[j] = t;
            const UnionArgs& a = p.job[j];
            WorkItems wi{};
            switch (p.log2m[j]) {
                case 4: wi = job_items<4>(a); break;
                case 6: wi = job_items<6>(a); break;
                case 8: wi = job_items<8>(a); break;
                default: break;
            }
            s_wi[j] = wi;
            t += wi.n_work;
        }
        s_first[njobs] = t;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t total = s_first[njobs];
    uint32_t modc = 0, scanned = 0, sarcs = 0, vis = 0;
    uint32_t cur_job = 0xffffffffu;
    for (;;) {
        uint32_t w = 0;
        if (lane == 0) w = (uint32_t)atomicAdd(p.cursor, 1ull);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= total) break;
        uint32_t j = 0;
        while (j + 1 < njobs && s_first[j + 1] <= w) j++;
        if (j != cur_job) {
            if (cur_job != 0xffffffffu) flush_totals(p.job[cur_job], modc, scanned, sarcs, vis);
            cur_job = j;
        }
        const UnionArgs& a = p.job[j];
        const uint32_t k = w - s_first[j];
        const WorkItems wi = s_wi[j];
        switch (p.log2m[j]) {
            case 4: job_item<4>(a, wi, k, modc, scanned, sarcs, vis); break;
            case 6: job_item<6>(a, wi, k, modc, scanned, sarcs, vis); break;
            case 8: job_item<8>(a, wi, k, modc, scanned, sarcs, vis); break;
            default: break;
        }
    }
    if (cur_job != 0xffffffffu) flush_totals(p.job[cur_job], modc, scanned, sarcs, vis);
}

// batches: the chunks of the running instances, in chunk order. inst_chunk[i]
// is instance i's first chunk (inst_chunk[count] = n_chunks); an instance
// runs when its modified count of the previous iteration is nonzero (`all`:
// every instance, the first iteration). One thread per chunk; `at` holds the
// exclusive scan of the running instances' chunk counts (count + 1 words).
__global__ void k_inst_chunk_counts(const uint32_t* __restrict__ inst_chunk,
                                    const unsigned long long* __restrict__ inst_mod, uint32_t count,
                                    int all, unsigned long long* __restrict__ cnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= count; i += gridDim.x * blockDim.x)
        cnt[i] = i < count && (all || inst_mod[i] != 0) ? inst_chunk[i + 1] - inst_chunk[i] : 0;
}
__global__ void k_inst_queue(const uint32_t* __restrict__ inst_chunk,
                             const unsigned long long* __restrict__ inst_mod, uint32_t count, int all,
                             const uint64_t* __restrict__ at, uint32_t n_chunks,
                             uint32_t* __restrict__ queue, uint32_t* __restrict__ queue_len) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_chunks; k += gridDim.x * blockDim.x) {
        // the instance of chunk k: the last i with inst_chunk[i] <= k
        uint32_t lo = 0, hi = count;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (inst_chunk[mid] <= k) lo = mid;
            else hi = mid;
        }
        if (all || inst_mod[lo] != 0) queue[at[lo] + (k - inst_chunk[lo])] = k;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *queue_len = (uint32_t)at[count];
}
// inst_chunk[i] = the first chunk whose first node is at or after start[i]
__global__ void k_inst_first_chunk(const uint2* __restrict__ chunks, uint64_t n_chunks,
                                   const uint64_t* __restrict__ start, uint32_t count,
                                   uint32_t* __restrict__ inst_chunk) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= count; i += gridDim.x * blockDim.x) {
        uint64_t lo = 0, hi = n_chunks;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if ((uint64_t)__ldg(&chunks[mid].x) < start[i]) lo = mid + 1;
            else hi = mid;
        }
        inst_chunk[i] = (uint32_t)lo;
    }
}

// ---------------------------------------------------------------------------
// Staged window kernel for standard iterations (every node scanned).
//
// k_union_window spends most of a light node's time in dependent round trips
// that carry few bytes: the cursor atomic, the chunk descriptor, the
// offsets, the first successor id, the per-node sums after the merge. Here
// every warp runs a software pipeline over its work items:
//   * the cursor is read two items ahead and the item descriptor
//     ({first node, count | medium << 31, first arc, arcs}) one item ahead;
//   * while item k runs, cp.async copies item k+1's offsets, successor ids
//     (up to STAGE_IDS of them), cached estimates, per-node sums and
//     in-degrees into the warp's other shared-memory buffer;
// so an item starts with everything but the counters on chip: the own
// counter and the successor gathers are the only global round trips left,
// and the gathers of a lane are issued PIPE at a time from ids in shared
// memory. Nodes of an item are consecutive, so the modified bits of an item
// are one ballot and at most two atomicOr.
// The counters, the neighbourhood-function part of each item (same items,
// same lanes, same order) and every per-node value are those of
// k_union_window. Requires m < 2^32 (item arcs are u32).
// ---------------------------------------------------------------------------
constexpr int STAGE_IDS = 256;  // successor ids staged per item

template <int LOG2M>
struct StageGeo {
    static constexpr int MAXN = 32 / Geo<LOG2M>::CHUNKS;  // nodes of a light item (>= medium)
    static constexpr int IDW = STAGE_IDS + 8;             // room for the 16-byte alignment shift
    // byte offsets inside one buffer
    static constexpr int OFF_IDS = 0;
    static constexpr int OFF_OFF = OFF_IDS + IDW * 4;
    static constexpr int OFF_EST = OFF_OFF + ((MAXN + 2) / 2) * 16;
    static constexpr int OFF_SOD = OFF_EST + MAXN * 8;
    static constexpr int OFF_HARM = OFF_SOD + MAXN * 8;
    static constexpr int OFF_INDEG = OFF_HARM + MAXN * 8;
    static constexpr int OFF_DESC = OFF_INDEG + ((MAXN * 4 + 15) / 16) * 16;
    static constexpr int BUF = OFF_DESC + 16;
    static constexpr int WARP = 2 * BUF;
};

template <int LOG2M>
__host__ __device__ constexpr int staged_smem_bytes() {
    return 8 * StageGeo<LOG2M>::WARP;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Item k+1's per-node data and successor ids into buffer `buf` (byte address
// in shared memory) by the 32 lanes of the warp. d = {first, count | medium
// << 31, first arc, arcs}. The successor array is padded to a multiple of 4
// ids plus 8, so the last 16-byte copy stays inside it.
template <int LOG2M, bool IDS>
__device__ __forceinline__ void stage_item(const UnionArgs& a, uint4 d, uint32_t buf, int lane) {
    using SG = StageGeo<LOG2M>;
    const uint32_t first = d.x, cnt = d.y & 0x7fffffffu;
    // ids: 16-byte units from the aligned word at or below the first arc
    const uint32_t base = d.z & ~3u;
    const uint32_t want = IDS ? min(d.w, (uint32_t)STAGE_IDS) : 0u;
    const uint32_t units = (d.z + want - base + 3) >> 2;
    for (uint32_t u = lane; u < units; u += 32)
        cp_async16(buf + SG::OFF_IDS + 16 * u, a.succ + base + 4 * u);
    // cnt + 1 offsets: up to 33 of them
    for (uint32_t i = lane; i <= cnt; i += 32) cp_async8(buf + SG::OFF_OFF + 8 * i, a.off + first + i);
    if ((uint32_t)lane < cnt) {
        cp_async8(buf + SG::OFF_EST + 8 * lane, a.est + first + lane);
        if (a.sod) cp_async8(buf + SG::OFF_SOD + 8 * lane, a.sod + first + lane);
        if (a.harm) cp_async8(buf + SG::OFF_HARM + 8 * lane, a.harm + first + lane);
        cp_async4(buf + SG::OFF_INDEG + 4 * lane, a.indeg + first + lane);
    }
    if (lane == 0) {
        // the descriptor itself, for the lanes that run the item
        asm volatile("st.shared.v4.u32 [%0], {%1,%2,%3,%4};" ::"r"(buf + SG::OFF_DESC), "r"(d.x),
                     "r"(d.y), "r"(base), "r"(d.z + want) : "memory");
    }
}

template <class T>
__device__ __forceinline__ T lds(uint32_t addr);
template <>
__device__ __forceinline__ uint32_t lds<uint32_t>(uint32_t addr) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
    return v;
}
template <>
__device__ __forceinline__ unsigned long long lds<unsigned long long>(uint32_t addr) {
    unsigned long long v;
    asm volatile("ld.shared.u64 %0, [%1];" : "=l"(v) : "r"(addr));
    return v;
}
template <>
__device__ __forceinline__ double lds<double>(uint32_t addr) {
    double v;
    asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"(addr));
    return v;
}

// Successor id of arc e: from the staged ids when it is among them.
struct StagedIds {
    uint32_t smem;   // address of staged word 0 (arc `base`)
    uint32_t base;   // arc of staged word 0
    uint32_t end;    // arcs below this are staged
    const uint32_t* succ;
    __device__ __forceinline__ uint32_t operator()(uint32_t e) const {
        return e < end ? lds<uint32_t>(smem + 4 * (e - base)) : __ldg(succ + e);
    }
};

// Merges into acc (chunk c) the counters of arcs e0, e0 + stride, ... (< e1):
// all of them (gather_all) or the non-loop ones modified in the previous
// iteration. PIPE counter loads in flight per lane.
template <int LOG2M, int PIPE>
__device__ __forceinline__ void staged_gather(const UnionArgs& a, const StagedIds& ids, uint32_t v,
                                              int c, uint32_t e0, uint32_t e1, uint32_t stride,
                                              uint32_t (&acc)[Geo<LOG2M>::NW]) {
    using Gm = Geo<LOG2M>;
    constexpr int NW = Gm::NW, REGS = Gm::CHUNK_REGS;
    if (a.gather_all) {
        uint32_t y[PIPE][NW];
        bool have[PIPE];
#pragma unroll
        for (int k = 0; k < PIPE; k++) {
            const uint32_t e = e0 + k * stride;
            have[k] = e < e1;
            if (have[k]) load_chunk<LOG2M>(a.curr, ids(e), c, y[k]);
        }
        for (uint32_t e = e0 + PIPE * stride; have[0]; e += PIPE * stride) {
#pragma unroll
            for (int k = 0; k < PIPE; k++) {
                if (have[k]) merge_chunk<REGS>(acc, y[k]);
                const uint32_t ek = e + k * stride;
                have[k] = ek < e1;
                if (have[k]) load_chunk<LOG2M>(a.curr, ids(ek), c, y[k]);
            }
        }
        return;
    }
    // filtered: the ids and modified bits of 4 arcs load together, then the
    // counters of the modified ones
    constexpr int FK = 4;
    for (uint32_t e = e0; e < e1; e += FK * stride) {
        uint32_t id[FK];
#pragma unroll
        for (int k = 0; k < FK; k++) {
            const uint32_t ek = e + k * stride;
            id[k] = ek < e1 ? ids(ek) : v;
        }
        uint32_t want = 0;
#pragma unroll
        for (int k = 0; k < FK; k++) want |= (uint32_t)(id[k] != v && test_bit(a.curr_mod, id[k])) << k;
#pragma unroll
        for (int k = 0; k < FK; k++) {
            if (!((want >> k) & 1u)) continue;
            uint32_t y[NW];
            load_chunk<LOG2M>(a.curr, id[k], c, y);
            merge_chunk<REGS>(acc, y);
        }
    }
}

// One staged item: nodes [first, first + cnt), TB lanes per node (light:
// TB = G, medium: the team), from buffer `buf`.
template <int LOG2M, int TB, int PIPE>
__device__ __forceinline__ void staged_nodes(const UnionArgs& a, uint32_t buf, int lane, uint32_t& modc,
                                             uint32_t& scanned, uint32_t& sarcs, uint32_t& vis,
                                             double& nf) {
    using Gm = Geo<LOG2M>;
    using SG = StageGeo<LOG2M>;
    constexpr int G = Gm::CHUNKS, NW = Gm::NW;
    constexpr int PB = TB / G;   // arc lanes per node
    constexpr int NPW = 32 / TB; // nodes per item
    uint32_t d0, d1, d2, d3;
    asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(d0), "=r"(d1), "=r"(d2), "=r"(d3)
                 : "r"(buf + SG::OFF_DESC));
    const uint32_t first = d0, cnt = d1 & 0x7fffffffu;
    const StagedIds ids{buf + SG::OFF_IDS, d2, d3, a.succ};
    const int slot = lane / TB, tl = lane % TB, p = tl / G, c = tl % G;
    const unsigned tmask = TB == 32 ? 0xffffffffu : (((1u << TB) - 1u) << (slot * TB));
    const unsigned lmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (slot * TB));
    const bool live = (uint32_t)slot < cnt;
    const uint32_t v = first + (uint32_t)slot;
    bool changed = false;
    if (live) {
        const uint32_t s0 = (uint32_t)lds<unsigned long long>(buf + SG::OFF_OFF + 8 * slot);
        const uint32_t s1 = (uint32_t)lds<unsigned long long>(buf + SG::OFF_OFF + 8 * slot + 8);
        uint32_t acc[NW];
        if (PB == 1 || p == 0) {
            load_chunk<LOG2M>(a.curr, v, c, acc);
        } else {
#pragma unroll
            for (int k = 0; k < NW; k++) acc[k] = 0u;
        }
        staged_gather<LOG2M, PIPE>(a, ids, v, c, s0 + p, s1, PB, acc);
        if constexpr (PB > 1) {
            __syncwarp(tmask);
#pragma unroll
            for (int off = G; off < TB; off <<= 1) {
#pragma unroll
                for (int k = 0; k < NW; k += 4) {
                    uint32_t x4[4], y4[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        x4[j] = acc[k + j];
                        y4[j] = __shfl_xor_sync(tmask, acc[k + j], off);
                    }
                    merge_chunk<16>(x4, y4);
#pragma unroll
                    for (int j = 0; j < 4; j++) acc[k + j] = x4[j];
                }
            }
        }
        if (p == 0) {
            changed = differs_from<LOG2M>(a.curr, v, c, acc);
            if constexpr (G > 1) changed = __any_sync(lmask, changed);
            store_chunk<LOG2M>(a.next, v, c, acc);
            NodeSums ns{};
            if (c == 0) {
                scanned++;
                sarcs += s1 - s0;
                ns.pre = lds<double>(buf + SG::OFF_EST + 8 * slot);
                ns.sod = a.sod ? lds<double>(buf + SG::OFF_SOD + 8 * slot) : 0.0;
                ns.harm = a.harm ? lds<double>(buf + SG::OFF_HARM + 8 * slot) : 0.0;
                ns.indeg = lds<uint32_t>(buf + SG::OFF_INDEG + 4 * slot);
            }
            finish_node<LOG2M>(a, v, c, lmask, acc, changed, ns, nf, vis);
        }
    }
    // modified bits: the item's nodes are consecutive, one bit per node slot
    const unsigned ball = __ballot_sync(0xffffffffu, changed && p == 0 && c == 0);
    if (lane == 0 && ball) {
        uint32_t bits = 0;
#pragma unroll
        for (int k = 0; k < NPW; k++) bits |= ((ball >> (k * TB)) & 1u) << k;
        const uint32_t w = first >> 5, sh = first & 31;
        atomicOr(a.next_mod + w, bits << sh);
        if (sh && (bits >> (32 - sh))) atomicOr(a.next_mod + w + 1, bits >> (32 - sh));
        modc += __popc(bits);
    }
}

// PIPE_L: counter loads in flight per lane of a light node (pipe_depth);
// IDS: successor ids staged too (else read from global memory in the loop)
template <int LOG2M, int MINB, int PIPE_L, bool IDS>
__global__ void __launch_bounds__(256, MINB) k_union_staged(const __grid_constant__ UnionArgs a) {
    using Gm = Geo<LOG2M>;
    using SG = StageGeo<LOG2M>;
    constexpr int G = Gm::CHUNKS;
    constexpr int TB_MED = team_lanes<LOG2M>();
    const int lane = threadIdx.x & 31;
    const uint32_t bufs = (uint32_t)__cvta_generic_to_shared(far_smem) + (threadIdx.x >> 5) * SG::WARP;
    const uint32_t n_work = (uint32_t)a.n_chunks;
    uint32_t modc = 0, scanned = 0, sarcs = 0, vis = 0;
    auto item = [&](uint32_t k) -> uint4 {
        return k < n_work ? __ldg(a.items + k) : make_uint4(0u, 0u, 0u, 0xffffffffu);
    };
    // pipeline: cur (staged), nxt (descriptor loaded), the cursor value of
    // the item after (lane 0, pending)
    uint32_t k_cur = 0, k_nxt = 0;
    unsigned long long atom = 0;
    if (lane == 0) k_cur = (uint32_t)atomicAdd(a.cursor, 1ull);
    k_cur = __shfl_sync(0xffffffffu, k_cur, 0);
    if (lane == 0) k_nxt = (uint32_t)atomicAdd(a.cursor, 1ull);
    k_nxt = __shfl_sync(0xffffffffu, k_nxt, 0);
    if (lane == 0) atom = atomicAdd(a.cursor, 1ull);
    uint4 nxt = item(k_nxt);
    {
        const uint4 cur = item(k_cur);
        if (k_cur < n_work) stage_item<LOG2M, IDS>(a, cur, bufs, lane);
        cp_async_commit();
    }
    for (uint32_t it = 0; k_cur < n_work; it++) {
        const uint32_t k_after = __shfl_sync(0xffffffffu, (uint32_t)atom, 0);
        if (lane == 0 && k_after < n_work) atom = atomicAdd(a.cursor, 1ull);
        const uint4 after = item(k_after);
        if (k_nxt < n_work) stage_item<LOG2M, IDS>(a, nxt, bufs + ((it + 1) & 1) * SG::BUF, lane);
        cp_async_commit();
        cp_async_wait<1>();
        __syncwarp();
        const uint32_t buf = bufs + (it & 1) * SG::BUF;
        double nf = 0.0;
        if (lds<uint32_t>(buf + SG::OFF_DESC + 4) >> 31)
            staged_nodes<LOG2M, TB_MED, 1>(a, buf, lane, modc, scanned, sarcs, vis, nf);
        else
            staged_nodes<LOG2M, G, PIPE_L>(a, buf, lane, modc, scanned, sarcs, vis, nf);
        nf = warp_sum_f64(nf);
        if (lane == 0) a.nf_items[k_cur] = nf;
        __syncwarp();
        k_cur = k_nxt;
        k_nxt = k_after;
        nxt = after;
    }
    cp_async_wait<0>();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        modc += __shfl_xor_sync(0xffffffffu, modc, off);
        scanned += __shfl_xor_sync(0xffffffffu, scanned, off);
        sarcs += __shfl_xor_sync(0xffffffffu, sarcs, off);
        vis += __shfl_xor_sync(0xffffffffu, vis, off);
    }
    if (lane == 0) {
        TilePartial* t = a.partials + a.acc_slot;
        if (modc) atomicAdd(&t->mod, (unsigned long long)modc);
        if (scanned) atomicAdd(&t->scanned, (unsigned long long)scanned);
        if (sarcs) atomicAdd(&t->sarcs, (unsigned long long)sarcs);
        if (vis) atomicAdd(&t->vis, (unsigned long long)vis);
    }
}

// item table of the staged kernel: {first, count | medium << 31, first arc, arcs}
__global__ void k_chunk_items(const uint2* __restrict__ chunks, uint64_t n_chunks,
                              const uint64_t* __restrict__ off, uint4* __restrict__ items) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n_chunks;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 d = chunks[k];
        const uint64_t a0 = off[d.x], a1 = off[d.x + (d.y & 0x7fffffffu)];
        items[k] = make_uint4(d.x, d.y, (uint32_t)a0, (uint32_t)(a1 - a0));
    }
}

// ---------------------------------------------------------------------------
// heavy nodes: one CTA per work item. An item is a whole heavy node, or, for
// a node of more than HEAVY_SPLIT arcs, one segment of HEAVY_SEG of its arcs
// (a single CTA on the largest R-MAT node, 240 K arcs at 2^24, took the whole
// heavy kernel's time). Lanes split the item's successors (G lanes per
// counter); the per-lane partial counters are merged by a butterfly of
// shuffles and then across warps through shared memory. A segment stores its
// partial counter in the node's slot and counts itself in; the last segment
// to arrive merges the node's partials (and the node's own counter) and ends
// the node as a whole node does. The maximum is order independent, so the
// result is the same whichever segment arrives last.
// ---------------------------------------------------------------------------
// chunk c of a partial counter written by another block of this launch (L2,
// not the non-coherent path)
template <int LOG2M>
__device__ __forceinline__ void load_chunk_cg(const uint8_t* base, uint64_t slot, int c,
                                              uint32_t (&w)[Geo<LOG2M>::NW]) {
    using Gm = Geo<LOG2M>;
    const uint4* p = reinterpret_cast<const uint4*>(base + slot * (uint64_t)Gm::COUNTER_BYTES +
                                                    (uint64_t)c * Gm::CHUNK_BYTES);
#pragma unroll
    for (int q = 0; q < Gm::NW / 4; q++) {
        const uint4 t = __ldcg(p + q);
        w[4 * q] = t.x;
        w[4 * q + 1] = t.y;
        w[4 * q + 2] = t.z;
        w[4 * q + 3] = t.w;
    }
}

template <int LOG2M>
__global__ void __launch_bounds__(256) k_union_heavy(UnionArgs a) {
    using Gm = Geo<LOG2M>;
    constexpr int G = Gm::CHUNKS, NW = Gm::NW, REGS = Gm::CHUNK_REGS;
    constexpr int TEAM = 256, P = TEAM / G, WARPS = TEAM / 32;
    __shared__ uint32_t red[WARPS][G][NW];
    __shared__ uint32_t s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tid = threadIdx.x;
    const int p = tid / G, c = tid % G;
    const unsigned leader_mask = G == 32 ? 0xffffffffu : ((1u << G) - 1u);
    uint32_t modc = 0, scanned = 0, sarcs = 0, vis = 0;
    for (uint64_t idx = blockIdx.x; idx < a.heavy_len; idx += gridDim.x) {
        double nf = 0.0;
        // {heavy index, segment, segments of the node, the node's first partial slot}
        const uint4 it = __ldg(a.heavy_items + idx);
        const uint32_t hi = it.x, seg = it.y, nseg = it.z, slot = it.w;
        const uint64_t v = __ldg(a.list + hi);
        const uint64_t s0 = __ldg(a.off + v), s1 = __ldg(a.off + v + 1);
        const uint64_t e0 = s0 + (uint64_t)seg * HEAVY_SEG;
        const uint64_t e1 = nseg == 1 ? s1 : min(s1, e0 + (uint64_t)HEAVY_SEG);
        const bool scan = !a.systolic || test_bit(a.mbc, v);
        if (scan) {
            uint32_t prev[NW], acc[NW];
            if (p == 0 && seg == 0) {
                load_chunk<LOG2M>(a.curr, v, c, prev);
#pragma unroll
                for (int i = 0; i < NW; i++) acc[i] = prev[i];
            } else {
#pragma unroll
                for (int i = 0; i < NW; i++) acc[i] = prev[i] = 0u;
            }
            gather_rolling<LOG2M>(a, (uint32_t)v, c, e0 + p, e1, P, !a.gather_all, acc, 0);
            __syncwarp();
#pragma unroll
            for (int off = G; off < 32; off <<= 1) {
                uint32_t y[NW];
#pragma unroll
                for (int i = 0; i < NW; i++) y[i] = __shfl_xor_sync(0xffffffffu, acc[i], off);
                merge_chunk<REGS>(acc, y);
            }
            if (lane < G) {
#pragma unroll
                for (int i = 0; i < NW; i++) red[warp][c][i] = acc[i];
            }
            __syncthreads();
            if (warp == 0 && lane < G) {
                for (int w = 1; w < WARPS; w++) {
                    uint32_t y[NW];
#pragma unroll
                    for (int i = 0; i < NW; i++) y[i] = red[w][c][i];
                    merge_chunk<REGS>(acc, y);
                }
            }
            bool last = true;
            if (nseg > 1) {
                // this segment's partial into its slot, then count it in
                if (warp == 0 && lane < G) {
                    store_chunk<LOG2M>(a.heavy_part, (uint64_t)slot + seg, c, acc);
                    __threadfence();
                }
                __syncthreads();
                if (tid == 0) {
                    const uint32_t before = atomicAdd(a.heavy_arrive + slot, 1u);
                    s_last = before == nseg - 1;
                    __threadfence();
                }
                __syncthreads();
                last = s_last != 0;
                if (last && warp == 0 && lane < G) {
                    // the node's own counter and every segment's partial
                    load_chunk<LOG2M>(a.curr, v, c, prev);
#pragma unroll
                    for (int i = 0; i < NW; i++) acc[i] = prev[i];
                    for (uint32_t k = 0; k < nseg; k++) {
                        uint32_t y[NW];
                        load_chunk_cg<LOG2M>(a.heavy_part, (uint64_t)slot + k, c, y);
                        merge_chunk<REGS>(acc, y);
                    }
                    if (lane == 0) a.heavy_arrive[slot] = 0u;  // ready for the next launch
                }
            }
            if (last && warp == 0 && lane < G) {
                NodeSums ns{};
                if (c == 0) ns = load_sums(a, (uint32_t)v);
                const bool changed = commit_node<LOG2M>(a, v, c, leader_mask, prev, acc);
                if (c == 0) {
                    scanned++;
                    sarcs += (uint32_t)(s1 - s0);
                    if (changed) {
                        atomicOr(a.next_mod + (v >> 5), 1u << (v & 31));
                        modc++;
                    }
                }
                finish_node<LOG2M>(a, (uint32_t)v, c, leader_mask, acc, changed, ns, nf, vis);
                if (c == 0) a.nf_items[a.heavy_item_base + hi] = nf;
            }
        } else if (seg == 0 && test_bit(a.curr_mod, v)) {
            if (tid < G) {
                uint32_t prev[NW];
                load_chunk<LOG2M>(a.curr, v, c, prev);
                store_chunk<LOG2M>(a.next, v, c, prev);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        modc += __shfl_xor_sync(0xffffffffu, modc, off);
        scanned += __shfl_xor_sync(0xffffffffu, scanned, off);
        sarcs += __shfl_xor_sync(0xffffffffu, sarcs, off);
        vis += __shfl_xor_sync(0xffffffffu, vis, off);
    }
    if (lane == 0) {
        // integer totals are order independent
        TilePartial* t = a.partials + a.acc_slot;
        if (modc) atomicAdd(&t->mod, (unsigned long long)modc);
        if (scanned) atomicAdd(&t->scanned, (unsigned long long)scanned);
        if (sarcs) atomicAdd(&t->sarcs, (unsigned long long)sarcs);
        if (vis) atomicAdd(&t->vis, (unsigned long long)vis);
    }
}

// ---------------------------------------------------------------------------
// init (HB:1155-1213): every counter gets add(node) (or its weighted values)
// ---------------------------------------------------------------------------
template <int LOG2M>
__device__ __forceinline__ uint32_t add_hash(uint8_t* counter, uint64_t x) {
    const uint32_t j = (uint32_t)(x & ((1ull << LOG2M) - 1ull));
    const uint64_t y = (x >> LOG2M) | (1ull << 30);
    const uint32_t cand = (uint32_t)__ffsll((long long)y);  // trailing zeros + 1
    if (counter[j] < cand) counter[j] = (uint8_t)cand;
    return cand;
}

template <int LOG2M>
__global__ void __launch_bounds__(256) k_init(InitArgs a) {
    using Gm = Geo<LOG2M>;
    bool saw31 = false;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < a.n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        uint8_t* counter = a.curr + v * (uint64_t)Gm::COUNTER_BYTES;
        if (a.weights == nullptr) {
            // the caller's id is hashed (an instance's own id in a batch)
            const uint64_t u = a.hash_id ? __ldg(a.hash_id + v) : __ldg(a.perm + v);
            const uint64_t x = a.hash_kind == 1 ? hash_jenkins(u, a.seed) : hash_sip13(u);
            const uint32_t val = add_hash<LOG2M>(counter, x);
            saw31 |= val == 31u;
            // one register holds val, the other m-1 are zero
            const uint64_t hs = (uint64_t)(Gm::M - 1) * 0x80000000ull + (uint64_t)(0x80000000u >> val);
            const uint32_t c31 = val == 31u;
            a.est[v] = estimate(signed_hsum(hs, c31, a.quirk), (uint32_t)(Gm::M - 1), a.alpha_m_m,
                                (double)Gm::M, a.ln_table);
        } else {
            // HB:1167-1174 adds random values; here value k of node v is
            // SplitMix64 step k from weight_seed ^ v * golden, hashed as usual.
            const uint64_t u = a.hash_id ? __ldg(a.hash_id + v) : __ldg(a.perm + v);
            uint64_t s = a.weight_seed ^ (u * 0x9e3779b97f4a7c15ull);
            const uint64_t w = a.weights[u];
            for (uint64_t k = 0; k < w; k++) {
                s += 0x9e3779b97f4a7c15ull;
                uint64_t z = s;
                z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
                z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
                z ^= z >> 31;
                const uint64_t x = a.hash_kind == 1 ? hash_jenkins(z, a.seed) : hash_sip13(z);
                saw31 |= add_hash<LOG2M>(counter, x) == 31u;
            }
            uint64_t hs = 0;
            uint32_t z = 0, c31 = 0;
            for (uint32_t j = 0; j < (uint32_t)Gm::M; j++) {
                const uint32_t r = counter[j];
                hs += (uint64_t)(0x80000000u >> r);
                z += r == 0u;
                c31 += r == 31u;
            }
            a.est[v] = estimate(signed_hsum(hs, c31, a.quirk), z, a.alpha_m_m, (double)Gm::M,
                                a.ln_table);
        }
    }
    // Registers only ever take values some initial register had; remember
    // whether 31 occurs so counts can skip looking for it.
    if (__syncthreads_or(saw31) && threadIdx.x == 0) atomicOr(a.any31, 1);
}

// ---------------------------------------------------------------------------
// byte registers -> the reference's packed layout (5-bit registers LSB-first,
// HLL:72-115): one thread per group of 8 registers (8 bytes in, 5 bytes out)
// ---------------------------------------------------------------------------
template <int LOG2M>
__global__ void __launch_bounds__(256) k_pack_counters(const uint8_t* __restrict__ src,
                                                       const uint32_t* __restrict__ inv,
                                                       uint8_t* __restrict__ dst, uint64_t n) {
    using Gm = Geo<LOG2M>;
    constexpr uint64_t GROUPS = Gm::M / 8;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * GROUPS;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t v = i / GROUPS, g = i % GROUPS;
        const uint64_t dv = __ldg(inv + v);
        const uint2 r = __ldg(reinterpret_cast<const uint2*>(src + dv * Gm::COUNTER_BYTES) + g);
        uint64_t bits = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            bits |= (uint64_t)((r.x >> (8 * k)) & 31u) << (5 * k);
            bits |= (uint64_t)((r.y >> (8 * k)) & 31u) << (5 * (k + 4));
        }
        uint8_t* o = dst + v * (uint64_t)Gm::PACKED_BYTES + g * 5;
#pragma unroll
        for (int k = 0; k < 5; k++) o[k] = (uint8_t)(bits >> (8 * k));
    }
}

// rows[v] += indeg[v] for v < n: transpose row lengths from in-degrees and self-loops
__global__ void k_add_indeg(unsigned long long* __restrict__ rows, const uint32_t* __restrict__ indeg,
                            uint64_t n) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x)
        rows[v] += indeg[v];
}

// fixed-order sum of doubles: block b sums its contiguous range (strided by
// thread, then a tree); a second launch sums the block results the same way
__global__ void k_sum_f64(const double* __restrict__ in, uint64_t count, double* __restrict__ out) {
    __shared__ double s[256];
    const uint64_t per = (count + gridDim.x - 1) / gridDim.x;
    const uint64_t b = (uint64_t)blockIdx.x * per, e = min(count, b + per);
    double x = 0.0;
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) x = __dadd_rn(x, in[i]);
    s[threadIdx.x] = x;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] = __dadd_rn(s[threadIdx.x], s[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = s[0];
}

// ---------------------------------------------------------------------------
// batches: per instance (a device id range) the number of modified counters
// and the neighbourhood function (sum of the cached estimates) of the
// iteration just run; one block per running instance, fixed order
// ---------------------------------------------------------------------------
constexpr int INST_THREADS = 512;
__global__ void __launch_bounds__(INST_THREADS) k_inst_stats(const uint32_t* __restrict__ next_mod,
                                                             const double* __restrict__ est,
                                                             const uint64_t* __restrict__ starts,
                                                             uint32_t count,
                                                             unsigned long long* __restrict__ mods,
                                                             double* __restrict__ nfs) {
    // One block per instance, a fixed order: thread t keeps four running
    // sums (nodes b + t + 512 (4j + k) go to sum k, so four loads are in
    // flight), adds them as (s0 + s1) + (s2 + s3), then a fixed tree. (With
    // one sum, 256 threads, the largest instance's block took most of the
    // kernel's time.) An instance whose previous iteration modified nothing
    // has stopped: its values stay.
    constexpr int T = INST_THREADS;
    __shared__ double s_nf[T];
    __shared__ unsigned long long s_mc[T];
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        if (mods[i] == 0) continue;  // uniform over the block
        __syncthreads();
        const uint64_t b = __ldg(starts + i), e = __ldg(starts + i + 1);
        double s4[4] = {0.0, 0.0, 0.0, 0.0};
        uint64_t v = b + threadIdx.x;
        for (; v + 3 * T < e; v += 4 * T) {
            double x[4];
#pragma unroll
            for (int k = 0; k < 4; k++) x[k] = __ldg(est + v + k * T);
#pragma unroll
            for (int k = 0; k < 4; k++) s4[k] = __dadd_rn(s4[k], x[k]);
        }
        // at most three nodes left for this thread
#pragma unroll
        for (int k = 0; k < 3; k++)
            if (v + k * T < e) s4[k] = __dadd_rn(s4[k], __ldg(est + v + k * T));
        const double sum = __dadd_rn(__dadd_rn(s4[0], s4[1]), __dadd_rn(s4[2], s4[3]));
        unsigned long long mc = 0;
        if (e > b) {
            const uint64_t w0 = b >> 5, w1 = (e - 1) >> 5;
            for (uint64_t w = w0 + threadIdx.x; w <= w1; w += blockDim.x) {
                uint32_t bits = __ldg(next_mod + w);
                if (w == w0) bits &= 0xffffffffu << (b & 31);
                if (w == w1 && ((e & 31) != 0)) bits &= 0xffffffffu >> (32 - (e & 31));
                mc += __popc(bits);
            }
        }
        s_nf[threadIdx.x] = sum;
        s_mc[threadIdx.x] = mc;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) {
                s_nf[threadIdx.x] = __dadd_rn(s_nf[threadIdx.x], s_nf[threadIdx.x + w]);
                s_mc[threadIdx.x] += s_mc[threadIdx.x + w];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            mods[i] = s_mc[0];
            nfs[i] = s_nf[0];
        }
    }
}

// ---------------------------------------------------------------------------
// renumbering (see "windows and chunks") and results back in caller order
// ---------------------------------------------------------------------------
__global__ void k_perm_degree(const uint64_t* __restrict__ off0, const uint32_t* __restrict__ perm,
                              uint64_t n, unsigned long long* __restrict__ deg) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (i == n) {
            deg[n] = 0;
        } else {
            const uint32_t u = __ldg(perm + i);
            deg[i] = __ldg(off0 + u + 1) - __ldg(off0 + u);
        }
    }
}

// ---------------------------------------------------------------------------
// Arc-parallel passes over a CSR: tiles of LBS_TILE consecutive arcs, every
// thread on LBS_ITEMS arcs of its tile (coalesced), the source of each arc
// found in shared memory: the nodes whose rows start inside the tile are
// written at their start positions, and a running maximum over the tile
// carries each of them to the rest of its row. tile_start[k] is the node
// holding arc k * LBS_TILE.
// ---------------------------------------------------------------------------
constexpr int LBS_THREADS = 256, LBS_ITEMS = 8, LBS_TILE = LBS_THREADS * LBS_ITEMS;

__global__ void k_tile_start(const uint64_t* __restrict__ off, uint64_t n, uint32_t* __restrict__ tile_start) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a = __ldg(off + v), b = __ldg(off + v + 1);
        for (uint64_t k = (a + LBS_TILE - 1) / LBS_TILE; k * LBS_TILE < b; k++) tile_start[k] = (uint32_t)v;
    }
}

// src[i] = source node of arc base + i, i < LBS_TILE (entries past the last
// arc are meaningless); ends with a barrier
__device__ __forceinline__ void lbs_sources(const uint64_t* __restrict__ off, uint64_t n, uint64_t m,
                                            const uint32_t* __restrict__ tile_start, uint64_t ntiles,
                                            uint64_t k, uint32_t* src, uint32_t* warp_max) {
    const uint64_t base = k * LBS_TILE;
    const uint64_t lo = tile_start[k], hi = k + 1 < ntiles ? tile_start[k + 1] : n - 1;
    for (int i = threadIdx.x; i < LBS_TILE; i += LBS_THREADS) src[i] = 0;
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(src, (uint32_t)lo);
    for (uint64_t v = lo + 1 + threadIdx.x; v <= hi; v += LBS_THREADS) {
        const uint64_t o = __ldg(off + v);
        if (o >= base && o < base + LBS_TILE && o < m) atomicMax(src + (o - base), (uint32_t)v);
    }
    __syncthreads();
    // inclusive running maximum: per thread over its LBS_ITEMS entries, then
    // across the warp and the block
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x[LBS_ITEMS], run = 0;
#pragma unroll
    for (int j = 0; j < LBS_ITEMS; j++) {
        run = max(run, src[threadIdx.x * LBS_ITEMS + j]);
        x[j] = run;
    }
    uint32_t w = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w = max(w, y);
    }
    if (lane == 31) warp_max[warp] = w;
    __syncthreads();
    uint32_t before = __shfl_up_sync(0xffffffffu, w, 1);
    if (lane == 0) before = 0;
    for (int q = 0; q < warp; q++) before = max(before, warp_max[q]);
#pragma unroll
    for (int j = 0; j < LBS_ITEMS; j++) src[threadIdx.x * LBS_ITEMS + j] = max(x[j], before);
    __syncthreads();
}

// The renumbered successors: arc e of new node i is arc e - off[i] of caller
// row perm[i], its target mapped through inv. Out-of-range targets set *bad
// (and are written as 0). With indeg: in-degrees without self-loops, and the
// self-loops into *loops and, with trows, trows[i] (zeroed by the caller).
__global__ void __launch_bounds__(LBS_THREADS) k_relabel_arcs(
    const uint64_t* __restrict__ off, uint64_t n, uint64_t m, const uint32_t* __restrict__ tile_start,
    uint64_t ntiles, const uint32_t* __restrict__ perm, const uint64_t* __restrict__ off0,
    const uint32_t* __restrict__ succ0, const uint32_t* __restrict__ inv, uint32_t* __restrict__ succ,
    uint32_t* __restrict__ indeg, unsigned long long* __restrict__ loops,
    unsigned long long* __restrict__ trows, int* __restrict__ bad) {
    __shared__ uint32_t src[LBS_TILE];
    __shared__ uint32_t warp_max[LBS_THREADS / 32];
    uint32_t nl = 0;
    for (uint64_t k = blockIdx.x; k < ntiles; k += gridDim.x) {
        lbs_sources(off, n, m, tile_start, ntiles, k, src, warp_max);
        const uint64_t base = k * LBS_TILE;
#pragma unroll 4
        for (int j = 0; j < LBS_ITEMS; j++) {
            const uint64_t e = base + j * LBS_THREADS + threadIdx.x;
            if (e >= m) break;
            const uint32_t i = src[j * LBS_THREADS + threadIdx.x];
            const uint32_t s0 = __ldg(succ0 + __ldg(off0 + __ldg(perm + i)) + (e - __ldg(off + i)));
            uint32_t t = 0;
            if (s0 < n)
                t = __ldg(inv + s0);
            else
                *bad = 1;
            succ[e] = t;
            if (indeg && s0 < n) {
                if (t == i) {
                    nl++;
                    if (trows) atomicAdd(trows + i, 1ull);
                } else {
                    atomicAdd(indeg + t, 1u);
                }
            }
        }
        __syncthreads();
    }
    if (indeg) {
        for (int o = 16; o > 0; o >>= 1) nl += __shfl_xor_sync(0xffffffffu, nl, o);
        if ((threadIdx.x & 31) == 0 && nl) atomicAdd(loops, (unsigned long long)nl);
    }
}

// transpose scatter: arc i -> s becomes s -> i at the row cursor of s
__global__ void __launch_bounds__(LBS_THREADS) k_scatter_arcs(
    const uint64_t* __restrict__ off, uint64_t n, uint64_t m, const uint32_t* __restrict__ tile_start,
    uint64_t ntiles, const uint32_t* __restrict__ succ, unsigned long long* __restrict__ cursor,
    uint32_t* __restrict__ tsucc) {
    __shared__ uint32_t src[LBS_TILE];
    __shared__ uint32_t warp_max[LBS_THREADS / 32];
    for (uint64_t k = blockIdx.x; k < ntiles; k += gridDim.x) {
        lbs_sources(off, n, m, tile_start, ntiles, k, src, warp_max);
        const uint64_t base = k * LBS_TILE;
#pragma unroll
        for (int j = 0; j < LBS_ITEMS; j++) {
            const uint64_t e = base + j * LBS_THREADS + threadIdx.x;
            if (e < m) {
                const unsigned long long pos = atomicAdd(cursor + __ldg(succ + e), 1ull);
                tsucc[pos] = src[j * LBS_THREADS + threadIdx.x];
            }
        }
        __syncthreads();
    }
}

__global__ void k_gather_f64(const double* __restrict__ src, const uint32_t* __restrict__ inv,
                             double* __restrict__ dst, uint64_t n) {
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n;
         u += (uint64_t)gridDim.x * blockDim.x)
        dst[u] = src[__ldg(inv + u)];
}

// ---------------------------------------------------------------------------
// systolic marking: every predecessor of a modified node must be checked
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_mark_preds(const uint32_t* __restrict__ next_mod,
                                                    const uint64_t* __restrict__ toff,
                                                    const uint32_t* __restrict__ tsucc,
                                                    uint32_t* __restrict__ next_mbc, uint64_t n) {
    const int lane = threadIdx.x & 31;
    const uint64_t nwords = (n + 31) >> 5;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    // a warp reads 32 bitmap words at once (one per lane), then walks the
    // in-arcs of each modified node with all lanes
    for (uint64_t base = gw * 32; base < nwords; base += nw * 32) {
        const uint64_t wi = base + lane;
        const uint32_t bits = wi < nwords ? __ldg(next_mod + wi) : 0u;
        uint32_t busy = __ballot_sync(0xffffffffu, bits != 0u);
        while (busy) {
            const int src = __ffs(busy) - 1;
            busy &= busy - 1u;
            uint32_t b = __shfl_sync(0xffffffffu, bits, src);
            while (b) {
                const uint64_t v = ((base + (uint64_t)src) << 5) + (uint64_t)(__ffs(b) - 1);
                b &= b - 1u;
                const uint64_t e0 = __ldg(toff + v), e1 = __ldg(toff + v + 1);
                for (uint64_t e = e0 + lane; e < e1; e += 32) {
                    const uint32_t p = __ldg(tsucc + e);
                    atomicOr(next_mbc + (p >> 5), 1u << (p & 31));
                }
            }
        }
    }
}

// Fixed-order reduction of the per-tile / per-block partials: stage 1 sums
// contiguous ranges (one block each), stage 2 sums the stage-1 results, so
// the neighbourhood function is reproducible run to run.
constexpr int REDUCE_BLOCKS = 256;

__global__ void k_reduce_partials(const TilePartial* __restrict__ in, uint64_t count,
                                  TilePartial* __restrict__ out) {
    __shared__ double s_nf[256];
    __shared__ unsigned long long s_v[256], s_m[256], s_s[256], s_a[256];
    const uint64_t per = (count + gridDim.x - 1) / gridDim.x;
    const uint64_t b = (uint64_t)blockIdx.x * per, e = min(count, b + per);
    double nf = 0.0;
    unsigned long long v = 0, mo = 0, sc = 0, sa = 0;
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        nf = __dadd_rn(nf, in[i].nf);
        v += in[i].vis;
        mo += in[i].mod;
        sc += in[i].scanned;
        sa += in[i].sarcs;
    }
    s_nf[threadIdx.x] = nf;
    s_v[threadIdx.x] = v;
    s_m[threadIdx.x] = mo;
    s_s[threadIdx.x] = sc;
    s_a[threadIdx.x] = sa;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s_nf[threadIdx.x] = __dadd_rn(s_nf[threadIdx.x], s_nf[threadIdx.x + w]);
            s_v[threadIdx.x] += s_v[threadIdx.x + w];
            s_m[threadIdx.x] += s_m[threadIdx.x + w];
            s_s[threadIdx.x] += s_s[threadIdx.x + w];
            s_a[threadIdx.x] += s_a[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = TilePartial{s_nf[0], s_v[0], s_m[0], s_s[0], s_a[0]};
}

// Systolic iterations: flags the windows holding a node that must be checked
// or copied; the union kernel skips the chunks of the other windows.
// bits of word i split into light and medium nodes
__device__ __forceinline__ void split_word(uint64_t i, uint32_t bits, const uint32_t* medium_bits,
                                           const uint32_t* light_bits, uint32_t& lb, uint32_t& mb) {
    lb = bits & __ldg(light_bits + i);
    mb = bits & __ldg(medium_bits + i);
}

__global__ void k_list_count(const uint32_t* __restrict__ mbc, const uint32_t* __restrict__ curr_mod,
                             const uint32_t* __restrict__ medium_bits,
                             const uint32_t* __restrict__ light_bits, uint64_t nwords,
                             unsigned long long* __restrict__ cnt) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nwords;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (i == nwords) {
            cnt[i] = 0;
            continue;
        }
        uint32_t lb, mb;
        split_word(i, __ldg(mbc + i) | __ldg(curr_mod + i), medium_bits, light_bits, lb, mb);
        cnt[i] = (unsigned long long)__popc(lb) | ((unsigned long long)__popc(mb) << 32);
    }
}

__global__ void k_list_fill(const uint32_t* __restrict__ mbc, const uint32_t* __restrict__ curr_mod,
                            const uint32_t* __restrict__ medium_bits,
                            const uint32_t* __restrict__ light_bits, uint64_t nwords,
                            const uint64_t* __restrict__ off, uint32_t* __restrict__ light_list,
                            uint32_t* __restrict__ medium_list) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nwords;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lb, mb;
        split_word(i, __ldg(mbc + i) | __ldg(curr_mod + i), medium_bits, light_bits, lb, mb);
        const uint64_t o = off[i];
        uint32_t ol = (uint32_t)o, om = (uint32_t)(o >> 32);
        const uint32_t lo = (uint32_t)(i << 5);
        while (lb) {
            light_list[ol++] = lo + (uint32_t)(__ffs(lb) - 1);
            lb &= lb - 1u;
        }
        while (mb) {
            medium_list[om++] = lo + (uint32_t)(__ffs(mb) - 1);
            mb &= mb - 1u;
        }
    }
}

__global__ void k_fill_u32(uint32_t* p, uint32_t v, uint64_t count) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// ---------------------------------------------------------------------------
// transpose on the device: in-degree count, exclusive scan, scatter
// ---------------------------------------------------------------------------
__global__ void k_count_indeg(const uint32_t* __restrict__ succ, uint64_t m,
                              unsigned long long* indeg) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(indeg + __ldg(succ + e), 1ull);
}

constexpr int SCAN_THREADS = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// exclusive scan of one tile; tile total to sums[blockIdx]
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile(const unsigned long long* __restrict__ in,
                                                          unsigned long long* out, uint64_t count,
                                                          unsigned long long* sums) {
    __shared__ unsigned long long s_warp[SCAN_THREADS / 32];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    unsigned long long v[SCAN_ITEMS], t = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        v[i] = (base + i < count) ? in[base + i] : 0ull;
        t += v[i];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = t;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < SCAN_THREADS / 32 ? s_warp[lane] : 0ull;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        if (lane < SCAN_THREADS / 32) s_warp[lane] = w;
    }
    __syncthreads();
    unsigned long long run = x - t + (warp > 0 ? s_warp[warp - 1] : 0ull);
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        if (base + i < count) out[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == SCAN_THREADS - 1) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(unsigned long long* out, uint64_t count,
                           const unsigned long long* __restrict__ offs) {
    const uint64_t i = (uint64_t)blockIdx.x * SCAN_TILE;
    const unsigned long long o = offs[blockIdx.x];
    for (uint64_t j = threadIdx.x; j < SCAN_TILE && i + j < count; j += blockDim.x) out[i + j] += o;
}

__global__ void k_transpose_scatter(const uint64_t* __restrict__ off, const uint32_t* __restrict__ succ,
                                    uint64_t n, unsigned long long* cursor, uint32_t* tsucc) {
    const int lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t v = gw; v < n; v += nw) {
        const uint64_t e0 = __ldg(off + v), e1 = __ldg(off + v + 1);
        for (uint64_t e = e0 + lane; e < e1; e += 32) {
            const uint32_t s = __ldg(succ + e);
            const unsigned long long pos = atomicAdd(cursor + s, 1ull);
            tsucc[pos] = (uint32_t)v;
        }
    }
}

// CSR validation: offsets non-decreasing, successors < n; sets *bad = 1
__global__ void k_validate(const uint64_t* __restrict__ off, const uint32_t* __restrict__ succ,
                           uint64_t n, uint64_t m, int* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint64_t v = t0; v < n; v += stride)
        if (off[v] > off[v + 1]) *bad = 1;
    for (uint64_t e = t0; e < m; e += stride)
        if (succ[e] >= n) *bad = 1;
}

// ---------------------------------------------------------------------------
// Work partition and renumbering. Segments (at most WINDOW consecutive caller
// ids, tiles[w] .. tiles[w + 1]) are renumbered in place: heavy nodes
// (out-degree > medium_max), then medium (> small_max), then light, each kind
// by decreasing out-degree, ties by id.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int node_kind(uint64_t d, uint64_t small_max, uint64_t medium_max) {
    return d > medium_max ? 0 : d > small_max ? 1 : 2;
}

// per segment: chunks of its medium and light runs, and its heavy nodes;
// index nseg gets zeros (the scans' last input); one warp per segment
__global__ void k_part_count(const uint64_t* __restrict__ off, const uint32_t* __restrict__ tiles,
                             uint64_t nseg, uint64_t small_max, uint64_t medium_max,
                             uint32_t per_light, uint32_t per_medium,
                             unsigned long long* __restrict__ seg_chunks,
                             unsigned long long* __restrict__ seg_heavy) {
    const int lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t w = gw; w <= nseg; w += nw) {
        uint32_t c[3] = {0, 0, 0};
        if (w < nseg)
            for (uint64_t v = tiles[w] + lane; v < tiles[w + 1]; v += 32)
                c[node_kind(__ldg(off + v + 1) - __ldg(off + v), small_max, medium_max)]++;
#pragma unroll
        for (int k = 0; k < 3; k++)
            for (int o = 16; o > 0; o >>= 1) c[k] += __shfl_xor_sync(0xffffffffu, c[k], o);
        if (lane == 0) {
            seg_chunks[w] = (c[1] + per_medium - 1) / per_medium + (c[2] + per_light - 1) / per_light;
            seg_heavy[w] = c[0];
        }
    }
}

// one block per segment: a bitonic sort of the segment's keys (kind, inverted
// degree, local id) in shared memory gives the new order; then perm / inv,
// the chunk table, the heavy keys (inverted degree << 32 | new id), the kind
// bitmaps (zeroed by the caller) and, for batches, the hashed ids
__global__ void __launch_bounds__(256) k_part_place(
    const uint64_t* __restrict__ off, const uint32_t* __restrict__ tiles, uint64_t nseg,
    uint64_t small_max, uint64_t medium_max, uint32_t per_light, uint32_t per_medium,
    const unsigned long long* __restrict__ chunk_at, const unsigned long long* __restrict__ heavy_at,
    const uint32_t* __restrict__ seg_base, uint32_t* __restrict__ perm, uint32_t* __restrict__ inv,
    uint2* __restrict__ chunks, unsigned long long* __restrict__ heavy_keys,
    uint32_t* __restrict__ light_bits, uint32_t* __restrict__ medium_bits,
    uint32_t* __restrict__ hash_id) {
    __shared__ unsigned long long key[WINDOW];
    __shared__ uint32_t cnt[3];
    const int lane = threadIdx.x & 31;
    for (uint64_t w = blockIdx.x; w < nseg; w += gridDim.x) {
        const uint32_t v0 = tiles[w], size = tiles[w + 1] - v0;
        uint32_t P = 32;
        while (P < size) P <<= 1;
        if (threadIdx.x < 3) cnt[threadIdx.x] = 0;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
            unsigned long long k = ~0ull;
            int kind = 3;
            if (i < size) {
                const uint64_t d = __ldg(off + v0 + i + 1) - __ldg(off + v0 + i);
                kind = node_kind(d, small_max, medium_max);
                const uint64_t inv_d = 0xffffffffull - (d < 0xffffffffull ? d : 0xffffffffull);
                k = ((unsigned long long)kind << 43) | (inv_d << 11) | i;
            }
            key[i] = k;
#pragma unroll
            for (int q = 0; q < 3; q++) {
                const uint32_t b = __ballot_sync(0xffffffffu, kind == q);
                if (lane == 0 && b) atomicAdd(&cnt[q], (uint32_t)__popc(b));
            }
        }
        __syncthreads();
        for (uint32_t s = 2; s <= P; s <<= 1)
            for (uint32_t j = s >> 1; j > 0; j >>= 1) {
                for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                    const uint32_t x = i ^ j;
                    if (x > i) {
                        const unsigned long long a = key[i], b = key[x];
                        if ((a > b) == ((i & s) == 0)) {
                            key[i] = b;
                            key[x] = a;
                        }
                    }
                }
                __syncthreads();
            }
        const uint32_t nh = cnt[0], nm = cnt[1], nl = cnt[2];
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
            const uint32_t pos = v0 + i;
            const unsigned long long k = key[i];
            const int kind = i < size ? (int)(k >> 43) : 3;
            if (i < size) {
                const uint32_t v = v0 + (uint32_t)(k & 2047);
                perm[pos] = v;
                inv[v] = pos;
                if (hash_id) hash_id[pos] = v - seg_base[w];
                if (kind == 0) heavy_keys[heavy_at[w] + i] = (((k >> 11) & 0xffffffffull) << 32) | pos;
            }
            // kind bits: lanes sharing a bitmap word are contiguous; the
            // lowest of them merges their bits into one atomic per word
            const uint32_t word = pos >> 5;
            const uint32_t grp = __match_any_sync(0xffffffffu, word);
            const uint32_t lb = __ballot_sync(0xffffffffu, kind == 2);
            const uint32_t mb = __ballot_sync(0xffffffffu, kind == 1);
            const int l0 = __ffs(grp) - 1;
            if (lane == l0) {
                const uint32_t b0 = pos & 31;
                const uint32_t lw = ((lb & grp) >> l0) << b0, mw = ((mb & grp) >> l0) << b0;
                if (lw) atomicOr(light_bits + word, lw);
                if (mw) atomicOr(medium_bits + word, mw);
            }
        }
        // chunks: the medium run, then the light run, one warp-step each
        const uint32_t cm = (nm + per_medium - 1) / per_medium, cl = (nl + per_light - 1) / per_light;
        for (uint32_t j = threadIdx.x; j < cm + cl; j += blockDim.x) {
            uint2 c;
            if (j < cm) {
                const uint32_t first = j * per_medium;
                c = make_uint2(v0 + nh + first, min(per_medium, nm - first) | 0x80000000u);
            } else {
                const uint32_t first = (j - cm) * per_light;
                c = make_uint2(v0 + nh + nm + first, min(per_light, nl - first));
            }
            chunks[chunk_at[w] + j] = c;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int num_sms(int device) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    return v > 0 ? v : 1;
}

#define HB_DISPATCH_LOG2M(l, CALL) \
    switch (l) {                   \
        case 4: return CALL(4);    \
        case 5: return CALL(5);    \
        case 6: return CALL(6);    \
        case 7: return CALL(7);    \
        case 8: return CALL(8);    \
        case 9: return CALL(9);    \
        case 10: return CALL(10);  \
        default: return (int)cudaErrorInvalidValue; \
    }

template <int LOG2M>
static int init_impl(const InitArgs& a, cudaStream_t s) {
    const int grid = (int)std::min<uint64_t>((a.n + 255) / 256 + 1, 65535);
    ++t_launches;
    k_init<LOG2M><<<grid, 256, 0, s>>>(a);
    return (int)cudaGetLastError();
}

template <int LOG2M>
static int pack_impl(const uint8_t* src, const uint32_t* inv, uint8_t* dst, uint64_t n,
                     cudaStream_t s) {
    const uint64_t items = n * (uint64_t)(Geo<LOG2M>::M / 8);
    const int grid = (int)std::min<uint64_t>((items + 255) / 256 + 1, 65535);
    ++t_launches;
    k_pack_counters<LOG2M><<<grid, 256, 0, s>>>(src, inv, dst, n);
    return (int)cudaGetLastError();
}

template <int LOG2M, bool FAR>
constexpr int far_bytes() { return FAR ? 8 * FarGeo<LOG2M>::WARP_BYTES : 0; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (EncodeTiledFn) nullptr;
        }
        return (EncodeTiledFn)p;
    }();
    return fn;
}

template <int LOG2M>
static int encode_far_impl(const uint8_t* counters, uint64_t n, CUtensorMap* out) {
    if constexpr (!FarGeo<LOG2M>::ON) {
        return 1;
    } else {
        if (n == 0 || n >= (1ull << 31) || ((uintptr_t)counters & 15u)) return 1;
        EncodeTiledFn fn = encode_tiled();
        if (!fn) return 1;
        // rows of 2^log2m bytes; a box is one row (gather4 takes four rows)
        const cuuint64_t dims[2] = {(cuuint64_t)FarGeo<LOG2M>::ROW, (cuuint64_t)n};
        const cuuint64_t strides[1] = {(cuuint64_t)FarGeo<LOG2M>::ROW};
        const cuuint32_t box[2] = {(cuuint32_t)FarGeo<LOG2M>::ROW, 1};
        const cuuint32_t elem[2] = {1, 1};
        const CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)counters, dims, strides, box,
                              elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        return r == CUDA_SUCCESS ? 0 : 1;
    }
}

int encode_far_map(int log2m, const uint8_t* counters, uint64_t n, CUtensorMap* out) {
#define CALL(L) encode_far_impl<L>(counters, n, out)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

template <int LOG2M, bool FAR, int MINB, int PIPEX = 0>
static int tile_launch(const UnionArgs& a, int grid, cudaStream_t s) {
    constexpr int smem = far_bytes<LOG2M, FAR>();
    if constexpr (smem > 48 * 1024) {
        static const cudaError_t attr = cudaFuncSetAttribute(
            k_union_window<LOG2M, FAR, MINB, PIPEX>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (attr != cudaSuccess) return (int)attr;
    }
    ++t_launches;
    k_union_window<LOG2M, FAR, MINB, PIPEX><<<grid, 256, smem, s>>>(a);
    return (int)cudaGetLastError();
}

template <int LOG2M>
static int tile_impl(const UnionArgs& a, int grid, cudaStream_t s) {
    if constexpr (FarGeo<LOG2M>::ON)
        if (a.far_tma) return tile_launch<LOG2M, true, 3>(a, grid, s);
    if (a.occ == 2) return tile_launch<LOG2M, false, 2, Geo<LOG2M>::NW >= 16 ? 2 : 0>(a, grid, s);
    if (a.occ) return tile_launch<LOG2M, false, 4>(a, grid, s);
    return tile_launch<LOG2M, false, 3>(a, grid, s);
}

template <int LOG2M, int MINB, bool IDS>
static int staged_launch(const UnionArgs& a, int grid, cudaStream_t s) {
    constexpr int smem = staged_smem_bytes<LOG2M>();
    constexpr int PIPE_L = pipe_depth<Geo<LOG2M>::NW>();
    if constexpr (smem > 48 * 1024) {
        static const cudaError_t attr = cudaFuncSetAttribute(
            k_union_staged<LOG2M, MINB, PIPE_L, IDS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (attr != cudaSuccess) return (int)attr;
    }
    ++t_launches;
    k_union_staged<LOG2M, MINB, PIPE_L, IDS><<<grid, 256, smem, s>>>(a);
    return (int)cudaGetLastError();
}

// a.staged: 1 = ids staged, 2 = ids from global memory
template <int LOG2M>
static int staged_impl(const UnionArgs& a, int grid, cudaStream_t s) {
    if (a.staged == 2) {
        if (a.occ) return staged_launch<LOG2M, 4, false>(a, grid, s);
        return staged_launch<LOG2M, 3, false>(a, grid, s);
    }
    if (a.occ) return staged_launch<LOG2M, 4, true>(a, grid, s);
    return staged_launch<LOG2M, 3, true>(a, grid, s);
}

template <int LOG2M>
static int staged_grid_impl(int device, int occ) {
    int per_sm = 1;
    constexpr int smem = staged_smem_bytes<LOG2M>();
    constexpr int PIPE_L = pipe_depth<Geo<LOG2M>::NW>();
    if (occ)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_union_staged<LOG2M, 4, PIPE_L, true>,
                                                      256, smem);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_union_staged<LOG2M, 3, PIPE_L, true>,
                                                      256, smem);
    return std::max(1, per_sm) * num_sms(device);
}

template <int LOG2M>
static int heavy_impl(const UnionArgs& a, int grid, cudaStream_t s) {
    ++t_launches;
    k_union_heavy<LOG2M><<<grid, 256, 0, s>>>(a);
    return (int)cudaGetLastError();
}




template <int LOG2M>
static int tile_grid_impl(int device, int occ) {
    int per_sm = 1;
    if (occ == 2)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, k_union_window<LOG2M, false, 2, Geo<LOG2M>::NW >= 16 ? 2 : 0>, 256, 0);
    else if (occ)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_union_window<LOG2M, false, 4>, 256, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_union_window<LOG2M, false, 3>, 256, 0);
    return std::max(1, per_sm) * num_sms(device);
}

template <int LOG2M>
static int heavy_grid_impl(int device) {
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_union_heavy<LOG2M>, 256, 0);
    return std::max(1, per_sm) * num_sms(device);
}

template <int L>
static int tile_caps(uint32_t* nodes, uint32_t* arcs) {
    *nodes = TileGeo<L>::NODES;
    *arcs = TileGeo<L>::ARCS;
    return 0;
}

int launch_init(int log2m, const InitArgs& a, void* stream) {
#define CALL(L) init_impl<L>(a, (cudaStream_t)stream)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int launch_pack_counters(int log2m, const uint8_t* src, const uint32_t* inv, uint8_t* dst,
                         uint64_t n, void* stream) {
#define CALL(L) pack_impl<L>(src, inv, dst, n, (cudaStream_t)stream)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

__global__ void k_copy_u64(const uint64_t* src, uint64_t* dst, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

int launch_copy_u64(const uint64_t* src, uint64_t* dst, uint64_t n, void* stream) {
    if (n == 0) return 0;
    const int grid = (int)std::min<uint64_t>((n + 255) / 256, 1024);
    ++t_launches;
    k_copy_u64<<<grid, 256, 0, (cudaStream_t)stream>>>(src, dst, n);
    return (int)cudaGetLastError();
}

int launch_add_indeg(unsigned long long* rows, const uint32_t* indeg, uint64_t n, void* stream) {
    if (n == 0) return 0;
    const int grid = (int)std::min<uint64_t>((n + 255) / 256, 8192);
    ++t_launches;
    k_add_indeg<<<grid, 256, 0, (cudaStream_t)stream>>>(rows, indeg, n);
    return (int)cudaGetLastError();
}

int launch_inst_stats(const uint32_t* next_mod, const double* est, const uint64_t* starts,
                      uint32_t count, unsigned long long* mods, double* nfs, void* stream) {
    const int grid = (int)std::min<uint64_t>((uint64_t)count, 16384);
    ++t_launches;
    if (grid)
        k_inst_stats<<<grid, INST_THREADS, 0, (cudaStream_t)stream>>>(next_mod, est, starts, count, mods, nfs);
    return (int)cudaGetLastError();
}

int launch_sum_f64(const double* in, uint64_t count, double* scratch, double* out, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    ++t_launches;
    k_sum_f64<<<REDUCE_BLOCKS, 256, 0, s>>>(in, count, scratch);
    ++t_launches;
    k_sum_f64<<<1, 256, 0, s>>>(scratch, REDUCE_BLOCKS, out);
    return (int)cudaGetLastError();
}

int launch_perm_degree(const uint64_t* off0, const uint32_t* perm, uint64_t n,
                       unsigned long long* deg, void* stream) {
    const int grid = (int)std::min<uint64_t>((n + 256) / 256 + 1, 8192);
    ++t_launches;
    k_perm_degree<<<grid, 256, 0, (cudaStream_t)stream>>>(off0, perm, n, deg);
    return (int)cudaGetLastError();
}

uint64_t arc_tiles(uint64_t m) { return (m + LBS_TILE - 1) / LBS_TILE; }

int launch_tile_start(const uint64_t* off, uint64_t n, uint32_t* tile_start, void* stream) {
    if (n == 0) return 0;
    const int grid = (int)std::min<uint64_t>((n + 255) / 256, 8192);
    ++t_launches;
    k_tile_start<<<grid, 256, 0, (cudaStream_t)stream>>>(off, n, tile_start);
    return (int)cudaGetLastError();
}

static int arc_grid(uint64_t ntiles) { return (int)std::min<uint64_t>(ntiles, 1u << 20); }

int launch_relabel_arcs(const uint64_t* off, uint64_t n, uint64_t m, const uint32_t* tile_start,
                        const uint32_t* perm, const uint64_t* off0, const uint32_t* succ0,
                        const uint32_t* inv, uint32_t* succ, uint32_t* indeg, unsigned long long* loops,
                        unsigned long long* trows, int* bad, void* stream) {
    const uint64_t nt = arc_tiles(m);
    if (nt == 0) return 0;
    ++t_launches;
    k_relabel_arcs<<<arc_grid(nt), LBS_THREADS, 0, (cudaStream_t)stream>>>(
        off, n, m, tile_start, nt, perm, off0, succ0, inv, succ, indeg, loops, trows, bad);
    return (int)cudaGetLastError();
}

int launch_scatter_arcs(const uint64_t* off, uint64_t n, uint64_t m, const uint32_t* tile_start,
                        const uint32_t* succ, unsigned long long* cursor, uint32_t* tsucc, void* stream) {
    const uint64_t nt = arc_tiles(m);
    if (nt == 0) return 0;
    ++t_launches;
    k_scatter_arcs<<<arc_grid(nt), LBS_THREADS, 0, (cudaStream_t)stream>>>(off, n, m, tile_start, nt,
                                                                         succ, cursor, tsucc);
    return (int)cudaGetLastError();
}

int launch_gather_f64(const double* src, const uint32_t* inv, double* dst, uint64_t n,
                      void* stream) {
    const int grid = (int)std::min<uint64_t>((n + 255) / 256 + 1, 8192);
    ++t_launches;
    k_gather_f64<<<grid, 256, 0, (cudaStream_t)stream>>>(src, inv, dst, n);
    return (int)cudaGetLastError();
}

int launch_union_tile(int log2m, const UnionArgs& a, int grid, void* stream) {
#define CALL(L) tile_impl<L>(a, grid, (cudaStream_t)stream)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int launch_union_staged(int log2m, const UnionArgs& a, int grid, void* stream) {
#define CALL(L) staged_impl<L>(a, grid, (cudaStream_t)stream)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int staged_grid(int log2m, int device, int occ) {
#define CALL(L) staged_grid_impl<L>(device, occ)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

// 3 blocks per SM (80 registers, a few spilled) measured faster than 2
// (128 registers, none spilled) on the batched workload: 266.6 against
// 313.6 ms of union time per run
int launch_union_jobs(const JobsArgs& p, int grid, void* stream) {
    if (p.njobs > (uint32_t)MAX_JOBS) return (int)cudaErrorInvalidValue;
    ++t_launches;
    k_union_jobs<3><<<grid, 256, 0, (cudaStream_t)stream>>>(p);
    return (int)cudaGetLastError();
}

int jobs_grid(int device) {
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_union_jobs<3>, 256, 0);
    return std::max(1, per_sm) * num_sms(device);
}

int launch_inst_queue(const uint32_t* inst_chunk, const unsigned long long* inst_mod, uint32_t count,
                      int all, uint32_t n_chunks, unsigned long long* cnt, uint64_t* at,
                      unsigned long long* scratch, uint64_t scratch_len, uint32_t* queue,
                      uint32_t* queue_len, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const int g1 = (int)std::min<uint64_t>((count + 256) / 256, 4096);
    ++t_launches;
    k_inst_chunk_counts<<<g1, 256, 0, s>>>(inst_chunk, inst_mod, count, all, cnt);
    int e = (int)cudaGetLastError();
    if (e) return e;
    e = launch_exclusive_scan_u64(cnt, at, count + 1, scratch, scratch_len, stream);
    if (e) return e;
    const int g2 = (int)std::min<uint64_t>((n_chunks + 255) / 256 + 1, 8192);
    ++t_launches;
    k_inst_queue<<<g2, 256, 0, s>>>(inst_chunk, inst_mod, count, all, at, n_chunks, queue, queue_len);
    return (int)cudaGetLastError();
}

int launch_inst_first_chunk(const uint2* chunks, uint64_t n_chunks, const uint64_t* start,
                            uint32_t count, uint32_t* inst_chunk, void* stream) {
    const int grid = (int)std::min<uint64_t>((count + 256) / 256, 4096);
    ++t_launches;
    k_inst_first_chunk<<<grid, 256, 0, (cudaStream_t)stream>>>(chunks, n_chunks, start, count, inst_chunk);
    return (int)cudaGetLastError();
}

int launch_chunk_items(const uint2* chunks, uint64_t n_chunks, const uint64_t* off, uint4* items,
                       void* stream) {
    if (n_chunks == 0) return 0;
    const int grid = (int)std::min<uint64_t>((n_chunks + 255) / 256, 8192);
    ++t_launches;
    k_chunk_items<<<grid, 256, 0, (cudaStream_t)stream>>>(chunks, n_chunks, off, items);
    return (int)cudaGetLastError();
}

int launch_union_heavy(int log2m, const UnionArgs& a, int grid, void* stream) {
#define CALL(L) heavy_impl<L>(a, grid, (cudaStream_t)stream)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int tile_grid(int log2m, int device, int occ) {
#define CALL(L) tile_grid_impl<L>(device, occ)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int heavy_grid(int log2m, int device) {
#define CALL(L) heavy_grid_impl<L>(device)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int tile_capacity(int log2m, uint32_t* nodes, uint32_t* arcs) {
#define CALL(L) tile_caps<L>(nodes, arcs)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

template <int L>
static int chunk_nodes_impl(uint32_t* light, uint32_t* medium) {
    constexpr int G = Geo<L>::CHUNKS;
    constexpr int TB_MED = team_lanes<L>();
    *light = 32 / G;
    *medium = 32 / TB_MED;
    return 0;
}

int chunk_nodes(int log2m, uint32_t* light, uint32_t* medium) {
#define CALL(L) chunk_nodes_impl<L>(light, medium)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int launch_work_lists(const uint32_t* mbc, const uint32_t* curr_mod, const uint32_t* medium_bits,
                      const uint32_t* light_bits, uint64_t n, unsigned long long* cnt, uint64_t* off,
                      unsigned long long* scratch, uint64_t scratch_len, uint32_t* light_list,
                      uint32_t* medium_list, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t nwords = (n + 31) / 32;
    const int grid = (int)std::min<uint64_t>((nwords + 256) / 256 + 1, 8192);
    ++t_launches;
    k_list_count<<<grid, 256, 0, s>>>(mbc, curr_mod, medium_bits, light_bits, nwords, cnt);
    int e = (int)cudaGetLastError();
    if (e) return e;
    e = launch_exclusive_scan_u64(cnt, off, nwords + 1, scratch, scratch_len, stream);
    if (e) return e;
    ++t_launches;
    k_list_fill<<<grid, 256, 0, s>>>(mbc, curr_mod, medium_bits, light_bits, nwords, off, light_list,
                                     medium_list);
    return (int)cudaGetLastError();
}


int launch_reduce_partials(const TilePartial* in, uint64_t count, TilePartial* scratch,
                           TilePartial* out, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    ++t_launches;
    k_reduce_partials<<<REDUCE_BLOCKS, 256, 0, s>>>(in, count, scratch);
    ++t_launches;
    k_reduce_partials<<<1, 256, 0, s>>>(scratch, REDUCE_BLOCKS, out);
    return (int)cudaGetLastError();
}

int launch_mark_preds(const uint32_t* next_mod, const uint64_t* toff, const uint32_t* tsucc,
                      uint32_t* next_mbc, uint64_t n, int grid, void* stream) {
    ++t_launches;
    k_mark_preds<<<grid, 256, 0, (cudaStream_t)stream>>>(next_mod, toff, tsucc, next_mbc, n);
    return (int)cudaGetLastError();
}

int launch_fill_u32(uint32_t* p, uint32_t v, uint64_t count, void* stream) {
    if (count == 0) return 0;
    const int grid = (int)std::min<uint64_t>((count + 255) / 256, 4096);
    ++t_launches;
    k_fill_u32<<<grid, 256, 0, (cudaStream_t)stream>>>(p, v, count);
    return (int)cudaGetLastError();
}

int launch_transpose_count(const uint32_t* succ, uint64_t m, unsigned long long* indeg,
                           void* stream) {
    if (m == 0) return 0;
    const int grid = (int)std::min<uint64_t>((m + 255) / 256, 8192);
    ++t_launches;
    k_count_indeg<<<grid, 256, 0, (cudaStream_t)stream>>>(succ, m, indeg);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Fixed device scratch of hb_device_transpose_noalloc: cursors for up to
// NOALLOC_MAX_NODES + 1 rows, the scan scratch for that many, one flag word.
// A file-scope device array, so using it allocates nothing; its address is
// looked up once per device.
// ---------------------------------------------------------------------------
constexpr uint64_t noalloc_scan_len(uint64_t count) {
    uint64_t total = 0;
    while (count > 1) {
        count = (count + SCAN_TILE - 1) / SCAN_TILE;
        total += 2 * count;
    }
    return total + 2;
}
constexpr uint64_t NOALLOC_WORDS =
    (NOALLOC_MAX_NODES + 1) + noalloc_scan_len(NOALLOC_MAX_NODES + 1) + 1;
static __device__ __align__(256) unsigned long long g_noalloc_scratch[NOALLOC_WORDS];

int noalloc_scratch(unsigned long long** out, uint64_t* words) {
    constexpr int MAX_DEVICES = 64;
    static std::mutex mu;
    static unsigned long long* ptrs[MAX_DEVICES] = {};
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (dev < 0 || dev >= MAX_DEVICES) return (int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!ptrs[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return (int)e;
        ptrs[dev] = (unsigned long long*)p;
    }
    *out = ptrs[dev];
    *words = NOALLOC_WORDS;
    return 0;
}

uint64_t scan_scratch_len(uint64_t count) {
    uint64_t total = 0;
    while (count > 1) {
        count = (count + SCAN_TILE - 1) / SCAN_TILE;
        total += 2 * count;  // sums + their scan
    }
    return total + 2;
}

// exclusive scan, recursive over tile sums
int launch_exclusive_scan_u64(const unsigned long long* in, uint64_t* out_, uint64_t count,
                              unsigned long long* scratch, uint64_t scratch_len, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long* out = (unsigned long long*)out_;
    if (count == 0) return 0;
    const uint64_t tiles = (count + SCAN_TILE - 1) / SCAN_TILE;
    if (2 * tiles > scratch_len) return (int)cudaErrorInvalidValue;
    unsigned long long* sums = scratch;
    unsigned long long* sums_scan = scratch + tiles;
    ++t_launches;
    k_scan_tile<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, out, count, sums);
    int e = (int)cudaGetLastError();
    if (e) return e;
    if (tiles > 1) {
        e = launch_exclusive_scan_u64(sums, (uint64_t*)sums_scan, tiles, scratch + 2 * tiles,
                                      scratch_len - 2 * tiles, stream);
        if (e) return e;
        ++t_launches;
        k_scan_add<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(out, count, sums_scan);
        e = (int)cudaGetLastError();
    }
    return e;
}

int launch_transpose_scatter(const uint64_t* off, const uint32_t* succ, uint64_t n,
                             unsigned long long* cursor, uint32_t* tsucc, void* stream) {
    if (n == 0) return 0;
    const int grid = (int)std::min<uint64_t>((n * 32 + 255) / 256, 8192);
    ++t_launches;
    k_transpose_scatter<<<grid, 256, 0, (cudaStream_t)stream>>>(off, succ, n, cursor, tsucc);
    return (int)cudaGetLastError();
}

int launch_part_count(const uint64_t* off, const uint32_t* tiles, uint64_t nseg, uint64_t small_max,
                      uint64_t medium_max, uint32_t per_light, uint32_t per_medium,
                      unsigned long long* seg_chunks, unsigned long long* seg_heavy, void* stream) {
    const int grid = (int)std::min<uint64_t>((nseg + 1 + 7) / 8, 8192);
    ++t_launches;
    k_part_count<<<grid, 256, 0, (cudaStream_t)stream>>>(off, tiles, nseg, small_max, medium_max,
                                                         per_light, per_medium, seg_chunks, seg_heavy);
    return (int)cudaGetLastError();
}

int launch_part_place(const uint64_t* off, const uint32_t* tiles, uint64_t nseg, uint64_t small_max,
                      uint64_t medium_max, uint32_t per_light, uint32_t per_medium,
                      const unsigned long long* chunk_at, const unsigned long long* heavy_at,
                      const uint32_t* seg_base, uint32_t* perm, uint32_t* inv, uint2* chunks,
                      unsigned long long* heavy_keys, uint32_t* light_bits, uint32_t* medium_bits,
                      uint32_t* hash_id, void* stream) {
    if (nseg == 0) return 0;
    const int grid = (int)std::min<uint64_t>(nseg, 65535);
    ++t_launches;
    k_part_place<<<grid, 256, 0, (cudaStream_t)stream>>>(off, tiles, nseg, small_max, medium_max,
                                                         per_light, per_medium, chunk_at, heavy_at,
                                                         seg_base, perm, inv, chunks, heavy_keys,
                                                         light_bits, medium_bits, hash_id);
    return (int)cudaGetLastError();
}

int launch_validate(const uint64_t* off, const uint32_t* succ, uint64_t n, uint64_t m, int* bad,
                    void* stream) {
    const int grid = (int)std::min<uint64_t>((std::max(n, m) + 255) / 256 + 1, 8192);
    ++t_launches;
    k_validate<<<grid, 256, 0, (cudaStream_t)stream>>>(off, succ, n, m, bad);
    return (int)cudaGetLastError();
}

}  // namespace hbk
