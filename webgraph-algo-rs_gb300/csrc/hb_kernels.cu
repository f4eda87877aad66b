// HyperBall kernels for sm_103a.
//
// One HyperBall iteration (reference: HyperBall::iterate / parallel_task,
// src/algo/hyperball/hyperball_impl.rs:775-1152) runs as
//   1. k_union_group  — nodes of out-degree <= small_max_degree, one lane-group
//                       (one lane per 64-register chunk) per node, walking the
//                       node's successors sequentially;
//   2. k_union_team<32>  — listed medium nodes, one warp per node;
//   3. k_union_team<256> — listed heavy nodes, one CTA per node;
//   4. k_mark_preds   — systolic iterations: predecessors of modified nodes
//                       (through the transpose) into next-must-be-checked;
//   5. k_reduce_nf    — neighbourhood-function block partials summed in a
//                       fixed order (deterministic).
// All three union kernels share the per-node epilogue (finalize_node):
// modified test, exact count, neighbourhood-function contribution, per-node
// f64 sums, next-state store. Only successors flagged in the previous
// iteration's modified bitmap are merged (HB:1038), so later iterations read
// little counter data.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "hb_internal.h"
#include "hll_device.cuh"

using namespace hbd;

namespace hbk {

constexpr int STAT_VISITED = 0, STAT_MODIFIED = 1, STAT_SCANNED = 2;

// ---------------------------------------------------------------------------
// block-level publish of per-thread statistics
// ---------------------------------------------------------------------------
__device__ __forceinline__ void publish(double nf, unsigned long long vis, unsigned long long modc,
                                        unsigned long long scanned, const UnionArgs& a) {
    __shared__ double s_nf[32];
    __shared__ unsigned long long s_v[32], s_m[32], s_s[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        nf += __shfl_xor_sync(0xffffffffu, nf, off);
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
            t += s_nf[w];
            tv += s_v[w];
            tm += s_m[w];
            ts += s_s[w];
        }
        a.nf_partials[blockIdx.x] = t;
        if (tv) atomicAdd(a.stats_out + STAT_VISITED, tv);
        if (tm) atomicAdd(a.stats_out + STAT_MODIFIED, tm);
        if (ts) atomicAdd(a.stats_out + STAT_SCANNED, ts);
    }
}

// ---------------------------------------------------------------------------
// per-node epilogue, run by the G lanes (one per chunk) of a team
// ---------------------------------------------------------------------------
template <int LOG2M>
__device__ __forceinline__ bool finalize_node(const UnionArgs& a, uint64_t v, int c,
                                              unsigned team_mask,
                                              const uint32_t (&prev)[Geo<LOG2M>::NW],
                                              const uint32_t (&acc)[Geo<LOG2M>::NW],
                                              double& nf_acc) {
    using Gm = Geo<LOG2M>;
    constexpr int G = Gm::CHUNKS, NW = Gm::NW, REGS = Gm::CHUNK_REGS;
    uint32_t diff = 0;
#pragma unroll
    for (int i = 0; i < NW; i++) diff |= prev[i] ^ acc[i];
    bool changed = diff != 0u;
    if constexpr (G > 1) changed = __any_sync(team_mask, changed);
    store_chunk<LOG2M>(a.next, v, c, acc);
    if (changed) {
        uint64_t hs = 0;
        uint32_t z = 0, c31 = 0;
        count_chunk<REGS>(acc, hs, z, c31);
        if constexpr (G > 1) {
#pragma unroll
            for (int off = 1; off < G; off <<= 1) {
                hs += __shfl_xor_sync(team_mask, hs, off);
                z += __shfl_xor_sync(team_mask, z, off);
                c31 += __shfl_xor_sync(team_mask, c31, off);
            }
        }
        if (c == 0) {
            const double post =
                estimate(signed_hsum(hs, c31, a.quirk), z, a.alpha_m_m, (double)Gm::M, a.ln_table);
            const double pre = a.est[v];
            a.est[v] = post;
            if (a.systolic) {
                nf_acc = __dadd_rn(nf_acc, -pre);
                nf_acc = __dadd_rn(nf_acc, post);
            } else {
                nf_acc = __dadd_rn(nf_acc, post);
            }
            const double delta = __dsub_rn(post, pre);
            if (delta > 0.0) {
                const double d1 = (double)(a.iter + 1);
                if (a.sod) a.sod[v] = __dadd_rn(a.sod[v], __dmul_rn(delta, d1));
                if (a.harm) a.harm[v] = __dadd_rn(a.harm[v], __ddiv_rn(delta, d1));
                for (int k = 0; k < a.ndisc; k++)
                    a.disc[k][v] = __dadd_rn(a.disc[k][v], __dmul_rn(delta, a.disc_factor[k]));
            }
        }
    } else if (!a.systolic && c == 0) {
        nf_acc = __dadd_rn(nf_acc, a.est[v]);
    }
    return changed;
}

// ---------------------------------------------------------------------------
// light nodes: one team of G lanes per node, nodes in index order
// ---------------------------------------------------------------------------
template <int LOG2M>
__global__ void __launch_bounds__(256) k_union_group(UnionArgs a) {
    using Gm = Geo<LOG2M>;
    constexpr int G = Gm::CHUNKS, NW = Gm::NW, REGS = Gm::CHUNK_REGS, NPW = 32 / G;
    const int lane = threadIdx.x & 31;
    const int c = lane % G, slot = lane / G;
    const unsigned team_mask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (slot * G));
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    double nf_acc = 0.0;
    unsigned long long vis = 0, modc = 0, scanned = 0;
    for (uint64_t wb = gw * NPW; wb < a.n; wb += nw * NPW) {
        const uint64_t v = wb + slot;
        bool scan = false, copy = false;
        uint64_t s0 = 0, s1 = 0;
        if (v < a.n) {
            s0 = __ldg(a.off + v);
            s1 = __ldg(a.off + v + 1);
            if (s1 - s0 <= a.small_max_degree) {
                if (!a.systolic || test_bit(a.mbc, v))
                    scan = true;
                else if (test_bit(a.curr_mod, v))
                    copy = true;
            }
        }
        bool changed = false;
        if (scan) {
            uint32_t prev[NW], acc[NW];
            load_chunk<LOG2M>(a.curr, v, c, prev);
#pragma unroll
            for (int i = 0; i < NW; i++) acc[i] = prev[i];
            for (uint64_t e = s0; e < s1; e++) {
                const uint32_t s = __ldg(a.succ + e);
                if (s != v && test_bit(a.curr_mod, s)) {
                    vis += (c == 0);
                    uint32_t y[NW];
                    load_chunk<LOG2M>(a.curr, s, c, y);
                    merge_chunk<REGS>(acc, y);
                }
            }
            changed = finalize_node<LOG2M>(a, v, c, team_mask, prev, acc, nf_acc);
            scanned += (c == 0);
        } else if (copy) {
            uint32_t prev[NW];
            load_chunk<LOG2M>(a.curr, v, c, prev);
            store_chunk<LOG2M>(a.next, v, c, prev);
        }
        __syncwarp();
        const unsigned bits =
            __reduce_or_sync(0xffffffffu, (changed && c == 0) ? (1u << slot) : 0u);
        if (lane == 0 && bits) {
            atomicOr(a.next_mod + (wb >> 5), bits << (wb & 31));
            modc += __popc(bits);
        }
    }
    publish(nf_acc, vis, modc, scanned, a);
}

// ---------------------------------------------------------------------------
// listed nodes: one team of TEAM threads (warp or CTA) per node
// ---------------------------------------------------------------------------
template <int LOG2M, int TEAM>
__global__ void __launch_bounds__(256) k_union_team(UnionArgs a) {
    using Gm = Geo<LOG2M>;
    constexpr int G = Gm::CHUNKS, NW = Gm::NW, REGS = Gm::CHUNK_REGS, P = TEAM / G;
    constexpr int WARPS = TEAM / 32;
    __shared__ uint32_t red[WARPS > 1 ? WARPS : 1][G][NW];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tid = TEAM == 32 ? lane : (int)threadIdx.x;
    const int p = tid / G, c = tid % G;
    uint64_t team_id, nteams;
    if (TEAM == 32) {
        team_id = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        nteams = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    } else {
        team_id = blockIdx.x;
        nteams = gridDim.x;
    }
    const unsigned leader_mask = G == 32 ? 0xffffffffu : ((1u << G) - 1u);
    double nf_acc = 0.0;
    unsigned long long vis = 0, modc = 0, scanned = 0;
    for (uint64_t idx = team_id; idx < a.list_len; idx += nteams) {
        const uint64_t v = __ldg(a.list + idx);
        const uint64_t s0 = __ldg(a.off + v), s1 = __ldg(a.off + v + 1);
        const bool scan = !a.systolic || test_bit(a.mbc, v);
        if (scan) {
            uint32_t prev[NW], acc[NW];
            if (p == 0) {
                load_chunk<LOG2M>(a.curr, v, c, prev);
#pragma unroll
                for (int i = 0; i < NW; i++) acc[i] = prev[i];
            } else {
#pragma unroll
                for (int i = 0; i < NW; i++) acc[i] = prev[i] = 0u;
            }
            for (uint64_t e = s0 + p; e < s1; e += P) {
                const uint32_t s = __ldg(a.succ + e);
                if (s != v && test_bit(a.curr_mod, s)) {
                    vis += (c == 0);
                    uint32_t y[NW];
                    load_chunk<LOG2M>(a.curr, s, c, y);
                    merge_chunk<REGS>(acc, y);
                }
            }
            __syncwarp();
#pragma unroll
            for (int off = G; off < 32; off <<= 1) {
                uint32_t y[NW];
#pragma unroll
                for (int i = 0; i < NW; i++) y[i] = __shfl_xor_sync(0xffffffffu, acc[i], off);
                merge_chunk<REGS>(acc, y);
            }
            if constexpr (WARPS > 1) {
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
            }
            if (warp == 0 && lane < G) {
                const bool changed = finalize_node<LOG2M>(a, v, c, leader_mask, prev, acc, nf_acc);
                if (c == 0) {
                    scanned++;
                    if (changed) {
                        atomicOr(a.next_mod + (v >> 5), 1u << (v & 31));
                        modc++;
                    }
                }
            }
        } else if (test_bit(a.curr_mod, v)) {
            if (tid < G) {
                uint32_t prev[NW];
                load_chunk<LOG2M>(a.curr, v, c, prev);
                store_chunk<LOG2M>(a.next, v, c, prev);
            }
        }
        if constexpr (WARPS > 1) __syncthreads();
    }
    publish(nf_acc, vis, modc, scanned, a);
}

// ---------------------------------------------------------------------------
// init (HB:1155-1213): every counter gets add(node) (or its weighted values)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t get_reg(const uint8_t* c, uint32_t j) {
    const uint32_t bit = 5u * j, byte = bit >> 3, sh = bit & 7u;
    const uint32_t w = (uint32_t)c[byte] | ((sh + 5u > 8u) ? ((uint32_t)c[byte + 1] << 8) : 0u);
    return (w >> sh) & 31u;
}
__device__ __forceinline__ void set_reg(uint8_t* c, uint32_t j, uint32_t val) {
    const uint32_t bit = 5u * j, byte = bit >> 3, sh = bit & 7u;
    const uint32_t mask = 31u << sh;
    c[byte] = (uint8_t)((c[byte] & ~mask) | ((val << sh) & 0xffu));
    if (sh + 5u > 8u)
        c[byte + 1] = (uint8_t)((c[byte + 1] & ~(mask >> 8)) | (val >> (8u - sh)));
}

template <int LOG2M>
__device__ __forceinline__ void add_hash(uint8_t* counter, uint64_t x) {
    const uint32_t j = (uint32_t)(x & ((1ull << LOG2M) - 1ull));
    const uint64_t y = (x >> LOG2M) | (1ull << 30);
    const uint32_t r = (uint32_t)(__ffsll((long long)y) - 1);
    const uint32_t cand = r + 1u;
    if (get_reg(counter, j) < cand) set_reg(counter, j, cand);
}

template <int LOG2M>
__global__ void __launch_bounds__(256) k_init(InitArgs a) {
    using Gm = Geo<LOG2M>;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < a.n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        uint8_t* counter = a.curr + v * (uint64_t)Gm::COUNTER_BYTES;
        if (a.weights == nullptr) {
            const uint64_t x = a.hash_kind == 1 ? hash_jenkins(v, a.seed) : hash_sip13(v);
            add_hash<LOG2M>(counter, x);
            const uint32_t val = (uint32_t)__ffsll((long long)((x >> LOG2M) | (1ull << 30)));
            // one register holds val, the other m-1 are zero
            const uint64_t hs = (uint64_t)(Gm::M - 1) * 0x80000000ull + (uint64_t)(0x80000000u >> val);
            const uint32_t c31 = val == 31u;
            a.est[v] = estimate(signed_hsum(hs, c31, a.quirk), (uint32_t)(Gm::M - 1), a.alpha_m_m,
                                (double)Gm::M, a.ln_table);
        } else {
            // HB:1167-1174 adds random values; here value k of node v is
            // SplitMix64 step k from weight_seed ^ v * golden, hashed as usual.
            uint64_t s = a.weight_seed ^ (v * 0x9e3779b97f4a7c15ull);
            const uint64_t w = a.weights[v];
            for (uint64_t k = 0; k < w; k++) {
                s += 0x9e3779b97f4a7c15ull;
                uint64_t z = s;
                z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
                z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
                z ^= z >> 31;
                const uint64_t x = a.hash_kind == 1 ? hash_jenkins(z, a.seed) : hash_sip13(z);
                add_hash<LOG2M>(counter, x);
            }
            uint64_t hs = 0;
            uint32_t z = 0, c31 = 0;
            for (uint32_t j = 0; j < (uint32_t)Gm::M; j++) {
                const uint32_t r = get_reg(counter, j);
                hs += (uint64_t)(0x80000000u >> r);
                z += r == 0u;
                c31 += r == 31u;
            }
            a.est[v] = estimate(signed_hsum(hs, c31, a.quirk), z, a.alpha_m_m, (double)Gm::M,
                                a.ln_table);
        }
    }
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
    for (uint64_t wi = gw; wi < nwords; wi += nw) {
        uint32_t bits = __ldg(next_mod + wi);
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1u;
            const uint64_t v = (wi << 5) + (uint64_t)b;
            const uint64_t e0 = __ldg(toff + v), e1 = __ldg(toff + v + 1);
            for (uint64_t e = e0 + lane; e < e1; e += 32) {
                const uint32_t p = __ldg(tsucc + e);
                atomicOr(next_mbc + (p >> 5), 1u << (p & 31));
            }
        }
    }
}

// fixed-order sum of block partials (one block)
__global__ void k_reduce_nf(const double* __restrict__ partials, int count, double* out) {
    __shared__ double s[256];
    double t = 0.0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) t = __dadd_rn(t, partials[i]);
    s[threadIdx.x] = t;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] = __dadd_rn(s[threadIdx.x], s[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
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
    // inclusive scan of thread totals across the block
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
// launchers
// ---------------------------------------------------------------------------
int num_sms(int device) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    return v > 0 ? v : 1;
}

template <int LOG2M>
static int init_impl(const InitArgs& a, cudaStream_t s) {
    const int grid = (int)std::min<uint64_t>((a.n + 255) / 256 + 1, 65535);
    k_init<LOG2M><<<grid, 256, 0, s>>>(a);
    return (int)cudaGetLastError();
}

template <int LOG2M>
static int group_impl(const UnionArgs& a, int grid, int block, cudaStream_t s) {
    k_union_group<LOG2M><<<grid, block, 0, s>>>(a);
    return (int)cudaGetLastError();
}

template <int LOG2M>
static int team_impl(int team, const UnionArgs& a, int grid, cudaStream_t s) {
    if (team == 32)
        k_union_team<LOG2M, 32><<<grid, 256, 0, s>>>(a);
    else
        k_union_team<LOG2M, 256><<<grid, 256, 0, s>>>(a);
    return (int)cudaGetLastError();
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

int launch_init(int log2m, const InitArgs& a, void* stream) {
#define CALL(L) init_impl<L>(a, (cudaStream_t)stream)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int launch_union_group(int log2m, const UnionArgs& a, int grid, int block, void* stream) {
#define CALL(L) group_impl<L>(a, grid, block, (cudaStream_t)stream)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int launch_union_team(int log2m, int team, const UnionArgs& a, int grid, void* stream) {
#define CALL(L) team_impl<L>(team, a, grid, (cudaStream_t)stream)
    HB_DISPATCH_LOG2M(log2m, CALL)
#undef CALL
}

int launch_mark_preds(const uint32_t* next_mod, const uint64_t* toff, const uint32_t* tsucc,
                      uint32_t* next_mbc, uint64_t n, int grid, void* stream) {
    k_mark_preds<<<grid, 256, 0, (cudaStream_t)stream>>>(next_mod, toff, tsucc, next_mbc, n);
    return (int)cudaGetLastError();
}

int launch_reduce_nf(const double* partials, int count, double* out, void* stream) {
    k_reduce_nf<<<1, 256, 0, (cudaStream_t)stream>>>(partials, count, out);
    return (int)cudaGetLastError();
}

int launch_fill_u32(uint32_t* p, uint32_t v, uint64_t count, void* stream) {
    if (count == 0) return 0;
    const int grid = (int)std::min<uint64_t>((count + 255) / 256, 4096);
    k_fill_u32<<<grid, 256, 0, (cudaStream_t)stream>>>(p, v, count);
    return (int)cudaGetLastError();
}

int launch_transpose_count(const uint32_t* succ, uint64_t m, unsigned long long* indeg,
                           void* stream) {
    if (m == 0) return 0;
    const int grid = (int)std::min<uint64_t>((m + 255) / 256, 8192);
    k_count_indeg<<<grid, 256, 0, (cudaStream_t)stream>>>(succ, m, indeg);
    return (int)cudaGetLastError();
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
    k_scan_tile<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, out, count, sums);
    int e = (int)cudaGetLastError();
    if (e) return e;
    if (tiles > 1) {
        e = launch_exclusive_scan_u64(sums, (uint64_t*)sums_scan, tiles, scratch + 2 * tiles,
                                      scratch_len - 2 * tiles, stream);
        if (e) return e;
        k_scan_add<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(out, count, sums_scan);
        e = (int)cudaGetLastError();
    }
    return e;
}

int launch_transpose_scatter(const uint64_t* off, const uint32_t* succ, uint64_t n,
                             unsigned long long* cursor, uint32_t* tsucc, void* stream) {
    if (n == 0) return 0;
    const int grid = (int)std::min<uint64_t>((n * 32 + 255) / 256, 8192);
    k_transpose_scatter<<<grid, 256, 0, (cudaStream_t)stream>>>(off, succ, n, cursor, tsucc);
    return (int)cudaGetLastError();
}

int launch_validate(const uint64_t* off, const uint32_t* succ, uint64_t n, uint64_t m, int* bad,
                    void* stream) {
    const int grid = (int)std::min<uint64_t>((std::max(n, m) + 255) / 256 + 1, 8192);
    k_validate<<<grid, 256, 0, (cudaStream_t)stream>>>(off, succ, n, m, bad);
    return (int)cudaGetLastError();
}

// Occupancy-derived grid for the union kernels.
int union_grid(int log2m, int kind, int device) {
    int per_sm = 1;
    const void* fn = nullptr;
#define FN(L)                                                                              \
    (kind == 0 ? (const void*)k_union_group<L>                                            \
               : (kind == 1 ? (const void*)k_union_team<L, 32> : (const void*)k_union_team<L, 256>))
    switch (log2m) {
        case 4: fn = FN(4); break;
        case 5: fn = FN(5); break;
        case 6: fn = FN(6); break;
        case 7: fn = FN(7); break;
        case 8: fn = FN(8); break;
        case 9: fn = FN(9); break;
        case 10: fn = FN(10); break;
        default: return 1;
    }
#undef FN
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0);
    if (per_sm < 1) per_sm = 1;
    return per_sm * num_sms(device);
}

}  // namespace hbk
