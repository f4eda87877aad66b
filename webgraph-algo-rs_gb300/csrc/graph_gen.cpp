// Deterministic synthetic graph generators and the host CSR helpers.
//
// This file depends on nothing but the C++ standard library: it is compiled
// into the product library and, unchanged, into the oracle's library, so the
// GPU path and the CPU baseline build their inputs from the same code without
// the CPU side loading the product library.
//
// CSR layout: offsets[n+1] as u64, successors[m] as u32, every successor list
// sorted ascending without duplicates.
//
// Generators use only integer arithmetic and IEEE +,-,*,/ (no libm, built with
// -ffp-contract=off), so x86 and aarch64 hosts produce identical graphs.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "graph_gen.h"

namespace hbg {

// ---------------------------------------------------------------------------
// threading helper: static partition of [0, n) over T threads.
// ---------------------------------------------------------------------------
static int host_threads() {
    unsigned t = std::thread::hardware_concurrency();
    if (const char* e = std::getenv("HB_HOST_THREADS")) t = (unsigned)std::atoi(e);
    return t == 0 ? 1 : (int)std::min(t, 256u);
}

template <class F>
static void parallel_for(uint64_t n, F f) {
    int T = host_threads();
    if (n < 4096 || T == 1) {
        f(0, n, 0);
        return;
    }
    std::vector<std::thread> ts;
    for (int t = 0; t < T; t++) {
        uint64_t a = n * t / T, b = n * (t + 1) / T;
        ts.emplace_back([=] { f(a, b, t); });
    }
    for (auto& th : ts) th.join();
}

// SplitMix64 (Steele, Lea & Flood 2014).
static inline uint64_t splitmix_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        s += 0x9e3779b97f4a7c15ull;
        return splitmix_mix(s);
    }
    // uniform in [0, bound) by multiply-high
    uint64_t below(uint64_t bound) { return (uint64_t)(((unsigned __int128)next() * bound) >> 64); }
};

// ---------------------------------------------------------------------------
// CSR helpers
// ---------------------------------------------------------------------------
// Sorts and deduplicates each row of a CSR given row buckets, drops
// self-loops, and compacts into g.
static void finalize_rows(uint64_t n, std::vector<uint64_t>& row_off, std::vector<uint32_t>& col,
                          Csr& g) {
    std::vector<uint64_t> deg(n);
    parallel_for(n, [&](uint64_t a, uint64_t b, int) {
        for (uint64_t v = a; v < b; v++) {
            uint32_t* s = col.data() + row_off[v];
            uint32_t* e = col.data() + row_off[v + 1];
            std::sort(s, e);
            uint32_t* w = s;
            for (uint32_t* p = s; p < e; p++) {
                if (*p == v) continue;
                if (w != s && w[-1] == *p) continue;
                *w++ = *p;
            }
            deg[v] = (uint64_t)(w - s);
        }
    });
    g.n = n;
    g.offsets.assign(n + 1, 0);
    for (uint64_t v = 0; v < n; v++) g.offsets[v + 1] = g.offsets[v] + deg[v];
    g.m = g.offsets[n];
    g.successors.resize(g.m);
    parallel_for(n, [&](uint64_t a, uint64_t b, int) {
        for (uint64_t v = a; v < b; v++)
            std::memcpy(g.successors.data() + g.offsets[v], col.data() + row_off[v],
                        deg[v] * sizeof(uint32_t));
    });
}

void transpose(const Csr& g, Csr& t) {
    const uint64_t n = g.n;
    t.n = n;
    t.m = g.m;
    t.offsets.assign(n + 1, 0);
    std::vector<uint64_t> cnt(n + 1, 0);
    for (uint64_t a = 0; a < g.m; a++) cnt[g.successors[a] + 1]++;
    for (uint64_t v = 0; v < n; v++) cnt[v + 1] += cnt[v];
    t.offsets = cnt;
    t.successors.resize(g.m);
    std::vector<uint64_t> cur(cnt.begin(), cnt.end() - 1);
    // Sources are visited in increasing order, so every row comes out sorted.
    for (uint64_t v = 0; v < n; v++)
        for (uint64_t a = g.offsets[v]; a < g.offsets[v + 1]; a++)
            t.successors[cur[g.successors[a]]++] = (uint32_t)v;
}

// ---------------------------------------------------------------------------
// Erdős–Rényi out-regular digraph: node v gets min(d, n-1) distinct uniform
// successors other than itself, drawn from one SplitMix64(seed) stream in node
// order, then sorted.
// ---------------------------------------------------------------------------
void gen_er(uint64_t n, uint32_t d, uint64_t seed, Csr& g) {
    SplitMix64 rng(seed);
    g.n = n;
    g.offsets.assign(n + 1, 0);
    g.successors.clear();
    const uint64_t k = n == 0 ? 0 : std::min<uint64_t>(d, n - 1);
    g.successors.reserve(n * k);
    std::vector<uint32_t> row;
    for (uint64_t v = 0; v < n; v++) {
        row.clear();
        while (row.size() < k) {
            uint32_t s = (uint32_t)rng.below(n);
            if (s == v) continue;
            if (std::find(row.begin(), row.end(), s) != row.end()) continue;
            row.push_back(s);
        }
        std::sort(row.begin(), row.end());
        g.successors.insert(g.successors.end(), row.begin(), row.end());
        g.offsets[v + 1] = g.successors.size();
    }
    g.m = g.successors.size();
}

// ---------------------------------------------------------------------------
// R-MAT (Chakrabarti, Zhan & Faloutsos 2004): 2^scale nodes, edges_per_node *
// 2^scale arcs drawn by recursive quadrant choice with probabilities
// (a, b, c, 1-a-b-c); arc i uses the stream SplitMix64(seed ^ mix(i / 2^16)).
// Duplicates and self-loops are removed.
// ---------------------------------------------------------------------------
void gen_rmat(int scale, uint64_t edges_per_node, double a, double b, double c, uint64_t seed,
              Csr& g) {
    const uint64_t n = 1ull << scale;
    const uint64_t m0 = edges_per_node * n;
    // 32-bit thresholds for the quadrant choice
    const uint64_t TA = (uint64_t)(a * 4294967296.0);
    const uint64_t TB = (uint64_t)((a + b) * 4294967296.0);
    const uint64_t TC = (uint64_t)((a + b + c) * 4294967296.0);
    std::vector<uint64_t> arcs(m0);
    const uint64_t BLK = 1ull << 16;
    const uint64_t nblk = (m0 + BLK - 1) / BLK;
    parallel_for(nblk, [&](uint64_t b0, uint64_t b1, int) {
        for (uint64_t blk = b0; blk < b1; blk++) {
            SplitMix64 rng(seed ^ splitmix_mix(blk + 0x5851f42d4c957f2dull));
            uint64_t e = std::min(m0, (blk + 1) * BLK);
            for (uint64_t i = blk * BLK; i < e; i++) {
                uint64_t src = 0, dst = 0;
                uint64_t r = 0;
                for (int l = 0; l < scale; l++) {
                    if ((l & 1) == 0) r = rng.next();
                    uint64_t x = (l & 1) ? (r >> 32) : (r & 0xffffffffull);
                    src <<= 1;
                    dst <<= 1;
                    if (x < TA) {
                    } else if (x < TB) {
                        dst |= 1;
                    } else if (x < TC) {
                        src |= 1;
                    } else {
                        src |= 1;
                        dst |= 1;
                    }
                }
                arcs[i] = (src << 32) | dst;
            }
        }
    });
    // bucket by source
    std::vector<uint64_t> row_off(n + 1, 0);
    {
        std::vector<std::atomic<uint64_t>> cnt(n);
        for (auto& x : cnt) x.store(0, std::memory_order_relaxed);
        parallel_for(m0, [&](uint64_t i0, uint64_t i1, int) {
            for (uint64_t i = i0; i < i1; i++) cnt[arcs[i] >> 32].fetch_add(1, std::memory_order_relaxed);
        });
        for (uint64_t v = 0; v < n; v++) row_off[v + 1] = row_off[v] + cnt[v].load();
    }
    std::vector<uint32_t> col(m0);
    {
        std::vector<std::atomic<uint64_t>> cur(n);
        for (uint64_t v = 0; v < n; v++) cur[v].store(row_off[v], std::memory_order_relaxed);
        parallel_for(m0, [&](uint64_t i0, uint64_t i1, int) {
            for (uint64_t i = i0; i < i1; i++) {
                uint64_t p = cur[arcs[i] >> 32].fetch_add(1, std::memory_order_relaxed);
                col[p] = (uint32_t)(arcs[i] & 0xffffffffull);
            }
        });
    }
    std::vector<uint64_t>().swap(arcs);
    finalize_rows(n, row_off, col, g);
}

// ---------------------------------------------------------------------------
// Web-like graph: out-degree k in [1, cap] with P(k) proportional to
// (k + shift)^-exponent (a Zipf–Mandelbrot law; shift 1.266 with exponent 2.1
// and cap 1e5 gives mean 12.00); each of the k draws is, with probability 4/5,
// uniform in [v-window, v+window] (wrapped mod n: URL-order locality) and
// otherwise uniform over all nodes. Node v draws from
// SplitMix64(mix(seed * 2^32 + v)). Rows are sorted, deduplicated and
// self-loop free, so final degrees are at most k.
// ---------------------------------------------------------------------------
// x^(1/10) for x >= 1 by Newton's method with basic IEEE operations only.
static double root10(double x) {
    double y = 1.0 + (x - 1.0) / 10.0;
    for (int i = 0; i < 200; i++) {
        double y2 = y * y, y4 = y2 * y2, y8 = y4 * y4, y9 = y8 * y;
        double ny = (9.0 * y + x / y9) / 10.0;
        if (!(ny < y)) break;
        y = ny;
    }
    return y;
}

static std::vector<uint64_t> zipf_thresholds(uint64_t cap, double exponent_tenths, double shift) {
    // exponent is 2.1 = 2 + 1/10: w(k) = 1 / ((k+s)^2 * (k+s)^(1/10))
    (void)exponent_tenths;
    std::vector<double> cum(cap + 1, 0.0);
    for (uint64_t k = 1; k <= cap; k++) {
        double x = (double)k + shift;
        double w = 1.0 / (x * x * root10(x));
        cum[k] = cum[k - 1] + w;
    }
    std::vector<uint64_t> t(cap + 1, 0);
    const double total = cum[cap];
    for (uint64_t k = 1; k <= cap; k++) {
        double f = cum[k] / total * 18446744073709551616.0;
        t[k] = f >= 18446744073709551616.0 ? UINT64_MAX : (uint64_t)f;
    }
    t[cap] = UINT64_MAX;
    return t;
}

void gen_weblike(uint64_t n, uint64_t cap, double shift, uint64_t window, uint64_t seed, Csr& g) {
    const std::vector<uint64_t> thr = zipf_thresholds(cap, 2.1, shift);
    auto degree_of = [&](SplitMix64& rng) -> uint64_t {
        uint64_t r = rng.next();
        // smallest k >= 1 with thr[k] > r
        auto it = std::upper_bound(thr.begin() + 1, thr.end(), r);
        uint64_t k = (uint64_t)(it - thr.begin());
        return k > cap ? cap : k;
    };
    auto gen_row = [&](uint64_t v, std::vector<uint32_t>& row) {
        SplitMix64 rng(splitmix_mix((seed << 32) + v));
        uint64_t k = degree_of(rng);
        row.clear();
        for (uint64_t j = 0; j < k; j++) {
            uint64_t r = rng.next();
            uint64_t s;
            if ((((unsigned __int128)r * 5) >> 64) != 0) {
                uint64_t off = rng.below(2 * window + 1);
                s = (v + n - (window % n) + off % n) % n;
            } else {
                s = rng.below(n);
            }
            if (s != v) row.push_back((uint32_t)s);
        }
        std::sort(row.begin(), row.end());
        row.erase(std::unique(row.begin(), row.end()), row.end());
    };
    std::vector<uint64_t> deg(n);
    parallel_for(n, [&](uint64_t a, uint64_t b, int) {
        std::vector<uint32_t> row;
        for (uint64_t v = a; v < b; v++) {
            gen_row(v, row);
            deg[v] = row.size();
        }
    });
    g.n = n;
    g.offsets.assign(n + 1, 0);
    for (uint64_t v = 0; v < n; v++) g.offsets[v + 1] = g.offsets[v] + deg[v];
    g.m = g.offsets[n];
    g.successors.resize(g.m);
    parallel_for(n, [&](uint64_t a, uint64_t b, int) {
        std::vector<uint32_t> row;
        for (uint64_t v = a; v < b; v++) {
            gen_row(v, row);
            std::memcpy(g.successors.data() + g.offsets[v], row.data(), row.size() * 4);
        }
    });
}

}  // namespace hbg
