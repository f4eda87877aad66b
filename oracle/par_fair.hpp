// CPU oracle — test infrastructure only.
//
// One level of the reference's fair parallel breadth-first visit (webgraph-algo
// 0.1.0, src/algo/visits/breadth_first/par_fair.rs:172-212 for ParFair and
// :274-322 for ParFairPred): the frontier is cut into chunks of `granularity`
// nodes that `threads` threads take in turn (par_iter().chunks(granularity)),
// a successor is claimed by an atomic swap of its visited flag
// (visited.swap(succ, true)), and the claimed successors, each with the node
// that claimed it, form the next frontier. An arc whose target was already
// visited is a Known event. Distances are level numbers, so they do not depend
// on which thread claims a node; within a level the order of the next
// frontier is free, as in the reference.
//
// Levels smaller than PAR_MIN_LEVEL nodes run on the calling thread (starting
// threads would cost more than the level). Linked only into the oracle
// library, which tests/ and bench.py's CPU-baseline leg load.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <thread>
#include <utility>
#include <vector>

namespace hbo_par {

using Item = std::pair<uint32_t, uint32_t>;  // (node, predecessor)

constexpr uint64_t PAR_MIN_LEVEL = 4096;

// fn(t, begin, end) on `threads` threads over [0, count) cut into equal
// ranges (on the calling thread when threads <= 1 or count < min_count)
template <class F>
void parallel_ranges(unsigned threads, uint64_t count, F&& fn, uint64_t min_count = PAR_MIN_LEVEL) {
    if (threads <= 1 || count < min_count) {
        fn(0u, (uint64_t)0, count);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(threads);
    for (unsigned t = 0; t < threads; t++)
        pool.emplace_back([&, t] { fn(t, count * t / threads, count * (t + 1) / threads); });
    for (std::thread& th : pool) th.join();
}

// visited.swap(s, true) == false: the caller claimed s
inline bool claim(uint8_t* visited, uint32_t s) {
    if (__atomic_load_n(visited + s, __ATOMIC_RELAXED)) return false;
    return __atomic_exchange_n(visited + s, (uint8_t)1, __ATOMIC_RELAXED) == 0;
}

// Expands `frontier` into `next` (cleared first); returns the Known events.
inline uint64_t expand_level(const uint64_t* off, const uint32_t* succ, const std::vector<Item>& frontier,
                             uint8_t* visited, unsigned threads, std::vector<Item>& next,
                             uint64_t granularity = 64) {
    next.clear();
    std::atomic<uint64_t> cursor{0};
    auto work = [&](std::vector<Item>& out, uint64_t& known) {
        for (;;) {
            const uint64_t b = cursor.fetch_add(granularity, std::memory_order_relaxed);
            if (b >= frontier.size()) break;
            const uint64_t e = std::min<uint64_t>(b + granularity, frontier.size());
            for (uint64_t i = b; i < e; i++) {
                const uint32_t v = frontier[i].first;
                for (uint64_t a = off[v]; a < off[v + 1]; a++) {
                    const uint32_t s = succ[a];
                    if (claim(visited, s)) out.push_back({s, v});
                    else known++;
                }
            }
        }
    };
    if (threads <= 1 || frontier.size() < PAR_MIN_LEVEL) {
        uint64_t known = 0;
        work(next, known);
        return known;
    }
    std::vector<std::vector<Item>> outs(threads);
    std::vector<uint64_t> known(threads, 0);
    std::vector<std::thread> pool;
    pool.reserve(threads);
    for (unsigned t = 0; t < threads; t++) pool.emplace_back(work, std::ref(outs[t]), std::ref(known[t]));
    for (std::thread& th : pool) th.join();
    // the threads' claims, in thread order, copied in parallel
    std::vector<uint64_t> at(threads + 1, 0);
    uint64_t k = 0;
    for (unsigned t = 0; t < threads; t++) {
        at[t + 1] = at[t] + outs[t].size();
        k += known[t];
    }
    next.resize(at[threads]);
    parallel_ranges(
        threads, threads,
        [&](unsigned, uint64_t b, uint64_t e) {
            for (uint64_t t = b; t < e; t++) std::copy(outs[t].begin(), outs[t].end(), next.begin() + at[t]);
        },
        at[threads] < PAR_MIN_LEVEL ? threads + 1 : 0);
    return k;
}

}  // namespace hbo_par
