// CPU oracle of the breadth-first visits — test infrastructure only.
//
// A restatement of the reference's sequential breadth-first visit
// (webgraph-algo 0.1.0, src/algo/visits/breadth_first/seq.rs:113-224: roots
// already visited are skipped, each root is an Unknown event at distance 0,
// a FIFO queue with a level separator gives the distances) with the
// distance filter of its documentation example (seq.rs:78-80: nodes farther
// than max_distance are neither reported nor marked), and of the fair
// parallel visit with predecessors (par_fair.rs:226-323, hbo_par_visit_run)
// on host threads. Only tests/ and bench.py's CPU-baseline leg load it; the
// product never does.
#include <algorithm>
#include <cstdint>
#include <deque>
#include <utility>
#include <vector>

#include "par_fair.hpp"

struct hbo_visit {
    uint64_t n;
    const uint64_t* off;
    const uint32_t* succ;
    std::vector<uint8_t> visited;
};

extern "C" {

void* hbo_visit_create(uint64_t n, const uint64_t* off, const uint32_t* succ) {
    return new hbo_visit{n, off, succ, std::vector<uint8_t>(n, 0)};
}

void hbo_visit_destroy(void* v) { delete (hbo_visit*)v; }

// seq.rs:221-224
void hbo_visit_reset(void* vv) {
    hbo_visit* v = (hbo_visit*)vv;
    std::fill(v->visited.begin(), v->visited.end(), 0);
}

// One visit (seq.rs:113-219). The Unknown events go to nodes / preds /
// dists in event order (at most `capacity`); returns their number. Known
// events (arcs to visited nodes) are counted into *known.
uint64_t hbo_visit_run(void* vv, const uint64_t* roots, uint64_t nroots, uint64_t max_distance,
                       uint64_t* nodes, uint64_t* preds, uint64_t* dists, uint64_t capacity,
                       uint64_t* known) {
    hbo_visit* v = (hbo_visit*)vv;
    uint64_t cnt = 0, kn = 0;
    auto emit = [&](uint64_t node, uint64_t pred, uint64_t d) {
        if (cnt < capacity) {
            nodes[cnt] = node;
            preds[cnt] = pred;
            dists[cnt] = d;
        }
        cnt++;
    };
    // a separator of levels: UINT64_MAX
    std::deque<uint64_t> queue;
    for (uint64_t i = 0; i < nroots; i++) {
        const uint64_t r = roots[i];
        if (v->visited[r]) continue;
        v->visited[r] = 1;
        queue.push_back(r);
        emit(r, r, 0);
    }
    if (queue.empty()) {
        if (known) *known = 0;
        return 0;
    }
    queue.push_back(UINT64_MAX);
    uint64_t distance = 1;
    while (!queue.empty()) {
        const uint64_t node = queue.front();
        queue.pop_front();
        if (node != UINT64_MAX) {
            for (uint64_t e = v->off[node]; e < v->off[node + 1]; e++) {
                const uint64_t s = v->succ[e];
                if (!v->visited[s]) {
                    if (distance <= max_distance) {
                        v->visited[s] = 1;
                        emit(s, node, distance);
                        queue.push_back(s);
                    }
                } else {
                    kn++;
                }
            }
        } else if (!queue.empty()) {
            distance++;
            queue.push_back(UINT64_MAX);
        }
    }
    if (known) *known = kn;
    return cnt;
}

// One fair parallel visit with predecessors (ParFairPred, par_fair.rs:226-323)
// on `threads` threads, sharing the handle's visited set with hbo_visit_run.
// Roots not yet visited form level 0 (par_fair.rs:243-258); every frontier
// node is an Unknown event (node, pred, distance), level by level, in the
// order of the frontier (free within a level, as in the reference); the next
// level comes from hbo_par::expand_level. The distance filter (nodes farther
// than max_distance are neither reported nor marked) rejects every successor
// of the level at max_distance, so those arcs are not Known events either
// (par_fair.rs:295-309: Known only for arcs the filter passes). Returns the
// number of Unknown events (at most `capacity` stored).
uint64_t hbo_par_visit_run(void* vv, const uint64_t* roots, uint64_t nroots, uint64_t max_distance,
                           uint32_t threads, uint64_t* nodes, uint64_t* preds, uint64_t* dists,
                           uint64_t capacity, uint64_t* known) {
    hbo_visit* v = (hbo_visit*)vv;
    std::vector<hbo_par::Item> cur, next;
    for (uint64_t i = 0; i < nroots; i++) {
        const uint64_t r = roots[i];
        if (v->visited[r]) continue;
        v->visited[r] = 1;
        cur.push_back({(uint32_t)r, (uint32_t)r});
    }
    uint64_t cnt = 0, kn = 0;
    for (uint64_t d = 0; !cur.empty(); d++) {
        const uint64_t base = cnt, stored = cnt < capacity ? std::min<uint64_t>(cur.size(), capacity - cnt) : 0;
        hbo_par::parallel_ranges(threads, stored, [&](unsigned, uint64_t b, uint64_t e) {
            for (uint64_t i = b; i < e; i++) {
                nodes[base + i] = cur[i].first;
                preds[base + i] = cur[i].second;
                dists[base + i] = d;
            }
        });
        cnt += cur.size();
        if (d >= max_distance) break;
        kn += hbo_par::expand_level(v->off, v->succ, cur, v->visited.data(), threads, next);
        std::swap(cur, next);
    }
    if (known) *known = kn;
    return cnt;
}

// visit([root]) for each root in order (tests/test_bfv.rs:89-101): dist[node]
// for every node a visit reaches.
void hbo_visit_each(void* vv, const uint64_t* roots, uint64_t nroots, uint64_t* dist) {
    hbo_visit* v = (hbo_visit*)vv;
    std::vector<uint64_t> nodes(v->n), preds(v->n), ds(v->n);
    for (uint64_t i = 0; i < nroots; i++) {
        const uint64_t k = hbo_visit_run(vv, roots + i, 1, UINT64_MAX, nodes.data(), preds.data(),
                                         ds.data(), v->n, nullptr);
        for (uint64_t j = 0; j < k; j++) dist[nodes[j]] = ds[j];
    }
}

// The parallel visit from each root in order (tests/test_bfv.rs:251-283, the
// same test run on the parallel visits): dist[node] for every node a visit
// reaches.
void hbo_par_visit_each(void* vv, const uint64_t* roots, uint64_t nroots, uint32_t threads, uint64_t* dist) {
    hbo_visit* v = (hbo_visit*)vv;
    std::vector<uint64_t> nodes(v->n), preds(v->n), ds(v->n);
    for (uint64_t i = 0; i < nroots; i++) {
        const uint64_t k = hbo_par_visit_run(vv, roots + i, 1, UINT64_MAX, threads, nodes.data(), preds.data(),
                                             ds.data(), v->n, nullptr);
        for (uint64_t j = 0; j < k; j++) dist[nodes[j]] = ds[j];
    }
}

}  // extern "C"
