// CPU oracle of ExactSumSweep — test infrastructure only.
//
// A sequential restatement of the reference's ExactSumSweep (webgraph-algo
// 0.1.0, src/algo/exact_sum_sweep/: computer.rs, scc_graph.rs,
// output_level.rs) with its strongly connected components (src/algo/sccs/
// tarjan.rs for directed graphs, symm_seq.rs for symmetric ones) and its
// tie rules (src/utils/argmax.rs, argmin.rs). Every eccentricity, the radius
// and the diameter are exact values, so the brute-force eccentricities
// (hbo_eccentricities, one breadth-first visit per node) pin them. Where the
// reference's parallel visits leave a choice open (which of several nodes
// reaching a new minimal radius in one step becomes the radial vertex),
// this restatement takes the smallest node index; the device implementation
// follows the same rule. Only tests/ and bench.py's CPU-baseline leg load
// it; the product never does.
#include <algorithm>
#include <cstdint>
#include <deque>
#include <vector>

#include "par_fair.hpp"

namespace {

using u64 = uint64_t;
constexpr u64 NONE = ~0ull;

struct Csr {
    u64 n;
    const u64* off;
    const uint32_t* succ;
    u64 deg(u64 v) const { return off[v + 1] - off[v]; }
};

// Breadth-first distances from `root` (NONE: not reached); the visit of
// visits/breadth_first (each node once, distance = level).
void bfs(const Csr& g, u64 root, std::vector<u64>& dist) {
    std::deque<u64> q;
    dist[root] = 0;
    q.push_back(root);
    while (!q.empty()) {
        const u64 v = q.front();
        q.pop_front();
        for (u64 e = g.off[v]; e < g.off[v + 1]; e++) {
            const u64 s = g.succ[e];
            if (dist[s] != NONE) continue;
            dist[s] = dist[v] + 1;
            q.push_back(s);
        }
    }
}

// The same distances from the reference's fair parallel visit on `threads`
// threads (par_fair.rs:274-322, one level at a time; see par_fair.hpp), the
// visit the reference's ExactSumSweep runs.
void par_bfs(const Csr& g, u64 root, std::vector<u64>& dist, unsigned threads) {
    std::vector<uint8_t> visited(g.n, 0);
    std::vector<hbo_par::Item> cur{{(uint32_t)root, (uint32_t)root}}, next;
    visited[root] = 1;
    for (u64 d = 0; !cur.empty(); d++) {
        hbo_par::parallel_ranges(threads, cur.size(), [&](unsigned, u64 b, u64 e) {
            for (u64 i = b; i < e; i++) dist[cur[i].first] = d;
        });
        hbo_par::expand_level(g.off, g.succ, cur, visited.data(), threads, next);
        std::swap(cur, next);
    }
}

// tarjan.rs:14-121: components numbered as they are emitted (reverse
// topological order), roots tried in node order, successors in arc order.
// Iterative; the numbering is that of the recursive algorithm.
std::vector<u64> tarjan(const Csr& g, u64& ncomp) {
    const u64 n = g.n;
    std::vector<u64> index(n, NONE), low(n, 0), comp(n, NONE);
    std::vector<uint8_t> on_stack(n, 0);
    std::vector<u64> stack;
    std::vector<std::pair<u64, u64>> call;  // (node, next arc)
    u64 counter = 0;
    ncomp = 0;
    for (u64 r = 0; r < n; r++) {
        if (index[r] != NONE) continue;
        call.push_back({r, g.off[r]});
        index[r] = low[r] = counter++;
        stack.push_back(r);
        on_stack[r] = 1;
        while (!call.empty()) {
            u64 v = call.back().first;
            u64& e = call.back().second;
            if (e < g.off[v + 1]) {
                const u64 w = g.succ[e++];
                if (index[w] == NONE) {
                    index[w] = low[w] = counter++;
                    stack.push_back(w);
                    on_stack[w] = 1;
                    call.push_back({w, g.off[w]});
                } else if (on_stack[w]) {
                    low[v] = std::min(low[v], index[w]);
                }
                continue;
            }
            if (low[v] == index[v]) {
                for (;;) {
                    const u64 w = stack.back();
                    stack.pop_back();
                    on_stack[w] = 0;
                    comp[w] = ncomp;
                    if (w == v) break;
                }
                ncomp++;
            }
            call.pop_back();
            if (!call.empty()) {
                const u64 p = call.back().first;
                low[p] = std::min(low[p], low[v]);
            }
        }
    }
    return comp;
}

// symm_seq.rs:15-49: connected components of a symmetric graph, numbered in
// the order of their smallest node
std::vector<u64> symm_components(const Csr& g, u64& ncomp) {
    std::vector<u64> comp(g.n, NONE);
    ncomp = 0;
    std::vector<u64> st;
    for (u64 r = 0; r < g.n; r++) {
        if (comp[r] != NONE) continue;
        comp[r] = ncomp;
        st.push_back(r);
        while (!st.empty()) {
            const u64 v = st.back();
            st.pop_back();
            for (u64 e = g.off[v]; e < g.off[v + 1]; e++)
                if (comp[g.succ[e]] == NONE) {
                    comp[g.succ[e]] = ncomp;
                    st.push_back(g.succ[e]);
                }
        }
        ncomp++;
    }
    return comp;
}

struct Conn {
    u64 target, start, end;
};

// scc_graph.rs:118-227: for every component in index order, its children in
// order of first appearance (nodes of the component in increasing order,
// successors in arc order), each with the arc of largest
// indeg(start) + outdeg(end) (the first such arc on ties).
void scc_dag(const Csr& g, const Csr& t, const std::vector<u64>& comp, u64 ncomp,
             std::vector<u64>& seg, std::vector<Conn>& conns) {
    std::vector<std::vector<u64>> members(ncomp);
    for (u64 v = 0; v < g.n; v++) members[comp[v]].push_back(v);
    std::vector<u64> best_start(ncomp, NONE), best_end(ncomp, NONE);
    std::vector<u64> children;
    auto value = [&](u64 s, u64 e) { return t.deg(s) + g.deg(e); };
    seg.assign(ncomp, 0);
    conns.clear();
    for (u64 c = 0; c < ncomp; c++) {
        for (u64 v : members[c])
            for (u64 e = g.off[v]; e < g.off[v + 1]; e++) {
                const u64 s = g.succ[e];
                const u64 sc = comp[s];
                if (sc == c) continue;
                if (best_start[sc] == NONE) {
                    best_start[sc] = v;
                    best_end[sc] = s;
                    children.push_back(sc);
                }
                if (value(v, s) > value(best_start[sc], best_end[sc])) {
                    best_start[sc] = v;
                    best_end[sc] = s;
                }
            }
        seg[c] = conns.size();
        for (u64 ch : children) {
            conns.push_back({ch, best_start[ch], best_end[ch]});
            best_start[ch] = NONE;
        }
        children.clear();
    }
}

// argmax.rs: the largest (value, tie) among the kept indices, the smallest
// index among equals; NONE when nothing is kept
template <class V, class T, class F>
u64 argmax_kept(u64 n, const V& val, const T& tie, F keep) {
    u64 best = NONE;
    for (u64 i = 0; i < n; i++) {
        if (!keep(i)) continue;
        if (best == NONE || val[i] > val[best] || (val[i] == val[best] && tie[i] > tie[best])) best = i;
    }
    return best;
}

// argmin.rs: the smallest (value, tie) among the kept indices, the smallest
// index among equals; NONE when nothing is kept
template <class V, class T, class F>
u64 argmin_kept(u64 n, const V& val, const T& tie, F keep) {
    u64 best = NONE;
    for (u64 i = 0; i < n; i++) {
        if (!keep(i)) continue;
        if (best == NONE || val[i] < val[best] || (val[i] == val[best] && tie[i] < tie[best])) best = i;
    }
    return best;
}

enum Output { ALL = 0, ALL_FORWARD = 1, RADIUS_DIAMETER = 2, DIAMETER = 3, RADIUS = 4 };

struct Computer {
    Csr g, t;
    Output out;
    u64 n;
    std::vector<uint8_t> radial;
    bool compute_radial;
    u64 diameter_low = 0, radius_high = NONE, diameter_vertex = 0, radius_vertex = 0, iterations = 0;
    std::vector<u64> forward_low, forward_high, backward_low, backward_high, forward_tot, backward_tot;
    u64 radius_it = NONE, diameter_it = NONE, forward_it = NONE, all_it = NONE;
    std::vector<u64> comp;
    u64 ncomp = 0;
    std::vector<u64> seg;
    std::vector<Conn> conns;
    unsigned threads = 1;  // > 1: the visits run level by level on this many threads

    void visit(const Csr& h, u64 root, std::vector<u64>& d) const {
        if (threads > 1) par_bfs(h, root, d, threads);
        else bfs(h, root, d);
    }

    bool inc_f(u64 i) const { return forward_low[i] != forward_high[i]; }
    bool inc_b(u64 i) const { return backward_low[i] != backward_high[i]; }

    template <class F>
    u64 argmax_filtered(const std::vector<u64>& val, const std::vector<u64>& tie, F keep) const {
        return argmax_kept(n, val, tie, keep);
    }
    template <class F>
    u64 argmin_filtered(const std::vector<u64>& val, const std::vector<u64>& tie, F keep) const {
        return argmin_kept(n, val, tie, keep);
    }

    // computer.rs:487-542
    void compute_radial_vertices() {
        std::vector<u64> sizes(ncomp, 0);
        for (u64 v = 0; v < n; v++) sizes[comp[v]]++;
        u64 big = 0;  // argmax: the first largest
        for (u64 c = 1; c < ncomp; c++)
            if (sizes[c] > sizes[big]) big = c;
        u64 v = n;
        while (v > 0) {
            v--;
            if (comp[v] == big) break;
        }
        std::vector<u64> d(n, NONE);
        visit(t, v, d);
        for (u64 i = 0; i < n; i++)
            if (d[i] != NONE) radial[i] = 1;
    }

    // computer.rs:644-693
    void forward_step(u64 start) {
        std::vector<u64> d(n, NONE);
        visit(g, start, d);
        u64 ecc = 0;
        for (u64 v = 0; v < n; v++) {
            if (d[v] == NONE) continue;
            ecc = std::max(ecc, d[v]);
            backward_tot[v] += d[v];
            if (backward_low[v] != backward_high[v] && backward_low[v] < d[v]) backward_low[v] = d[v];
        }
        forward_low[start] = forward_high[start] = ecc;
        if (diameter_low < ecc) {
            diameter_low = ecc;
            diameter_vertex = start;
        }
        if (radial[start] && radius_high > ecc) {
            radius_high = ecc;
            radius_vertex = start;
        }
    }

    // computer.rs:572-642 (a new minimal radius: the smallest such node)
    void backward_step(u64 start) {
        std::vector<u64> d(n, NONE);
        visit(t, start, d);
        u64 ecc = 0, r = radius_high, rv = radius_vertex;
        for (u64 v = 0; v < n; v++) {
            if (d[v] == NONE) continue;
            ecc = std::max(ecc, d[v]);
            forward_tot[v] += d[v];
            if (forward_low[v] != forward_high[v] && forward_low[v] < d[v]) {
                forward_low[v] = d[v];
                if (d[v] == forward_high[v] && radial[v] && d[v] < r) {
                    r = d[v];
                    rv = v;
                }
            }
        }
        backward_low[start] = backward_high[start] = ecc;
        radius_high = r;
        radius_vertex = rv;
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

    // computer.rs:418-475: per component, the smallest (score, tot, node)
    std::vector<u64> best_pivot() const {
        std::vector<u64> pivot(ncomp, NONE);
        auto score = [&](u64 v) {
            return backward_low[v] + forward_low[v] + (inc_f(v) ? 0 : n) + (inc_b(v) ? 0 : n);
        };
        for (u64 v = n; v-- > 0;) {
            const u64 c = comp[v];
            const u64 p = pivot[c];
            if (p == NONE) {
                pivot[c] = v;
                continue;
            }
            const u64 cur = score(v), best = score(p);
            if (cur < best || (cur == best && forward_tot[v] + backward_tot[v] <= forward_tot[p] + backward_tot[p]))
                pivot[c] = v;
        }
        return pivot;
    }

    // computer.rs:745-809: distances from each component's pivot inside
    // the component, and each pivot's eccentricity there
    // (the components are disjoint, so one visit from all pivots at once,
    // never leaving a node's component, gives every component's distances)
    void dist_pivot(const Csr& h, const std::vector<u64>& pivot, std::vector<u64>& dist,
                    std::vector<u64>& ecc) const {
        dist.assign(n, NONE);
        ecc.assign(ncomp, 0);
        std::deque<u64> q;
        for (u64 c = 0; c < ncomp; c++) {
            dist[pivot[c]] = 0;
            q.push_back(pivot[c]);
        }
        while (!q.empty()) {
            const u64 v = q.front();
            q.pop_front();
            ecc[comp[v]] = std::max(ecc[comp[v]], dist[v]);
            for (u64 e = h.off[v]; e < h.off[v + 1]; e++) {
                const u64 s = h.succ[e];
                if (dist[s] != NONE || comp[s] != comp[v]) continue;
                dist[s] = dist[v] + 1;
                q.push_back(s);
            }
        }
    }

    // computer.rs:818-921
    void all_cc_upper_bound() {
        const std::vector<u64> pivot = best_pivot();
        std::vector<u64> df, ef, db, eb;
        dist_pivot(g, pivot, df, ef);
        dist_pivot(t, pivot, db, eb);
        for (u64 c = 0; c < ncomp; c++) {
            const u64 p = pivot[c];
            const u64 e1 = c + 1 < ncomp ? seg[c + 1] : conns.size();
            for (u64 k = seg[c]; k < e1; k++) {
                const Conn& x = conns[k];
                ef[c] = std::max(ef[c], df[x.start] + 1 + db[x.end] + ef[x.target]);
                if (ef[c] >= forward_high[p]) {
                    ef[c] = forward_high[p];
                    break;
                }
            }
        }
        for (u64 c = ncomp; c-- > 0;) {
            const u64 e1 = c + 1 < ncomp ? seg[c + 1] : conns.size();
            for (u64 k = seg[c]; k < e1; k++) {
                const Conn& x = conns[k];
                eb[x.target] = std::max(eb[x.target], df[x.start] + 1 + db[x.end] + eb[c]);
                if (eb[x.target] >= backward_high[pivot[x.target]]) eb[x.target] = backward_high[pivot[x.target]];
            }
        }
        u64 r = radius_high, rv = radius_vertex;
        for (u64 v = 0; v < n; v++) {
            u64 fh = forward_high[v];
            const u64 pv = db[v] + ef[comp[v]];
            if (pv < fh) {
                forward_high[v] = pv;
                fh = pv;
            }
            if (fh == forward_low[v] && radial[v] && fh < r) {
                r = fh;
                rv = v;
            }
            backward_high[v] = std::min(backward_high[v], df[v] + eb[comp[v]]);
        }
        radius_high = r;
        radius_vertex = rv;
        iterations += 3;
    }

    // computer.rs:929-1015
    u64 missing() {
        u64 mr = 0, mdf = 0, mdb = 0, maf = 0, mab = 0;
        for (u64 v = 0; v < n; v++) {
            if (inc_f(v)) {
                maf++;
                if (forward_high[v] > diameter_low) mdf++;
                if (radial[v] && forward_low[v] < radius_high) mr++;
            }
            if (inc_b(v)) {
                mab++;
                if (backward_high[v] > diameter_low) mdb++;
            }
        }
        if (mr == 0 && radius_it == NONE) radius_it = iterations;
        if ((mdf == 0 || mdb == 0) && diameter_it == NONE) diameter_it = iterations;
        if (maf == 0 && forward_it == NONE) forward_it = iterations;
        if (maf == 0 && mab == 0) all_it = iterations;
        switch (out) {
            case RADIUS: return mr;
            case DIAMETER: return std::min(mdf, mdb);
            case RADIUS_DIAMETER: return mr + std::min(mdf, mdb);
            case ALL_FORWARD: return maf;
            default: return mab + maf;
        }
    }

    // computer.rs:282-418
    void compute() {
        if (n == 0) return;
        if (compute_radial) compute_radial_vertices();
        u64 maxv = 0;  // the largest out-degree, the smallest node among equals
        for (u64 v = 1; v < n; v++)
            if (g.deg(v) > g.deg(maxv)) maxv = v;
        // the SumSweep heuristic (computer.rs:250-280), six visits
        step(maxv, true);
        for (int i = 2; i <= 6; i++) {
            if (i % 2 == 0)
                step(argmax_filtered(backward_tot, backward_low, [&](u64 k) { return inc_b(k); }), false);
            else
                step(argmax_filtered(forward_tot, forward_low, [&](u64 k) { return inc_f(k); }), true);
        }
        double points[5];
        for (double& p : points) p = (double)n;
        u64 miss = missing();
        while (miss > 0) {
            int s = 0;  // argmax: the first largest
            for (int i = 1; i < 5; i++)
                if (points[i] > points[s]) s = i;
            switch (s) {
                case 0: all_cc_upper_bound(); break;
                case 1:
                    step(argmax_filtered(forward_high, forward_tot, [&](u64 k) { return inc_f(k); }), true);
                    break;
                case 2:
                    step(argmin_filtered(forward_low, forward_tot, [&](u64 k) { return radial[k] != 0; }), true);
                    break;
                case 3:
                    step(argmax_filtered(backward_high, backward_tot, [&](u64 k) { return inc_b(k); }), false);
                    break;
                default:
                    step(argmax_filtered(backward_tot, backward_high, [&](u64 k) { return inc_b(k); }), false);
                    break;
            }
            const u64 old = miss;
            miss = missing();
            points[s] = (double)(old - miss);
            for (int i = 0; i < 5; i++)
                if (i != s && points[i] >= 0.0) points[i] += 2.0 / (double)iterations;
        }
    }
};

}  // namespace

extern "C" {

// hbo_sum_sweep_par (visits on `threads` threads) and hbo_sum_sweep (on the
// calling thread; the results do not depend on it):
// ExactSumSweep of a directed graph (toff/tsucc: its transpose) or, with
// toff == NULL, of a symmetric graph. level: 0 All, 1 AllForward,
// 2 RadiusDiameter, 3 Diameter, 4 Radius (output_level.rs). radial: n bytes
// or NULL (the nodes that reach the largest strongly connected component).
// res: diameter, radius, diametral vertex, radial vertex, and the radius,
// diameter, forward and all iterations (~0: not computed). Eccentricities go
// to fecc / becc when given (All: forward_low and backward_high; AllForward
// and symmetric All: forward_low). Returns 0, or -1 when the level's outputs
// were not all computed (output_level.rs asserts; an empty graph).
int hbo_sum_sweep_par(uint64_t n, const uint64_t* off, const uint32_t* succ, const uint64_t* toff,
                      const uint32_t* tsucc, int level, const uint8_t* radial, uint64_t* fecc,
                      uint64_t* becc, uint64_t* res, uint32_t threads) {
    Computer c;
    c.threads = threads;
    c.n = n;
    c.g = Csr{n, off, succ};
    const bool undirected = toff == nullptr;
    c.t = undirected ? c.g : Csr{n, toff, tsucc};
    Output o = (Output)level;
    if (undirected && (o == ALL || o == ALL_FORWARD)) o = ALL_FORWARD;  // computer.rs:109-114
    c.out = o;
    c.compute_radial = radial == nullptr;
    c.radial.assign(n, 0);
    if (radial)
        for (u64 i = 0; i < n; i++) c.radial[i] = radial[i] != 0;
    c.forward_low.assign(n, 0);
    c.forward_high.assign(n, n);
    c.backward_low.assign(n, 0);
    c.backward_high.assign(n, n);
    c.forward_tot.assign(n, 0);
    c.backward_tot.assign(n, 0);
    if (undirected) {
        c.comp = symm_components(c.g, c.ncomp);
        c.seg.assign(c.ncomp, 0);
    } else {
        c.comp = tarjan(c.g, c.ncomp);
        scc_dag(c.g, c.t, c.comp, c.ncomp, c.seg, c.conns);
    }
    c.compute();
    res[0] = c.diameter_low;
    res[1] = c.radius_high;
    res[2] = c.diameter_vertex;
    res[3] = c.radius_vertex;
    res[4] = c.radius_it;
    res[5] = c.diameter_it;
    res[6] = c.forward_it;
    res[7] = c.all_it;
    bool ok = true;
    switch (c.out) {
        case ALL: ok = c.all_it != NONE && c.forward_it != NONE && c.diameter_it != NONE && c.radius_it != NONE; break;
        case ALL_FORWARD: ok = c.forward_it != NONE && c.diameter_it != NONE && c.radius_it != NONE; break;
        case RADIUS_DIAMETER: ok = c.diameter_it != NONE && c.radius_it != NONE; break;
        case DIAMETER: ok = c.diameter_it != NONE; break;
        case RADIUS: ok = c.radius_it != NONE; break;
    }
    if (!ok) return -1;
    if (fecc && (c.out == ALL || c.out == ALL_FORWARD))
        for (u64 i = 0; i < n; i++) fecc[i] = c.forward_low[i];
    if (becc && c.out == ALL)
        for (u64 i = 0; i < n; i++) becc[i] = c.backward_high[i];
    return 0;
}

int hbo_sum_sweep(uint64_t n, const uint64_t* off, const uint32_t* succ, const uint64_t* toff,
                  const uint32_t* tsucc, int level, const uint8_t* radial, uint64_t* fecc,
                  uint64_t* becc, uint64_t* res) {
    return hbo_sum_sweep_par(n, off, succ, toff, tsucc, level, radial, fecc, becc, res, 1);
}

// The selections of the restatement, for the reference's own tests of them
// (tests/test_math.rs): the index of the largest (maximize) or smallest
// (value, tie) among the indices with keep[i] != 0, the smallest index among
// equals; ~0 when none is kept.
uint64_t hbo_arg_select(uint64_t n, const uint64_t* val, const uint64_t* tie, const uint8_t* keep, int maximize) {
    auto kept = [&](u64 i) { return keep[i] != 0; };
    return maximize ? argmax_kept(n, val, tie, kept) : argmin_kept(n, val, tie, kept);
}

// The components the restatement computes, for the reference's own tests
// of them (tests/test_sccs.rs): comp[v] for every node; returns their number.
// hbo_sccs_tarjan: sccs/tarjan.rs numbering; hbo_sccs_symm: sccs/symm_seq.rs
// numbering (symmetric graphs).
uint64_t hbo_sccs_tarjan(uint64_t n, const uint64_t* off, const uint32_t* succ, uint64_t* comp) {
    u64 nc = 0;
    const std::vector<u64> c = tarjan(Csr{n, off, succ}, nc);
    std::copy(c.begin(), c.end(), comp);
    return nc;
}

uint64_t hbo_sccs_symm(uint64_t n, const uint64_t* off, const uint32_t* succ, uint64_t* comp) {
    u64 nc = 0;
    const std::vector<u64> c = symm_components(Csr{n, off, succ}, nc);
    std::copy(c.begin(), c.end(), comp);
    return nc;
}

// Forward eccentricity of every node by one breadth-first visit each (the
// definition; small graphs only).
void hbo_eccentricities(uint64_t n, const uint64_t* off, const uint32_t* succ, uint64_t* ecc) {
    Csr g{n, off, succ};
    std::vector<u64> d(n);
    for (u64 v = 0; v < n; v++) {
        std::fill(d.begin(), d.end(), NONE);
        bfs(g, v, d);
        u64 e = 0;
        for (u64 x : d)
            if (x != NONE) e = std::max(e, x);
        ecc[v] = e;
    }
}

}  // extern "C"
