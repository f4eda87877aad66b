// CPU oracle — test infrastructure only.
//
// A C++17 restatement of the reference HyperBall (webgraph-algo 0.1.0,
// src/algo/hyperball/hyperball_impl.rs, cited as "HB:<line>") and of its
// sequential test recurrence SeqHyperBall (HB:1230-1261). It is the checker the
// GPU path is compared with, and (threaded) the CPU baseline bench.py reports.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// the shared library built from this file; the product never does.
//
// Structure follows the reference one-to-one:
//   init()          HB:1155-1213
//   iterate()       HB:775-949   (mode choice, bitmap prep, granularity, swap, NF)
//   parallel_task() HB:960-1152  (arc-balanced work stealing, union, centralities)
//   run()           HB:534-583
// Threads are std::thread; rayon's broadcast becomes "every worker runs
// parallel_task once". Per-node sums and the local checklist are guarded by
// one mutex each, as the reference guards them (HB:1078, HB:1082, HB:1101).
// The cumulative outdegree `succ` query (webgraph DCF, third party) is a
// lower_bound on the CSR offsets, which is what the Elias-Fano successor
// query returns on a cumulative outdegree list.
//
// Floating point: build with -ffp-contract=off so no multiply-add is fused
// (Rust never fuses), which keeps per-node sums bit-identical to the
// reference's arithmetic.
#include "hll_oracle.hpp"
#include "graph_gen.h"

#include <atomic>
#include <cstdio>
#include <memory>
#include <mutex>
#include <thread>

namespace hbo {

struct IterStats {
    uint64_t iteration;       // 1-based index of the iteration just run
    uint64_t modified;        // counters modified
    uint64_t visited_arcs;    // arcs (u,v), u != v, v modified in the previous iteration
    double nf;                // neighbourhood-function value pushed
    double relative_increment;
    int32_t systolic, local, pre_local, pad;
};

// KahanSum (kahan 0.1.4, third party): textbook compensated summation.
struct Kahan {
    double sum = 0.0, c = 0.0;
    void add(double x) {
        double y = x - c;
        double t = sum + y;
        c = (t - sum) - y;
        sum = t;
    }
};

struct AtomicBits {
    std::vector<std::atomic<uint64_t>> w;
    uint64_t n = 0;
    void init(uint64_t n_) {
        n = n_;
        std::vector<std::atomic<uint64_t>> v((n_ + 63) / 64);
        w.swap(v);
        fill(false);
    }
    void fill(bool b) {
        for (auto& x : w) x.store(b ? ~0ull : 0ull, std::memory_order_relaxed);
    }
    bool get(uint64_t i) const {
        return (w[i >> 6].load(std::memory_order_relaxed) >> (i & 63)) & 1;
    }
    void set(uint64_t i, bool b) {
        if (b)
            w[i >> 6].fetch_or(1ull << (i & 63), std::memory_order_relaxed);
        else
            w[i >> 6].fetch_and(~(1ull << (i & 63)), std::memory_order_relaxed);
    }
    void swap(AtomicBits& o) {
        w.swap(o.w);
        std::swap(n, o.n);
    }
};

struct Engine {
    virtual ~Engine() = default;
    virtual int run(uint64_t upper_bound, double threshold, int has_threshold) = 0;
    virtual int init() = 0;
    virtual int iterate(IterStats* out) = 0;
    virtual uint64_t words_per_counter() const = 0;
    virtual int word_bytes() const = 0;
    virtual void get_array(int which, void* dst) const = 0;
    virtual const std::vector<double>& nf() const = 0;
    virtual const std::vector<double>* sod() const = 0;
    virtual const std::vector<double>* harm() const = 0;
    virtual const std::vector<double>* discounted(size_t i) const = 0;
    virtual double count_node(uint64_t node) const = 0;
    virtual uint64_t iteration() const = 0;
    virtual IterStats last_stats() const = 0;
};

template <class W>
struct HyperBall : Engine {
    // graph
    uint64_t n, m;
    const uint64_t* off;
    const uint32_t* succ;
    const uint64_t* toff;
    const uint32_t* tsucc;
    bool has_transpose;
    const uint64_t* weights;
    uint64_t weight_seed;
    HllLogic<W> logic;
    std::vector<double> lnt;
    size_t wpc;
    std::vector<W> curr, next;
    int num_threads;
    uint64_t granularity;  // node granularity (arc_granularity of the builder)

    // IterationContext HB:413-471
    uint64_t iter = 0;
    double current_nf = 0.0;
    std::mutex nf_mu;
    uint64_t ic_arc_granularity = 0;
    std::atomic<uint64_t> node_cursor{0};
    std::mutex cursor_mu;
    uint64_t cursor_node = 0, cursor_arc = 0;
    std::atomic<uint64_t> visited_arcs{0}, modified_counters{0};
    bool systolic = false, local = false, pre_local = false;
    std::vector<uint32_t> local_checklist;
    std::vector<uint32_t> local_next_must_be_checked;
    std::mutex lnmbc_mu;
    AtomicBits must_be_checked, next_must_be_checked, curr_modified, next_modified;
    bool do_sod, do_harm;
    std::vector<double> sod_v, harm_v;
    std::mutex sod_mu, harm_mu;
    std::vector<double> disc_factor_table;  // func(d) for d = 1..; host-evaluated
    size_t n_disc;
    std::vector<std::vector<double>> disc_v;
    std::vector<double (*)(uint64_t, void*)> disc_fn;
    std::vector<void*> disc_ctx;
    std::mutex disc_mu;

    // HyperBall HB:477-509
    std::vector<double> neighborhood_function;
    double last = 0.0;
    double relative_increment = 0.0;
    bool completed = false;
    IterStats stats{};

    HyperBall(uint64_t n_, const uint64_t* off_, const uint32_t* succ_, const uint64_t* toff_,
              const uint32_t* tsucc_, const HllLogic<W>& lg, int threads, uint64_t gran, bool sod_,
              bool harm_, const uint64_t* weights_, uint64_t wseed)
        : n(n_), m(off_[n_]), off(off_), succ(succ_), toff(toff_), tsucc(tsucc_),
          has_transpose(toff_ != nullptr), weights(weights_), weight_seed(wseed), logic(lg),
          num_threads(threads < 1 ? 1 : threads), granularity(gran), do_sod(sod_), do_harm(harm_) {
        lnt = ln_table(logic.num_registers);
        wpc = logic.words_per_counter;
        curr.assign(n * wpc, 0);
        next.assign(n * wpc, 0);
        must_be_checked.init(n);
        next_must_be_checked.init(n);
        curr_modified.init(n);
        next_modified.init(n);
        if (do_sod) sod_v.assign(n, 0.0);
        if (do_harm) harm_v.assign(n, 0.0);
        n_disc = 0;
    }

    void add_discount(double (*fn)(uint64_t, void*), void* ctx) {
        disc_fn.push_back(fn);
        disc_ctx.push_back(ctx);
        disc_v.emplace_back(n, 0.0);
        n_disc = disc_fn.size();
    }

    uint64_t words_per_counter() const override { return wpc; }
    int word_bytes() const override { return (int)sizeof(W); }
    uint64_t iteration() const override { return iter; }
    IterStats last_stats() const override { return stats; }
    const std::vector<double>& nf() const override { return neighborhood_function; }
    const std::vector<double>* sod() const override { return do_sod ? &sod_v : nullptr; }
    const std::vector<double>* harm() const override { return do_harm ? &harm_v : nullptr; }
    const std::vector<double>* discounted(size_t i) const override {
        return i < n_disc ? &disc_v[i] : nullptr;
    }
    void get_array(int which, void* dst) const override {
        const std::vector<W>& a = which == 0 ? curr : next;
        std::memcpy(dst, a.data(), a.size() * sizeof(W));
    }
    double count_node(uint64_t node) const override {
        return logic.count(&curr[node * wpc], lnt.data());
    }

    // cumul_outdeg.succ(target): (smallest i with off[i] >= target, off[i]).
    std::pair<uint64_t, uint64_t> dcf_succ(uint64_t target) const {
        const uint64_t* p = std::lower_bound(off, off + n + 1, target);
        uint64_t i = (uint64_t)(p - off);
        return {i, off[i]};
    }

    // HB:1155-1213
    int init() override {
        std::fill(curr.begin(), curr.end(), (W)0);
        std::fill(next.begin(), next.end(), (W)0);
        if (weights) {
            // The reference adds `random::<u64>()` values (HB:1167-1174), which is
            // not reproducible; this restatement adds SplitMix64(weight_seed, node, k).
            for (uint64_t i = 0; i < n; i++) {
                uint64_t s = weight_seed ^ (i * 0x9e3779b97f4a7c15ull);
                for (uint64_t k = 0; k < weights[i]; k++) {
                    s += 0x9e3779b97f4a7c15ull;
                    uint64_t z = s;
                    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
                    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
                    z ^= z >> 31;
                    logic.add(&curr[i * wpc], z);
                }
            }
        } else {
            for (uint64_t i = 0; i < n; i++) logic.add(&curr[i * wpc], i);
        }
        completed = false;
        iter = 0;
        systolic = local = pre_local = false;
        reset(granularity);
        if (do_sod) std::fill(sod_v.begin(), sod_v.end(), 0.0);
        if (do_harm) std::fill(harm_v.begin(), harm_v.end(), 0.0);
        for (auto& d : disc_v) std::fill(d.begin(), d.end(), 0.0);
        last = (double)n;
        neighborhood_function.clear();
        neighborhood_function.push_back(last);
        curr_modified.fill(true);
        return 0;
    }

    void reset(uint64_t gran) {
        ic_arc_granularity = gran;
        node_cursor.store(0);
        cursor_node = 0;
        cursor_arc = 0;
        visited_arcs.store(0);
        modified_counters.store(0);
    }

    // HB:775-949
    int iterate(IterStats* out) override {
        const uint64_t num_nodes = n;
        const uint64_t num_arcs = m;
        const uint64_t mod_prev = modified_counters.load();
        const bool prev_was_systolic = systolic;
        const bool prev_was_local = local;
        systolic = has_transpose && iter > 0 && mod_prev < num_nodes / 4;
        current_nf = systolic ? last : 0.0;
        local = pre_local;
        pre_local = systolic && mod_prev < (num_nodes * num_nodes) / (num_arcs * 10);

        if (prev_was_local) {
            for (uint32_t node : local_checklist) next_modified.set(node, false);
        } else {
            next_modified.fill(false);
        }
        if (local) {
            local_checklist.clear();
            std::sort(local_next_must_be_checked.begin(), local_next_must_be_checked.end());
            local_next_must_be_checked.erase(
                std::unique(local_next_must_be_checked.begin(), local_next_must_be_checked.end()),
                local_next_must_be_checked.end());
            std::swap(local_checklist, local_next_must_be_checked);
        } else if (systolic) {
            next_must_be_checked.fill(false);
            if (!prev_was_systolic) must_be_checked.fill(true);
        }

        uint64_t gran = ic_arc_granularity;
        if (num_threads > 1 && !local) {
            if (iter > 0) {
                double a = (double)std::max<uint64_t>(1, num_nodes / (uint64_t)num_threads);
                double b = (double)gran *
                           ((double)num_nodes / (double)std::max<uint64_t>(1, mod_prev));
                gran = (uint64_t)std::min(a, b);
            }
        }
        reset(gran);

        if (num_threads == 1) {
            parallel_task();
        } else {
            std::vector<std::thread> ts;
            for (int t = 0; t < num_threads; t++) ts.emplace_back([this] { parallel_task(); });
            for (auto& t : ts) t.join();
        }

        const uint64_t modc = modified_counters.load();
        std::swap(curr, next);
        curr_modified.swap(next_modified);
        if (systolic) must_be_checked.swap(next_must_be_checked);

        last = current_nf;
        double last_output = neighborhood_function.back();
        if (current_nf < last_output) current_nf = last_output;
        relative_increment = current_nf / last_output;
        neighborhood_function.push_back(current_nf);
        iter += 1;

        stats.iteration = iter;
        stats.modified = modc;
        stats.visited_arcs = visited_arcs.load();
        stats.nf = current_nf;
        stats.relative_increment = relative_increment;
        stats.systolic = systolic;
        stats.local = local;
        stats.pre_local = pre_local;
        if (out) *out = stats;
        return 0;
    }

    // HB:960-1152
    void parallel_task() {
        const uint64_t node_granularity = ic_arc_granularity;
        const uint64_t arc_granularity =
            (uint64_t)std::ceil(((double)m * (double)node_granularity) / (double)n);
        const bool do_centrality = do_sod || do_harm || n_disc > 0;
        const uint64_t node_upper_limit = local ? (uint64_t)local_checklist.size() : n;
        uint64_t my_visited = 0, my_modified = 0;
        const uint64_t arc_upper_limit = m;
        Kahan nf_delta;
        std::vector<W> acc, mask;
        std::vector<W> next_counter(wpc);
        std::vector<double> disc_vals(n_disc);
        for (size_t k = 0; k < n_disc; k++) disc_vals[k] = disc_fn[k](iter + 1, disc_ctx[k]);

        for (;;) {
            uint64_t start, end;
            if (local) {
                start = std::min<uint64_t>(node_cursor.fetch_add(1), node_upper_limit);
                end = std::min<uint64_t>(start + 1, node_upper_limit);
            } else {
                std::lock_guard<std::mutex> g(cursor_mu);
                uint64_t next_node = cursor_node, next_arc = cursor_arc;
                if (next_node >= node_upper_limit) {
                    start = end = node_upper_limit;
                } else {
                    start = next_node;
                    uint64_t target = next_arc + arc_granularity;
                    if (target >= arc_upper_limit) {
                        next_node = node_upper_limit;
                    } else {
                        auto s = dcf_succ(target);
                        next_node = s.first;
                        next_arc = s.second;
                    }
                    end = next_node;
                    cursor_node = next_node;
                    cursor_arc = next_arc;
                }
            }
            if (start == node_upper_limit) break;

            for (uint64_t i = start; i < end; i++) {
                const uint64_t node = local ? local_checklist[i] : i;
                const W* prev_counter = &curr[node * wpc];
                if (!systolic || local || must_be_checked.get(node)) {
                    std::memcpy(next_counter.data(), prev_counter, wpc * sizeof(W));
                    bool modified = false;
                    for (uint64_t a = off[node]; a < off[node + 1]; a++) {
                        const uint64_t s = succ[a];
                        if (s != node && curr_modified.get(s)) {
                            my_visited++;
                            modified = true;
                            logic.merge(next_counter.data(), &curr[s * wpc], acc, mask);
                        }
                    }
                    double post = NAN;
                    const bool counter_modified =
                        modified &&
                        std::memcmp(next_counter.data(), prev_counter, wpc * sizeof(W)) != 0;
                    if (!systolic || counter_modified) post = logic.count(next_counter.data(), lnt.data());
                    if (!systolic) nf_delta.add(post);
                    if (counter_modified && (systolic || do_centrality)) {
                        const double pre = logic.count(prev_counter, lnt.data());
                        if (systolic) {
                            nf_delta.add(-pre);
                            nf_delta.add(post);
                        }
                        if (do_centrality) {
                            const double delta = post - pre;
                            if (delta > 0.0) {
                                if (do_sod) {
                                    const double nv = delta * (double)(iter + 1);
                                    std::lock_guard<std::mutex> g(sod_mu);
                                    sod_v[node] += nv;
                                }
                                if (do_harm) {
                                    const double nv = delta / (double)(iter + 1);
                                    std::lock_guard<std::mutex> g(harm_mu);
                                    harm_v[node] += nv;
                                }
                                for (size_t k = 0; k < n_disc; k++) {
                                    const double nv = delta * disc_vals[k];
                                    std::lock_guard<std::mutex> g(disc_mu);
                                    disc_v[k][node] += nv;
                                }
                            }
                        }
                    }
                    if (counter_modified) {
                        if (pre_local) {
                            std::lock_guard<std::mutex> g(lnmbc_mu);
                            local_next_must_be_checked.push_back((uint32_t)node);
                        }
                        next_modified.set(node, true);
                        if (systolic) {
                            if (pre_local) {
                                std::lock_guard<std::mutex> g(lnmbc_mu);
                                for (uint64_t a = toff[node]; a < toff[node + 1]; a++)
                                    local_next_must_be_checked.push_back(tsucc[a]);
                            } else {
                                for (uint64_t a = toff[node]; a < toff[node + 1]; a++)
                                    next_must_be_checked.set(tsucc[a], true);
                            }
                        }
                        my_modified++;
                    }
                    std::memcpy(&next[node * wpc], next_counter.data(), wpc * sizeof(W));
                } else {
                    if (curr_modified.get(node))
                        std::memcpy(&next[node * wpc], prev_counter, wpc * sizeof(W));
                }
            }
        }
        {
            std::lock_guard<std::mutex> g(nf_mu);
            current_nf += nf_delta.sum;
        }
        visited_arcs.fetch_add(my_visited);
        modified_counters.fetch_add(my_modified);
    }

    // HB:534-583
    int run(uint64_t upper_bound, double threshold, int has_threshold) override {
        upper_bound = std::min(upper_bound, n);
        init();
        for (uint64_t i = 0; i < upper_bound; i++) {
            iterate(nullptr);
            if (modified_counters.load() == 0) break;
            if (has_threshold && i > 3 && relative_increment < 1.0 + threshold) break;
        }
        return 0;
    }
};

// SeqHyperBall (HB:1230-1261): next[i] = curr[i] merged with every successor.
template <class W>
struct SeqHyperBall {
    uint64_t n;
    const uint64_t* off;
    const uint32_t* succ;
    HllLogic<W> logic;
    size_t wpc;
    std::vector<W> curr, next;
    SeqHyperBall(uint64_t n_, const uint64_t* o, const uint32_t* s, const HllLogic<W>& lg)
        : n(n_), off(o), succ(s), logic(lg), wpc(lg.words_per_counter) {
        curr.assign(n * wpc, 0);
        next.assign(n * wpc, 0);
    }
    void init() {
        for (uint64_t i = 0; i < n; i++) logic.add(&curr[i * wpc], i);
    }
    void iterate() {
        std::vector<W> acc, mask;
        for (uint64_t i = 0; i < n; i++) {
            W* c = &next[i * wpc];
            std::memcpy(c, &curr[i * wpc], wpc * sizeof(W));
            for (uint64_t a = off[i]; a < off[i + 1]; a++)
                logic.merge(c, &curr[(uint64_t)succ[a] * wpc], acc, mask);
        }
        std::swap(curr, next);
    }
};

}  // namespace hbo

using namespace hbo;

// ---------------------------------------------------------------------------
// C ABI for the tests (ctypes). Not part of the product.
// ---------------------------------------------------------------------------
extern "C" {

struct hbo_stats {
    uint64_t iteration, modified, visited_arcs;
    double nf, relative_increment;
    int32_t systolic, local, pre_local, pad;
};

static thread_local std::string g_err;

const char* hbo_last_error() { return g_err.c_str(); }

// word_bits: 16, 32 or 64 (the reference's W). num_elements 0 -> n.
void* hbo_create(uint64_t n, const uint64_t* off, const uint32_t* succ, const uint64_t* toff,
                 const uint32_t* tsucc, int log2m, int hash_kind, uint64_t seed,
                 uint64_t num_elements, int word_bits, int flags, int threads,
                 uint64_t granularity, const uint64_t* weights, uint64_t weight_seed) {
    try {
        const bool sod = flags & 1, harm = flags & 2, quirk = !(flags & 4);
        if (num_elements == 0) {
            if (weights) {
                for (uint64_t i = 0; i < n; i++) num_elements += weights[i];
            } else {
                num_elements = n;
            }
        }
        if (granularity == 0) granularity = 16 * 1024;
        Engine* e = nullptr;
        if (word_bits == 64) {
            HllLogic<uint64_t> lg(log2m, num_elements, hash_kind, seed, quirk);
            e = new HyperBall<uint64_t>(n, off, succ, toff, tsucc, lg, threads, granularity, sod,
                                        harm, weights, weight_seed);
        } else if (word_bits == 32) {
            HllLogic<uint32_t> lg(log2m, num_elements, hash_kind, seed, quirk);
            e = new HyperBall<uint32_t>(n, off, succ, toff, tsucc, lg, threads, granularity, sod,
                                        harm, weights, weight_seed);
        } else if (word_bits == 16) {
            HllLogic<uint16_t> lg(log2m, num_elements, hash_kind, seed, quirk);
            e = new HyperBall<uint16_t>(n, off, succ, toff, tsucc, lg, threads, granularity, sod,
                                        harm, weights, weight_seed);
        } else {
            g_err = "word_bits must be 16, 32 or 64";
            return nullptr;
        }
        return e;
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return nullptr;
    }
}

int hbo_add_discount(void* h, double (*fn)(uint64_t, void*), void* ctx) {
    Engine* e = (Engine*)h;
    if (auto p = dynamic_cast<HyperBall<uint64_t>*>(e)) p->add_discount(fn, ctx);
    else if (auto p = dynamic_cast<HyperBall<uint32_t>*>(e)) p->add_discount(fn, ctx);
    else if (auto p = dynamic_cast<HyperBall<uint16_t>*>(e)) p->add_discount(fn, ctx);
    return 0;
}

void hbo_destroy(void* h) { delete (Engine*)h; }
int hbo_init(void* h) { return ((Engine*)h)->init(); }
int hbo_iterate(void* h, hbo_stats* out) {
    IterStats s{};
    int r = ((Engine*)h)->iterate(&s);
    if (out) std::memcpy(out, &s, sizeof(s));
    return r;
}
int hbo_run(void* h, uint64_t upper_bound, double threshold, int has_threshold) {
    return ((Engine*)h)->run(upper_bound, threshold, has_threshold);
}
uint64_t hbo_iteration(void* h) { return ((Engine*)h)->iteration(); }
uint64_t hbo_words_per_counter(void* h) { return ((Engine*)h)->words_per_counter(); }
int hbo_word_bytes(void* h) { return ((Engine*)h)->word_bytes(); }
void hbo_last_stats(void* h, hbo_stats* out) {
    IterStats s = ((Engine*)h)->last_stats();
    std::memcpy(out, &s, sizeof(s));
}
// which: 0 = current state, 1 = next state (raw bytes, n * words * word_bytes)
void hbo_get_array(void* h, int which, void* dst) { ((Engine*)h)->get_array(which, dst); }
uint64_t hbo_nf_len(void* h) { return ((Engine*)h)->nf().size(); }
void hbo_get_nf(void* h, double* dst) {
    const auto& v = ((Engine*)h)->nf();
    std::memcpy(dst, v.data(), v.size() * sizeof(double));
}
int hbo_get_sod(void* h, double* dst) {
    auto v = ((Engine*)h)->sod();
    if (!v) return -1;
    std::memcpy(dst, v->data(), v->size() * sizeof(double));
    return 0;
}
int hbo_get_harm(void* h, double* dst) {
    auto v = ((Engine*)h)->harm();
    if (!v) return -1;
    std::memcpy(dst, v->data(), v->size() * sizeof(double));
    return 0;
}
int hbo_get_discounted(void* h, uint64_t i, double* dst) {
    auto v = ((Engine*)h)->discounted(i);
    if (!v) return -1;
    std::memcpy(dst, v->data(), v->size() * sizeof(double));
    return 0;
}
// reachable_nodes (HB:750-757): count of every current counter.
void hbo_get_reachable(void* h, uint64_t n, double* dst) {
    Engine* e = (Engine*)h;
    for (uint64_t i = 0; i < n; i++) dst[i] = e->count_node(i);
}

// --- SeqHyperBall (HB:1230-1261) ------------------------------------------
struct SeqBox {
    int wb;
    void* p;
};
void* hbo_seq_create(uint64_t n, const uint64_t* off, const uint32_t* succ, int log2m,
                     int hash_kind, uint64_t seed, int word_bits) {
    try {
        SeqBox* b = new SeqBox{word_bits, nullptr};
        if (word_bits == 64)
            b->p = new SeqHyperBall<uint64_t>(n, off, succ, HllLogic<uint64_t>(log2m, n, hash_kind, seed));
        else if (word_bits == 32)
            b->p = new SeqHyperBall<uint32_t>(n, off, succ, HllLogic<uint32_t>(log2m, n, hash_kind, seed));
        else
            b->p = new SeqHyperBall<uint16_t>(n, off, succ, HllLogic<uint16_t>(log2m, n, hash_kind, seed));
        return b;
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return nullptr;
    }
}
#define SEQ_DISPATCH(b, stmt)                                          \
    do {                                                               \
        if ((b)->wb == 64) { auto s = (SeqHyperBall<uint64_t>*)(b)->p; stmt; } \
        else if ((b)->wb == 32) { auto s = (SeqHyperBall<uint32_t>*)(b)->p; stmt; } \
        else { auto s = (SeqHyperBall<uint16_t>*)(b)->p; stmt; }       \
    } while (0)
void hbo_seq_init(void* h) { SEQ_DISPATCH((SeqBox*)h, s->init()); }
void hbo_seq_iterate(void* h) { SEQ_DISPATCH((SeqBox*)h, s->iterate()); }
void hbo_seq_get_array(void* h, int which, void* dst) {
    SEQ_DISPATCH((SeqBox*)h, {
        auto& a = which == 0 ? s->curr : s->next;
        std::memcpy(dst, a.data(), a.size() * sizeof(a[0]));
    });
}
void hbo_seq_destroy(void* h) {
    SeqBox* b = (SeqBox*)h;
    SEQ_DISPATCH(b, delete s);
    delete b;
}

// --- HLL primitives for unit tests ------------------------------------------
uint64_t hbo_hash(int kind, uint64_t seed, uint64_t x) { return hash_node(kind, seed, x); }
uint64_t hbo_siphash(int c, int d, uint64_t k0, uint64_t k1, const uint8_t* msg, uint64_t len) {
    return siphash(c, d, k0, k1, msg, (size_t)len);
}
int hbo_register_size(uint64_t n) { return register_size(n); }

// Counter-level helpers over raw bytes. `bytes` = 2^log2m * 5 / 8.
int hbo_hll_merge(int log2m, uint64_t n, int word_bits, void* x, const void* y) {
    try {
        if (word_bits == 64) {
            HllLogic<uint64_t> lg(log2m, n, 0, 0);
            std::vector<uint64_t> a, b;
            lg.merge((uint64_t*)x, (const uint64_t*)y, a, b);
        } else if (word_bits == 32) {
            HllLogic<uint32_t> lg(log2m, n, 0, 0);
            std::vector<uint32_t> a, b;
            lg.merge((uint32_t*)x, (const uint32_t*)y, a, b);
        } else {
            HllLogic<uint16_t> lg(log2m, n, 0, 0);
            std::vector<uint16_t> a, b;
            lg.merge((uint16_t*)x, (const uint16_t*)y, a, b);
        }
        return 0;
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return -1;
    }
}
double hbo_hll_count(int log2m, uint64_t n, int word_bits, const void* x, int quirk) {
    if (word_bits == 64) {
        HllLogic<uint64_t> lg(log2m, n, 0, 0, quirk != 0);
        return lg.count((const uint64_t*)x);
    } else if (word_bits == 32) {
        HllLogic<uint32_t> lg(log2m, n, 0, 0, quirk != 0);
        return lg.count((const uint32_t*)x);
    }
    HllLogic<uint16_t> lg(log2m, n, 0, 0, quirk != 0);
    return lg.count((const uint16_t*)x);
}
// add(element) with the given hasher into a counter.
void hbo_hll_add(int log2m, uint64_t n, int word_bits, int hash_kind, uint64_t seed, void* x,
                 uint64_t element) {
    if (word_bits == 64) {
        HllLogic<uint64_t> lg(log2m, n, hash_kind, seed);
        lg.add((uint64_t*)x, element);
    } else if (word_bits == 32) {
        HllLogic<uint32_t> lg(log2m, n, hash_kind, seed);
        lg.add((uint32_t*)x, element);
    } else {
        HllLogic<uint16_t> lg(log2m, n, hash_kind, seed);
        lg.add((uint16_t*)x, element);
    }
}
// add a precomputed 64-bit hash value (used by the statistical tests, which
// supply their own hasher exactly as the reference's HLL tests supply xxh3).
void hbo_hll_add_hash(int log2m, uint64_t n, void* x, uint64_t hash) {
    HllLogic<uint16_t> lg(log2m, n, 0, 0);
    lg.add_hash((uint16_t*)x, hash);
}
// Statistical tests (tests/test_hyperloglog_counter.rs): one counter fed with
// precomputed hashes, count() returned; with `merge_with` a second counter fed
// with the other hashes is merged in first.
double hbo_hll_count_hashes(int log2m, uint64_t n, const uint64_t* hashes, uint64_t k,
                            const uint64_t* hashes2, uint64_t k2) {
    HllLogic<uint16_t> lg(log2m, n, 0, 0);
    std::vector<uint16_t> a(lg.words_per_counter, 0), b(lg.words_per_counter, 0), s1, s2;
    for (uint64_t i = 0; i < k; i++) lg.add_hash(a.data(), hashes[i]);
    if (hashes2) {
        for (uint64_t i = 0; i < k2; i++) lg.add_hash(b.data(), hashes2[i]);
        lg.merge(a.data(), b.data(), s1, s2);
    }
    return lg.count(a.data());
}

// Checks the device's division by the iteration number: for d = 1..d_max and
// `samples` random positive doubles a (exponents spread over +-2^40, plus
// near-power-of-two cases), q0 = RN(a*rd), r = fma(-q0, d, a),
// q1 = fma(r, rd, q0) with rd = RN(1/d) must equal a / d. Returns mismatches.
uint64_t hbo_check_div_small_int(uint64_t d_max, uint64_t samples, uint64_t seed) {
    uint64_t bad = 0, s = seed;
    auto next = [&s]() {
        s += 0x9e3779b97f4a7c15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    };
    for (uint64_t di = 1; di <= d_max; di++) {
        const double d = (double)di, rd = 1.0 / d;
        for (uint64_t k = 0; k < samples; k++) {
            const uint64_t r = next();
            double a;
            const uint64_t mant = r & ((1ull << 52) - 1);
            const uint64_t ex = 1023 - 40 + ((r >> 52) % 81);
            uint64_t bits = (ex << 52) | mant;
            if (k % 8 == 0) bits = (ex << 52) | (r % 4 == 0 ? 0 : ((1ull << 52) - 1 - (r >> 60)));
            std::memcpy(&a, &bits, 8);
            const double q0 = a * rd;
            const double rr = std::fma(-q0, d, a);
            const double q1 = std::fma(rr, rd, q0);
            if (q1 != a / d) bad++;
        }
    }
    return bad;
}

// ---- input graphs ------------------------------------------------------------
// The seeded generators are webgraph-algo-rs_gb300/csrc/graph_gen.cpp compiled
// into this library (the product library compiles the same file), so the CPU
// baseline builds the GPU path's input graphs without loading the product.
void* hbo_gen_er(uint64_t n, uint32_t d, uint64_t seed) {
    Csr* g = new Csr();
    hbg::gen_er(n, d, seed, *g);
    return g;
}
void* hbo_gen_rmat(int scale, uint64_t edges_per_node, double a, double b, double c,
                   uint64_t seed) {
    Csr* g = new Csr();
    hbg::gen_rmat(scale, edges_per_node, a, b, c, seed, *g);
    return g;
}
void* hbo_gen_weblike(uint64_t n, uint64_t cap, double shift, uint64_t window, uint64_t seed) {
    Csr* g = new Csr();
    hbg::gen_weblike(n, cap, shift, window, seed, *g);
    return g;
}
void* hbo_graph_transpose(const void* g) {
    Csr* t = new Csr();
    hbg::transpose(*(const Csr*)g, *t);
    return t;
}
void* hbo_transpose_csr(uint64_t n, const uint64_t* off, const uint32_t* succ) {
    Csr g;
    g.n = n;
    g.m = off[n];
    g.offsets.assign(off, off + n + 1);
    g.successors.assign(succ, succ + g.m);
    Csr* t = new Csr();
    hbg::transpose(g, *t);
    return t;
}
uint64_t hbo_graph_nodes(const void* g) { return ((const Csr*)g)->n; }
uint64_t hbo_graph_arcs(const void* g) { return ((const Csr*)g)->m; }
const uint64_t* hbo_graph_offsets(const void* g) { return ((const Csr*)g)->offsets.data(); }
const uint32_t* hbo_graph_successors(const void* g) { return ((const Csr*)g)->successors.data(); }
void hbo_graph_free(void* g) { delete (Csr*)g; }

// Per-counter parameters for the tests.
void hbo_hll_params(int log2m, uint64_t n, double* alpha_m_m, uint64_t* words16) {
    HllLogic<uint16_t> lg(log2m, n, 0, 0);
    *alpha_m_m = lg.alpha_m_m;
    *words16 = lg.words_per_counter;
}

}  // extern "C"
