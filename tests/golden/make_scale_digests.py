"""Per-iteration oracle digests of the two large single-graph workloads.

The GPU is compared with the oracle on the graphs the throughput figures are
quoted on, where a lock-step comparison of full arrays would not fit the test
budget:

  rmat24     R-MAT, 2^24 nodes, 16 arcs drawn per node (a, b, c = .57, .19, .19),
             seed 1, log2m 8, SipHash-1-3 with zero keys, systolic iterations
             (transpose given)
  weblike26  web-like, 2^26 nodes (Zipf(2.1) out-degrees of mean 12, capped at
             10^5, 80% of successors within +/-1024 of the source), seed 2,
             log2m 6, the same hash and mode

For every iteration the oracle's threaded engine (the reference's
parallel_task restated, src/algo/hyperball/hyperball_impl.rs:960-1152) gives
the modified counters, visited arcs, mode flags, neighbourhood function and a
SHA-256 of the whole current counter array in the reference's packed layout
(src/utils/slice_counter_array.rs:166-169); at the end, the sums of distances
and harmonic centralities at 4,096 seeded nodes and the sum of each array.
The graph's own SHA-256 is recorded so a machine that regenerates it can tell
that its generator produced the same arcs.

Run on a host with about 20 GB of free memory (it takes minutes per case):
    python tests/golden/make_scale_digests.py [rmat24] [weblike26] [--small]
`--small` writes the same digests for reduced sizes into
scale_digests_small.json (used to check this script and the test quickly).
"""
import ctypes
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "webgraph-algo-rs_gb300"))

SAMPLE_NODES = 4096

CASES = {
    "rmat24": {"kind": "rmat", "log2n": 24, "small_log2n": 14, "edges_per_node": 16,
               "abc": [0.57, 0.19, 0.19], "seed": 1, "log2m": 8},
    "weblike26": {"kind": "weblike", "log2n": 26, "small_log2n": 16, "cap": 100_000,
                  "shift": 1.266, "window": 1024, "seed": 2, "log2m": 6},
}


def make_graph(hb, case, log2n):
    if case["kind"] == "rmat":
        a, b, c = case["abc"]
        return hb.Graph.rmat(log2n, case["edges_per_node"], a, b, c, seed=case["seed"])
    return hb.Graph.weblike(1 << log2n, case["cap"], case["shift"], case["window"], case["seed"])


def graph_sha256(g):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(g.offsets).tobytes())
    h.update(np.ascontiguousarray(g.successors).tobytes())
    return h.hexdigest()


def sample_nodes(n, seed=7):
    k = min(SAMPLE_NODES, n)
    return np.sort(np.random.default_rng(seed).choice(n, size=k, replace=False))


def run_case(name, small, threads):
    import hyperball_gb300 as hb
    from oracle import hbo

    case = CASES[name]
    log2n = case["small_log2n"] if small else case["log2n"]
    t0 = time.time()
    g = make_graph(hb, case, log2n)
    t = g.transpose()
    print(f"{name}: graph 2^{log2n}, {g.num_arcs} arcs, {time.time() - t0:.0f} s", flush=True)
    o = hbo.OracleHyperBall(g.offsets, g.successors, case["log2m"], 0, 0, t_offsets=t.offsets,
                            t_successors=t.successors, sod=True, harm=True, threads=threads)
    del t
    buf = np.empty((g.num_nodes, o.counter_bytes), dtype=np.uint8)
    o.init()
    its = []
    while True:
        t1 = time.time()
        s = o.iterate()
        hbo.lib().hbo_get_array(o._h, 0, buf.ctypes.data)
        its.append({"modified": s["modified"], "visited_arcs": s["visited_arcs"], "nf": s["nf"],
                    "systolic": s["systolic"], "local": s["local"], "pre_local": s["pre_local"],
                    "registers_sha256": hashlib.sha256(buf).hexdigest()})
        print(f"  iteration {len(its) - 1}: modified {s['modified']} visited {s['visited_arcs']}"
              f" systolic {s['systolic']} {time.time() - t1:.1f} s", flush=True)
        if s["modified"] == 0:
            break
    idx = sample_nodes(g.num_nodes)
    sod, harm = o.sum_of_distances(), o.harmonic_centralities()
    return {
        "graph": dict(case, log2n=log2n, nodes=g.num_nodes, arcs=g.num_arcs),
        "graph_sha256": graph_sha256(g),
        "hash": "SipHash-1-3, zero keys",
        "iterations": its,
        "neighborhood_function": [float(x) for x in o.neighborhood_function()],
        "sample_nodes": idx.tolist(),
        "sum_of_distances_at": [float(sod[i]) for i in idx],
        "harmonic_at": [float(harm[i]) for i in idx],
        "sum_of_distances_sum": float(np.sum(sod)),
        "harmonic_sum": float(np.sum(harm)),
        "oracle_threads": threads,
        "oracle_seconds": round(time.time() - t0, 1),
    }


def main(argv):
    small = "--small" in argv
    names = [a for a in argv if a in CASES] or list(CASES)
    out = os.path.join(HERE, "scale_digests_small.json" if small else "scale_digests.json")
    doc = {"cases": {}}
    if os.path.exists(out):
        doc = json.load(open(out))
    threads = len(os.sched_getaffinity(0))
    for name in names:
        doc["cases"][name] = run_case(name, small, threads)
        with open(out, "w") as f:
            json.dump(doc, f, indent=1)
    print("written", out)


if __name__ == "__main__":
    main(sys.argv[1:])
