"""Makes the test fixtures derived from the reference checkout.

Run with the environment variable HB_REFERENCE set to a checkout of the
reference crate. It
  1. copies the cnr-2000 BVGraph files and the five Java-produced HyperBall
     results into tests/golden/_data/ (git-ignored: used by the GPU tests on
     machines without the reference checkout);
  2. writes tests/golden/cnr2000_java_sample.json: the five Java result
     arrays (tests/hyperball_results/*, log2m 8, Jenkins seed 42) at 2,000
     seeded node indices plus a SHA-256 of each full file, so the oracle can
     be checked against the Java values even without the data copy;
  3. writes tests/golden/oracle_digests.json: per-iteration statistics and a
     SHA-256 of the current counter array of the oracle on the small
     configurations, checked by the CPU tests to detect oracle drift.
"""
import hashlib
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "webgraph-algo-rs_gb300"))

REF = os.environ.get("HB_REFERENCE")
if __name__ == "__main__" and not REF:
    raise SystemExit("set HB_REFERENCE to the reference checkout")
NAMES = ["sum_of_distances", "harmonic_centrality", "lin_centrality",
         "closeness_centrality", "nieminen_centrality"]


def copy_data():
    out = os.path.join(HERE, "_data")
    os.makedirs(out, exist_ok=True)
    g = os.path.join(REF, "tests", "graphs")
    for base in ("cnr-2000", "cnr-2000-t"):
        for ext in (".graph", ".properties", ".offsets"):
            shutil.copyfile(os.path.join(g, base + ext), os.path.join(out, base + ext))
    r = os.path.join(REF, "tests", "hyperball_results")
    for n in NAMES:
        shutil.copyfile(os.path.join(r, "cnr-2000_" + n), os.path.join(out, "cnr-2000_" + n))


def java_sample():
    r = os.path.join(REF, "tests", "hyperball_results")
    rng = np.random.default_rng(2024)
    idx = np.sort(rng.choice(325_557, size=2000, replace=False))
    doc = {"source": "tests/hyperball_results/cnr-2000_* (Java HyperBall, log2m 8, Jenkins 42)",
           "nodes": idx.tolist(), "values": {}, "sha256": {}}
    for n in NAMES:
        raw = open(os.path.join(r, "cnr-2000_" + n), "rb").read()
        doc["sha256"][n] = hashlib.sha256(raw).hexdigest()
        a = np.frombuffer(raw, dtype=">f4").astype(np.float64)
        doc["values"][n] = [float(a[i]) for i in idx]
    with open(os.path.join(HERE, "cnr2000_java_sample.json"), "w") as f:
        json.dump(doc, f)


def oracle_digests():
    import hyperball_gb300 as hb
    from oracle import hbo

    hb.load_library()
    cases = []
    for (n, d, seed, log2m, hk, hs) in ((10_000, 8, 0, 6, 0, 0), (3000, 5, 1, 4, 1, 42),
                                        (3000, 5, 2, 8, 0, 0)):
        g = hb.Graph.erdos_renyi(n, d, seed)
        t = g.transpose()
        o = hbo.OracleHyperBall(g.offsets, g.successors, log2m, hash_kind=hk, seed=hs,
                                t_offsets=t.offsets, t_successors=t.successors, sod=True, harm=True)
        o.init()
        its = []
        while True:
            s = o.iterate()
            its.append({"modified": s["modified"], "visited_arcs": s["visited_arcs"],
                        "nf": s["nf"], "systolic": s["systolic"], "local": s["local"],
                        "registers_sha256": hashlib.sha256(o.registers(0).tobytes()).hexdigest()})
            if s["modified"] == 0:
                break
        cases.append({"graph": f"erdos_renyi(n={n}, d={d}, seed={seed})", "log2m": log2m,
                      "hash_kind": hk, "hash_seed": hs,
                      "graph_sha256": hashlib.sha256(g.successors.tobytes()).hexdigest(),
                      "iterations": its,
                      "sum_of_distances_sum": float(np.sum(o.sum_of_distances())),
                      "harmonic_sum": float(np.sum(o.harmonic_centralities()))})
    with open(os.path.join(HERE, "oracle_digests.json"), "w") as f:
        json.dump({"cases": cases}, f, indent=1)


if __name__ == "__main__":
    copy_data()
    java_sample()
    oracle_digests()
    print("fixtures written")
