#!/usr/bin/env python3
"""HyperBall benchmark on one GB300: arc-register updates per second.

Workload: the synthetic web-like graph with 2^26 nodes (out-degrees Zipf with
exponent 2.1 and mean 12, capped at 10^5; 80% of the successors uniform
within +/-1024 of the source id, 20% uniform over all nodes; seed 2), HyperLogLog
counters with 2^6 registers (SipHash-1-3 node hash, seed 0), systolic
iterations with the transpose built on the device, sum of distances and
harmonic centrality, run until no counter changes.

A step is one complete HyperBall run (hb_run_until_done: init plus every
iteration). The work unit is the arc-register update: visited_arcs_t * 2^log2m
summed over the iterations (the visited arcs are deterministic). `value` is
measured with the graph resident in HBM; `e2e` goes through the public API
from pinned host buffers (hb_create copies the CSR in and builds the transpose
on the device, then the run, then the neighbourhood function, sums of
distances and harmonic centralities are read back). At one GPU the 2^26
web-like line also carries `rmat24`: the whole line of `--workload rmat` (R-MAT 2^24
with 2^8 registers per counter), run in a child process after the headline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`--impl reference` times the CPU restatement of the reference algorithm (the
oracle's threaded engine, one thread per host core) on the same workload and
the same work per step: one complete run (init plus every iteration to
stabilisation). Its graph comes from the generators compiled into the
oracle's library, so that process never loads the product library. The GPU
line's `cpu_baseline` is the same measurement.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "webgraph-algo-rs_gb300"))

METRIC = "HyperBall arc-register updates/s"
UNIT = "arc-register updates/s"
LOG2M = 6
COUNTER_BYTES = (1 << LOG2M) * 5 // 8
PROFILES = {"weblike": os.path.join(ROOT, "profiles", "union_weblike.md"),
            "rmat": os.path.join(ROOT, "profiles", "union_rmat.md")}
DIGESTS = os.path.join(ROOT, "tests", "golden", "scale_digests.json")


def parse_args():
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--log2n", type=int, default=None,
                   help="graph size (2^log2n nodes; default 26 web-like, 24 R-MAT)")
    p.add_argument("--e2e-steps", type=int, default=None, help="end-to-end steps (default: --steps)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-rmat", action="store_true",
                   help="web-like workload: skip the R-MAT 2^24 run reported beside it (rmat24)")
    p.add_argument("--workload", choices=["weblike", "rmat", "batched", "served", "visit", "sumsweep"],
                   default="weblike",
                   help="weblike: the 2^26 web-like graph (default); rmat: R-MAT 2^24 x 16, "
                        "log2m 8; batched: many small graphs; served: a Poisson stream of jobs "
                        "through the job server")
    p.add_argument("--batch-count", type=int, default=4096, help="graphs in the batched workload")
    p.add_argument("--alone-sample", type=int, default=0,
                   help="graphs of the batch also run one at a time (0: all of them)")
    p.add_argument("--jobs", type=int, default=2000, help="jobs of the served stream")
    p.add_argument("--rate", type=float, default=200.0, help="job arrivals per second")
    p.add_argument("--pool", type=int, default=48, help="distinct graphs the served jobs draw from")
    p.add_argument("--max-active", type=int, default=16, help="served: jobs on the device at once")
    p.add_argument("--sustained-rate", type=float, default=40.0,
                   help="served: a second, lower arrival rate (0: none)")
    p.add_argument("--setup-threads", type=int, default=0,
                   help="served: job creation / results threads (0: the server's default)")
    p.add_argument("--union-sm-reserve", type=int, default=None,
                   help="served: SMs the shared union launch leaves to job creation (default: the server's)")
    args = p.parse_args()
    set_workload(args)
    return args


def set_workload(args):
    """Graph size and counter size of the single-graph workloads."""
    global LOG2M, COUNTER_BYTES
    if args.workload == "rmat":
        LOG2M = 8
        if args.log2n is None:
            args.log2n = 24
    elif args.workload == "sumsweep" and args.log2n is None:
        args.log2n = 20
    elif args.log2n is None:
        args.log2n = 26
    COUNTER_BYTES = (1 << LOG2M) * 5 // 8


def make_graph(args):
    import hyperball_gb300 as hb
    if args.workload == "rmat":
        return hb.Graph.rmat(args.log2n, 16, 0.57, 0.19, 0.19, seed=1)
    return hb.Graph.weblike(1 << args.log2n)


def make_oracle_graph(args):
    """The same graph from the generators compiled into the oracle's library
    (same source file as the product's)."""
    from oracle import hbo
    if args.workload == "rmat":
        return hbo.OracleGraph.rmat(args.log2n, 16, 0.57, 0.19, 0.19, seed=1)
    return hbo.OracleGraph.weblike(1 << args.log2n)


def digest_key(args):
    """Name of the committed oracle digest of this workload, if there is one."""
    if args.workload == "rmat" and args.log2n == 24:
        return "rmat24"
    if args.workload == "weblike" and args.log2n == 26:
        return "weblike26"
    return None


def workload(args, arcs=None, iterations=None):
    if args.workload == "rmat":
        name = f"rmat-2^{args.log2n} HyperBall to stabilisation"
        graph = "R-MAT (0.57, 0.19, 0.19, 0.05), 16 arcs drawn per node, seed 1, duplicates and self-loops removed"
    else:
        name = f"weblike-2^{args.log2n} HyperBall to stabilisation"
        graph = ("web-like: Zipf(2.1) out-degree, mean 12, cap 1e5; 80% of successors within "
                 "+/-1024 of the source, 20% uniform; seed 2")
    return {
        "workload": name,
        "nodes": 1 << args.log2n,
        "graph": graph,
        "log2m": LOG2M,
        "hash": "SipHash-1-3, seed 0",
        "mode": "systolic, transpose built on device",
        "outputs": "neighbourhood function, sum of distances, harmonic centrality",
        "l2": f"inputs larger than L2 (two 2^n x {COUNTER_BYTES} B counter arrays, CSR 4 B/arc)",
        "arcs": arcs,
        "iterations": iterations,
        "parallelism": "replicas x" + os.environ.get("WORLD_SIZE", "1"),
    }


# ---------------------------------------------------------------------------
# replicas: one process per GPU, independent instances, no data-path collective
# ---------------------------------------------------------------------------
class Ranks:
    """Barrier and max-over-ranks for `world` replicas (torchrun env); a
    no-op for one process."""

    def __init__(self, world, backend, device=None):
        import torch
        self.world, self.dist, self.device = world, None, device
        if world > 1:
            import torch.distributed as dist
            kw = {"device_id": device} if backend == "nccl" else {}
            dist.init_process_group(backend, **kw)
            self.dist = dist
        self.torch = torch

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x):
        if self.dist is None:
            return x
        t = self.torch.tensor([float(x)], dtype=self.torch.float64,
                              device=self.device if self.device is not None else "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()


def job_value(world, steps, units_per_step, seconds):
    """Whole-job throughput: every replica did `steps` steps of `units_per_step`
    units; `seconds` is the max over replicas."""
    return world * steps * units_per_step / seconds


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu_id):
        self.samples = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-i", str(gpu_id), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                self.samples.append(f)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        return self.summarise(self.samples)

    @classmethod
    def summarise(cls, samples):
        """Median SM clock, max clock and the throttle reasons seen in
        `nvidia-smi --format=csv,noheader,nounits` rows of FIELDS."""
        sm, mx, reasons = [], None, set()
        for f in samples:
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(cls.NAMES, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# roofline model of the union kernels (k_union_window + k_union_heavy)
# ---------------------------------------------------------------------------
N_SUMS = 2  # sum of distances and harmonic centrality are requested


def union_model_bytes(stats, n, with_sums=False):
    """Compulsory HBM bytes of the union kernels of each iteration (the
    per-iteration model B_t of the hot-path measurement plan):
        8 (S_t + 1)   offsets of the scanned nodes
      + 4 A_t         successor ids of the scanned nodes
      + W U_t         one read per distinct modified successor counter
                      (U_t bounded by min(previously modified, visited arcs))
      + 2 W S_t       previous read and next write of the scanned nodes
      + n / 4         the four bitmaps
    with W the reference's counter size (2^log2m * 5 / 8 bytes). with_sums
    adds, per changed counter, the requested per-node sums and the estimate
    cache read and written once (16 + 16 * N_SUMS bytes)."""
    out = []
    prev_mod = n  # init marks every counter modified
    for s in stats:
        S, A, V, M = s["scanned_nodes"], s["scanned_arcs"], s["visited_arcs"], s["modified_counters"]
        U = min(prev_mod, V)
        b = 8 * (S + 1) + 4 * A + COUNTER_BYTES * U + 2 * COUNTER_BYTES * S + n // 4
        if with_sums:
            b += (16 + 16 * N_SUMS) * M
        out.append(b)
        prev_mod = M
    return out


def profiled_traffic_ratio(workload_name):
    """DRAM bytes per model byte of one union launch, from the committed ncu
    summary of this workload (None when there is none)."""
    try:
        text = open(PROFILES[workload_name]).read()
    except (OSError, KeyError):
        return None
    m = re.search(r"dram_bytes_per_model_byte:\s*([0-9.]+)", text)
    return float(m.group(1)) if m else None


# ---------------------------------------------------------------------------
# CPU restatement (oracle): one complete run of the same workload
# ---------------------------------------------------------------------------
def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_full_run(offsets, successors, t_offsets, t_successors, warm_iterations):
    """The oracle's threaded engine (one thread per host core) on the graph:
    `warm_iterations` iterations of a first run (untimed), then one complete
    run timed, init plus every iteration until no counter changes, which is
    the work of one GPU step. Returns units, seconds, iterations, cores."""
    from oracle import hbo
    cores = host_cores()
    o = hbo.OracleHyperBall(offsets, successors, LOG2M, 0, 0, t_offsets=t_offsets,
                            t_successors=t_successors, sod=True, harm=True, threads=cores)
    o.init()
    for _ in range(warm_iterations):
        if o.iterate()["modified"] == 0:
            break
    t = time.perf_counter()
    o.init()
    visited, iters = 0, 0
    while True:
        st = o.iterate()
        visited += st["visited_arcs"]
        iters += 1
        if st["modified"] == 0:
            break
    secs = time.perf_counter() - t
    return {"units": visited << LOG2M, "seconds": secs, "iterations": iters, "cores": cores}


def cpu_bounded_run(offsets, successors, t_offsets, t_successors, budget_s=30.0):
    """A bounded sample of the same run for the GPU line: init and the
    iterations of the run from the start until `budget_s` of CPU time has
    passed (the standard iterations that carry nearly all the arcs)."""
    from oracle import hbo
    cores = host_cores()
    o = hbo.OracleHyperBall(offsets, successors, LOG2M, 0, 0, t_offsets=t_offsets,
                            t_successors=t_successors, sod=True, harm=True, threads=cores)
    t = time.perf_counter()
    o.init()
    visited, iters, last = 0, 0, 0.0
    # at least one iteration; another only if one more like the last still
    # ends within the budget
    while iters == 0 or time.perf_counter() - t + last < budget_s:
        t_it = time.perf_counter()
        st = o.iterate()
        last = time.perf_counter() - t_it
        visited += st["visited_arcs"]
        iters += 1
        if st["modified"] == 0:
            break
    secs = time.perf_counter() - t
    return {"units": visited << LOG2M, "seconds": secs, "iterations": iters, "cores": cores,
            "visited": visited}


def cpu_baseline_object(r, warm_iterations):
    return {
        "value": r["units"] / r["seconds"], "unit": UNIT, "cores": r["cores"], "kind": "port",
        "sample": (f"C++ restatement of the reference algorithm (oracle), threaded engine, "
                   f"{r['cores']} threads: one complete run of the same graph (init + "
                   f"{r['iterations']} iterations to stabilisation, the GPU step's work) in "
                   f"{r['seconds']:.1f} s, after {warm_iterations} warm-up iterations"),
    }


# ---------------------------------------------------------------------------
def run_reference(args):
    """The CPU arm: only oracle/ libraries are loaded in this process."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    if args.workload == "sumsweep":
        return run_reference_sumsweep(args)
    if args.workload == "visit":
        return run_reference_visit(args)
    if args.workload not in ("weblike", "rmat"):
        print(json.dumps({"impl": "reference", "unavailable":
                          "the CPU arm times the single-graph workloads (weblike, rmat, visit) "
                          "and sumsweep"}),
              flush=True)
        return 0
    g = make_oracle_graph(args)
    t = g.transpose()
    # warm-up: the first iterations of an earlier run (at most 3: each is
    # seconds of CPU time, and the timed run is minutes)
    warm = min(args.warmup, 3)
    r = cpu_full_run(g.offsets, g.successors, t.offsets, t.successors, warm)
    value = r["units"] / r["seconds"]
    cb = cpu_baseline_object(r, warm)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": 1, "warmup": warm,
        "ms_per_step": 1e3 * r["seconds"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": workload(args, g.num_arcs, r["iterations"]),
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("one step = one complete run (minutes on the host cores), so one step is timed; "
                 "the warm-up is the first iterations of an earlier run"),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_reference_visit(args):
    """The oracle's fair parallel visit (par_fair.rs restated, all host
    threads) of the graph of --workload visit from node 0; each step is one
    complete visit after a reset."""
    import numpy as np
    from oracle import hbo
    g = make_oracle_graph(args)
    o = hbo.OracleVisit(g.offsets, g.successors)
    threads = os.cpu_count() or 1
    for _ in range(min(args.warmup, 1)):
        o.reset()
        nodes = o.par_visit([0], threads=threads)[0]
    off = np.asarray(g.offsets)
    idx = nodes.astype(np.int64)
    arcs = int(np.sum(off[idx + 1] - off[idx]))
    steps = max(1, min(args.steps, 3))
    secs = []
    for _ in range(steps):
        o.reset()
        t0 = time.perf_counter()
        nodes, _, dists = o.par_visit([0], threads=threads)
        secs.append(time.perf_counter() - t0)
    dt = sum(secs) / steps
    line = {
        "impl": "reference", "metric": "breadth-first visit arcs examined/s", "value": arcs / dt,
        "unit": "arcs/s", "n_gpus": args.gpus, "steps": steps, "warmup": min(args.warmup, 1),
        "ms_per_step": 1e3 * dt, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"weblike-2^{args.log2n} breadth-first visit from node 0",
                   "nodes": g.num_nodes, "arcs": g.num_arcs, "visited": len(nodes),
                   "levels": int(dists.max()) + 1 if len(dists) else 0, "arcs_examined": arcs},
        "cpu_baseline": {"value": arcs / dt, "unit": "arcs/s", "cores": threads, "kind": "port",
                         "sample": f"fair parallel breadth-first visit (par_fair.rs restated) on "
                                   f"{threads} threads, complete visits"},
        "e2e": {"value": arcs / dt, "unit": "arcs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_reference_sumsweep(args):
    """The oracle's ExactSumSweep (sequential visits) on the graph of
    --workload sumsweep; each step is one complete call."""
    from oracle import hbo
    g = hbo.OracleGraph.weblike(1 << args.log2n)
    t = g.transpose()
    level = "radius_diameter"
    threads = os.cpu_count() or 1
    for _ in range(min(args.warmup, 1)):
        hbo.sum_sweep(g.offsets, g.successors, t.offsets, t.successors, level=level, threads=threads)
    steps = max(1, min(args.steps, 2))
    t0 = time.perf_counter()
    for _ in range(steps):
        r = hbo.sum_sweep(g.offsets, g.successors, t.offsets, t.successors, level=level, threads=threads)
    dt = (time.perf_counter() - t0) / steps
    line = {
        "impl": "reference", "metric": "ExactSumSweep RadiusDiameter runs/s", "value": 1.0 / dt,
        "unit": "runs/s", "n_gpus": args.gpus, "steps": steps, "warmup": min(args.warmup, 1),
        "ms_per_step": 1e3 * dt, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"weblike-2^{args.log2n} ExactSumSweep RadiusDiameter (directed)",
                   "nodes": g.num_nodes, "arcs": g.num_arcs, "diameter": r["diameter"],
                   "radius": r["radius"], "diameter_iterations": r["diameter_iterations"]},
        "cpu_baseline": {"value": 1.0 / dt, "unit": "runs/s", "cores": threads, "kind": "port",
                         "sample": f"ExactSumSweep restated (computer.rs), fair parallel visits on "
                                   f"{threads} threads"},
        "e2e": {"value": 1.0 / dt, "unit": "runs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def check_digest(h, args, buf_holder):
    """Compares the last run of handle h with the committed oracle digest of
    this workload: per-iteration modified counters and visited arcs, the
    SHA-256 of the final registers and the neighbourhood function (1e-12).
    Raises on a mismatch; returns a summary (None without a digest)."""
    import hashlib
    import numpy as np
    key = digest_key(args)
    if key is None or not os.path.exists(DIGESTS):
        return None
    d = json.load(open(DIGESTS))["cases"].get(key)
    if d is None:
        return None
    st = h.iteration_stats()
    got = [(s["modified_counters"], s["visited_arcs"]) for s in st]
    want = [(it["modified"], it["visited_arcs"]) for it in d["iterations"]]
    if got != want:
        raise RuntimeError(f"oracle digest {key}: per-iteration counts differ")
    buf = h.registers(0)
    sha = hashlib.sha256(buf).hexdigest()
    del buf
    if sha != d["iterations"][-1]["registers_sha256"]:
        raise RuntimeError(f"oracle digest {key}: final registers differ")
    nf = h.neighborhood_function()
    ref = np.array(d["neighborhood_function"])
    err = float(np.max(np.abs(nf - ref) / np.maximum(np.abs(ref), 1e-300)))
    if len(nf) != len(ref) or err > 1e-12:
        raise RuntimeError(f"oracle digest {key}: neighbourhood function differs ({err:.2e})")
    return {"oracle_digest": key, "result": "match",
            "checked": "per-iteration modified counters and visited arcs, SHA-256 of the final "
                       "registers (bit-exact), neighbourhood function within 1e-12",
            "nf_max_rel_err": err}


def run_gb300(args):
    import numpy as np
    import torch
    import hyperball_gb300 as hb

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device (there is no CPU path)")
    torch.cuda.set_device(local)
    ranks = Ranks(world, "nccl", torch.device("cuda", local))
    barrier, max_over_ranks = ranks.barrier, ranks.max

    g = make_graph(args)
    n, m = g.num_nodes, g.num_arcs
    stream = torch.cuda.Stream()
    logic = hb.HyperLogLogBuilder(n).log_2_num_reg(LOG2M).build()
    # degree buckets chosen by the library's autotuner on this graph (outside
    # the timed regions; every pair gives identical results)
    t_tune = time.perf_counter()
    small, medium, _ = hb.tune_degree_buckets(g, logic, iterations=4, device=local,
                                              stream=stream.cuda_stream)
    t_tune = time.perf_counter() - t_tune
    h = (hb.HyperBallBuilder.new(g, logic).transpose_on_device(True)
         .sum_of_distances(True).sum_of_inverse_distances(True).degree_buckets(small, medium)
         .stream(stream.cuda_stream).device(local).build())

    for _ in range(args.warmup):
        h.run_until_done()
    # The union-kernel autotuner times one variant per sampled iteration (at
    # most one or two per run); the timed runs start once it has chosen for
    # both kinds of standard iteration, or once a run used the same variants
    # as the run before (a kind of iteration it never samples stays -1).
    tuning_runs = 0
    used = [s["union_variant"] for s in h.iteration_stats()]
    while -1 in list(h.union_variants_chosen())[:2] and tuning_runs < hb.union_variant_count():
        h.run_until_done()
        tuning_runs += 1
        now = [s["union_variant"] for s in h.iteration_stats()]
        if now == used:
            break
        used = now
    ref_stats = [dict(s) for s in h.iteration_stats()]
    units_per_step = sum(s["visited_arcs"] for s in ref_stats) << LOG2M
    # the run just finished against the oracle's digest of this workload
    parity = check_digest(h, args, None)

    # --- device-resident timed region -------------------------------------
    props = torch.cuda.get_device_properties(local)
    gpu_id = f"GPU-{props.uuid}" if getattr(props, "uuid", None) else str(local)
    barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(gpu_id)
    launches0 = h.kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    # the timed region is the profiled range (ncu --profile-from-start off)
    torch.cuda.profiler.start()
    ev0.record(stream)
    union_ms, model_bytes, model_sums, iters = 0.0, 0, 0, 0
    for _ in range(args.steps):
        h.run_until_done()
        st = h.iteration_stats()
        if [s["visited_arcs"] for s in st] != [s["visited_arcs"] for s in ref_stats]:
            raise RuntimeError("visited arcs differ between runs")
        union_ms += sum(s["union_ms"] for s in st)
        model_bytes += sum(union_model_bytes(st, n))
        model_sums += sum(union_model_bytes(st, n, with_sums=True))
        iters += len(st)
    ev1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    variants = h.union_variants_chosen()
    replayed = sum(s["from_graph"] for s in st)
    barrier()
    clk = clocks.stop()
    launches = h.kernel_launches() - launches0
    elapsed_ms = max_over_ranks(ev0.elapsed_time(ev1))
    value = job_value(world, args.steps, units_per_step, elapsed_ms / 1e3)

    achieved = model_bytes / (union_ms / 1e3) / 1e9
    peak = None
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        peak_src = "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "fallback"
    ratio = profiled_traffic_ratio(args.workload)
    per_launch_model = model_bytes / iters
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": peak_src,
        "traffic": ratio * per_launch_model if ratio else None,
        "traffic_source": (f"DRAM bytes per model byte of the committed ncu capture of this "
                           f"workload ({os.path.relpath(PROFILES[args.workload], ROOT)}) times "
                           f"the model bytes of the average launch") if ratio else
                          "no ncu capture of this workload",
        "kernel": ("union (k_union_window or k_union_staged, and k_union_heavy), one launch "
                   "each per iteration"),
        "model": "compulsory bytes: 8(S+1) + 4A + W U + 2 W S + n/4 per iteration",
        "model_bytes_per_launch": per_launch_model,
        "with_sums": {"achieved": model_sums / (union_ms / 1e3) / 1e9,
                      "frac": model_sums / (union_ms / 1e3) / 1e9 / peak,
                      "note": "the same model plus the per-node sums and estimate cache of "
                              "each changed counter (48 B)"},
        "union_ms_per_step": union_ms / args.steps,
    }

    # --- end to end through the public API from pinned host buffers ---------
    e2e_steps = args.e2e_steps if args.e2e_steps is not None else args.steps
    off_pin = torch.empty(n + 1, dtype=torch.int64).pin_memory()
    suc_pin = torch.empty(m, dtype=torch.int32).pin_memory()
    off_pin.numpy()[:] = np.asarray(g.offsets).view(np.int64)
    suc_pin.numpy()[:] = np.asarray(g.successors).view(np.int32)
    view = hb.CsrView(n, m, off_pin.data_ptr(), suc_pin.data_ptr(), owner=(off_pin, suc_pin))
    h.close()
    del h
    nf_len = len(ref_stats) + 1
    # per-node results land in page-locked host buffers
    sod_pin = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    harm_pin = torch.empty(n, dtype=torch.float64).pin_memory().numpy()

    phases = {"create": 0.0, "run": 0.0, "results": 0.0, "destroy": 0.0}

    def e2e_step():
        # every call below returns after its device work completed
        t = [time.perf_counter()]
        hh = (hb.HyperBallBuilder.new(view, logic).transpose_on_device(True)
              .sum_of_distances(True).sum_of_inverse_distances(True).degree_buckets(small, medium)
              .stream(stream.cuda_stream).device(local).build())
        t.append(time.perf_counter())
        hh.run_until_done()
        t.append(time.perf_counter())
        nf = hh.neighborhood_function()
        hh.sum_of_distances(out=sod_pin)
        hh.harmonic_centralities(out=harm_pin)
        t.append(time.perf_counter())
        k = hh.kernel_launches()
        hh.close()
        t.append(time.perf_counter())
        for i, name in enumerate(phases):
            phases[name] += 1e3 * (t[i + 1] - t[i])
        return len(nf), k

    e2e_step()  # warm-up
    for name in phases:
        phases[name] = 0.0
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_launches = 0
    for _ in range(e2e_steps):
        got, k = e2e_step()
        e2e_launches += k
        if got != nf_len:
            raise RuntimeError("end-to-end run took a different number of iterations")
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = {
        "value": job_value(world, e2e_steps, units_per_step, e2e_s), "unit": UNIT,
        "h2d_bytes_per_step": 8 * (n + 1) + 4 * m,
        "d2h_bytes_per_step": 16 * n + 8 * nf_len,
        "ms_per_step": 1e3 * e2e_s / e2e_steps,
        "phases_ms": {k: v / max(e2e_steps, 1) for k, v in phases.items()},
        "gpu_launches_per_step": e2e_launches // max(e2e_steps, 1),
    }

    cpu_baseline = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import hbo
        t = hbo.OracleGraph.transpose_of(g.offsets, g.successors)
        r = cpu_bounded_run(g.offsets, g.successors, t.offsets, t.successors)
        del t
        want = sum(s["visited_arcs"] for s in ref_stats[:r["iterations"]])
        if r["visited"] != want:
            raise RuntimeError("the oracle's iterations visited other arcs than the GPU's")
        cpu_baseline = {
            "value": r["units"] / r["seconds"], "unit": UNIT, "cores": r["cores"], "kind": "port",
            "sample": (f"C++ restatement of the reference algorithm (oracle), threaded engine, "
                       f"{r['cores']} threads: init + the first {r['iterations']} of the run's "
                       f"{len(ref_stats)} iterations ({r['visited']} of {units_per_step >> LOG2M} "
                       f"visited arcs) in {r['seconds']:.1f} s, a bounded sample; the reference "
                       f"arm (--impl reference) times the complete run"),
        }

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": workload(args, m, len(ref_stats)),
            "tuning": {"degree_buckets": [small, medium], "bucket_tuning_s": round(t_tune, 2),
                       "union_variants": variants, "variant_tuning_runs": tuning_runs,
                       "graph_replayed_iterations": f"{replayed} of {len(st)}"},
            "roofline": roofline, "cpu_baseline": cpu_baseline, "e2e": e2e,
            "parity": parity, "clocks": clk, "gpu_launches": launches,
            "iteration_union_ms": [round(s["union_ms"], 3) for s in st],
        }
    ranks.close()
    if rank == 0 and world == 1 and args.workload == "weblike" and args.log2n == 26 and not args.no_rmat:
        # the R-MAT 2^24 configuration in its own process, reported beside
        # the headline; this process's cached device memory is returned first
        del g
        hb.release_cached_memory(local)
        line["rmat24"] = rmat_subrun(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def rmat_subrun(args):
    """`bench.py --workload rmat` (R-MAT 2^24 x 16, log2m 8: every figure of
    its own line, parity against its oracle digest included) as a child
    process; a failure there fails this run."""
    cmd = [sys.executable, os.path.abspath(__file__), "--workload", "rmat",
           "--steps", str(min(args.steps, 5)), "--warmup", str(args.warmup), "--no-cpu-baseline"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT)
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    if r.returncode != 0 or not lines:
        sys.stderr.write(r.stdout[-2000:] + r.stderr[-4000:])
        raise RuntimeError(f"the R-MAT 2^24 run failed (exit {r.returncode})")
    sub = json.loads(lines[-1])
    sub["command"] = " ".join(["python", "bench.py"] + cmd[2:])
    return sub


# ---------------------------------------------------------------------------
# batched workload: many independent small graphs
# ---------------------------------------------------------------------------
def batch_specs(count, seed=2024):
    """(kind, nodes, degree, log2m, seed) of each graph: node counts log-uniform in
    [10^3, 2*10^5]; even seeds Erdos-Renyi with out-degree uniform in [4, 32],
    odd seeds R-MAT (0.57, 0.19, 0.19, 0.05) with 16 arcs per node (2^scale
    nodes, scale rounded from the drawn count); log2m uniform in {4, 6, 8}."""
    import numpy as np
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        n = int(round(10 ** rng.uniform(3.0, np.log10(2e5))))
        l2m = int(rng.choice([4, 6, 8]))
        if i % 2 == 0:
            specs.append(("er", n, int(rng.integers(4, 33)), l2m, i))
        else:
            specs.append(("rmat", int(round(np.log2(n))), 16, l2m, i))
    return specs


def make_batch_graphs(specs):
    import hyperball_gb300 as hb
    from concurrent.futures import ThreadPoolExecutor

    def one(sp):
        kind, size, deg, _, seed = sp
        if kind == "er":
            return hb.Graph.erdos_renyi(size, deg, seed)
        return hb.Graph.rmat(size, deg, seed=seed)

    with ThreadPoolExecutor(max_workers=host_cores()) as ex:
        return list(ex.map(one, specs))


def run_batched(args):
    import random
    import torch
    import hyperball_gb300 as hb

    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    torch.cuda.set_device(0)
    specs = batch_specs(args.batch_count)
    graphs = make_batch_graphs(specs)
    log2ms = [sp[3] for sp in specs]
    nodes = sum(g.num_nodes for g in graphs)
    arcs = sum(g.num_arcs for g in graphs)

    replays = [None]
    union_ms = [0.0]

    def batch_run():
        b = hb.HyperBallBatch(graphs, log2ms, sum_of_distances=True, sum_of_inverse_distances=True)
        torch.cuda.synchronize()
        t = time.perf_counter()
        b.run_until_done()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        st = b.stats()
        b.close()
        replays[0] = f'{st["graph_replays"]} of {st["group_iterations"]}'
        union_ms[0] = st["union_ms"]
        return st["register_updates"], dt, st["iterations"]

    for _ in range(max(args.warmup - 2, 1)):
        batch_run()
    units = secs = 0.0
    for _ in range(args.steps):
        u, dt, iters = batch_run()
        units += u
        secs += dt
    batched = units / secs

    # the same graphs one at a time through the single-instance API
    k = args.alone_sample if args.alone_sample > 0 else len(graphs)
    sample = sorted(random.Random(7).sample(range(len(graphs)), min(k, len(graphs))))
    a_units = a_secs = 0
    for i in sample:
        g = graphs[i]
        logic = hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(log2ms[i]).build()
        h = (hb.HyperBallBuilder.new(g, logic).transpose_on_device(True)
             .sum_of_distances(True).sum_of_inverse_distances(True).build())
        h.run_until_done()  # warm-up of this instance
        torch.cuda.synchronize()
        t = time.perf_counter()
        h.run_until_done()
        torch.cuda.synchronize()
        a_secs += time.perf_counter() - t
        a_units += sum(s["visited_arcs"] for s in h.iteration_stats()) << log2ms[i]
        h.close()
    alone = a_units / a_secs
    line = {
        "metric": METRIC + " (batched)", "value": batched, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic",
        "config": {"workload": f"{len(graphs)} independent graphs, batched", "nodes": nodes,
                   "arcs": arcs, "graphs": "n log-uniform in [1e3, 2e5]; even seeds Erdos-Renyi "
                   "out-degree U[4,32], odd seeds R-MAT(.57,.19,.19,.05) 16 arcs/node; "
                   "log2m in {4,6,8}", "iterations": iters,
                   "graph_replayed_steps": replays[0],
                   "union_ms_per_run": union_ms[0]},
        "one_at_a_time": {"value": alone, "unit": UNIT, "graphs": len(sample),
                          "seconds": a_secs,
                          "note": "single-instance API, each graph alone (same graphs, run to "
                                  "stabilisation once as warm-up, then timed), handle creation "
                                  "not timed"},
        "speedup_vs_one_at_a_time": batched / alone,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# served workload: a Poisson stream of jobs through the job server
# ---------------------------------------------------------------------------
def served_specs(count, pool, rate, seed=2025):
    """Jobs of the stream: arrival time (Poisson, `rate` per second), a graph
    of the pool and log2m in {4, 6, 8}. Pool graphs: node counts log-uniform in
    [10^3, 10^7]; even ones R-MAT (.57,.19,.19,.05) with arcs per node uniform in
    [4, 32] (2^scale nodes), odd ones web-like (mean out-degree 12)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    graphs = []
    for i in range(pool):
        n = int(round(10 ** rng.uniform(3.0, 7.0)))
        if i % 2 == 0:
            graphs.append(("rmat", int(round(np.log2(n))), int(rng.integers(4, 33)), 100 + i))
        else:
            graphs.append(("weblike", n, 12, 100 + i))
    t, jobs = 0.0, []
    for _ in range(count):
        t += rng.exponential(1.0 / rate)
        jobs.append((t, int(rng.integers(0, pool)), int(rng.choice([4, 6, 8]))))
    return graphs, jobs


def served_stream(server, graphs, jobs):
    """Submits `jobs` (arrival time, pool graph, log2m) on schedule and waits
    for all of them; returns (wall seconds, job infos, submission lateness)."""
    t0 = time.perf_counter()
    ids, sub_t = [], []
    for at, gi, l2m in jobs:
        delay = t0 + at - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        sub_t.append(time.perf_counter())
        # the pool graphs outlive the run, so jobs borrow them (no host copy
        # on the submitting thread: arrivals stay on schedule)
        ids.append(server.submit(graphs[gi], l2m, sum_of_distances=True, sum_of_inverse_distances=True,
                                 borrow=True))
    for j in ids:
        server.wait(j)
    wall = time.perf_counter() - t0
    infos = [server.info(j) for j in ids]
    for j in ids:
        server.release(j)
    late_ms = 1e3 * max(0.0, max(sub - (t0 + at) for sub, (at, _, _) in zip(sub_t, jobs)))
    return wall, infos, late_ms


def run_served(args):
    import numpy as np
    import hyperball_gb300 as hb
    from concurrent.futures import ThreadPoolExecutor

    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    gspecs, jobs = served_specs(args.jobs, args.pool, args.rate)

    def make(sp):
        kind, size, deg, seed = sp
        if kind == "rmat":
            return hb.Graph.rmat(size, deg, seed=seed)
        return hb.Graph.weblike(size, seed=seed)

    with ThreadPoolExecutor(max_workers=host_cores()) as ex:
        graphs = list(ex.map(make, gspecs))
    server = hb.HyperBallServer(max_active=args.max_active, setup_threads=args.setup_threads,
                                union_sm_reserve=args.union_sm_reserve)
    # warm-up: one job of each log2m
    for l2m in (4, 6, 8):
        j = server.submit(graphs[0], l2m, sum_of_distances=True, sum_of_inverse_distances=True)
        server.wait(j)
        server.release(j)

    def summary(wall, infos, late_ms, jobs):
        lat = np.array([i["latency_ms"] for i in infos])
        units = sum(i["register_updates"] for i in infos)
        return {"value": units / wall, "unit": UNIT, "jobs": len(jobs), "wall_s": wall,
                "jobs_per_s": len(jobs) / wall,
                "latency_ms": {"p50": float(np.percentile(lat, 50)),
                               "p99": float(np.percentile(lat, 99)), "max": float(lat.max())},
                "queue_ms_p50": float(np.percentile([i["queue_ms"] for i in infos], 50)),
                "max_submit_lateness_ms": late_ms,
                "arrival_span_s": jobs[-1][0] if jobs else 0.0}

    st0 = server.stats()
    wall, infos, late = served_stream(server, graphs, jobs)
    main_run = summary(wall, infos, late, jobs)
    st1 = server.stats()
    main_run["stepping"] = {k: st1[k] - st0[k] for k in st1 if k != "device_ms"}
    main_run["stepping"]["device_ms"] = {k: st1["device_ms"][k] - st0["device_ms"][k]
                                         for k in st1["device_ms"]}
    # a lower arrival rate, one the device can keep up with
    sustained = None
    if args.sustained_rate > 0:
        sjobs = served_specs(min(args.jobs, int(args.sustained_rate * 15)), args.pool,
                             args.sustained_rate)[1]
        w2, i2, l2 = served_stream(server, graphs, sjobs)
        sustained = dict(summary(w2, i2, l2, sjobs), rate=args.sustained_rate)
    server.close()

    # the same jobs one at a time: each (pool graph, log2m) pair once through
    # the single-instance API (create, run to stabilisation, results to the
    # host, destroy: a served job's work), summed over the stream's jobs
    alone_s = {}
    for _, gi, l2m in jobs:
        if (gi, l2m) in alone_s:
            continue
        g = graphs[gi]
        logic = hb.HyperLogLogBuilder(max(g.num_nodes, 1)).log_2_num_reg(l2m).build()
        t = time.perf_counter()
        h = (hb.HyperBallBuilder.new(g, logic).transpose_on_device(True)
             .sum_of_distances(True).sum_of_inverse_distances(True).build())
        h.run_until_done()
        if h.iteration:
            h.neighborhood_function()
            h.sum_of_distances()
            h.harmonic_centralities()
        h.close()
        alone_s[(gi, l2m)] = time.perf_counter() - t
    alone_total = sum(alone_s[(gi, l2m)] for _, gi, l2m in jobs)
    units = sum(i["register_updates"] for i in infos)
    line = {
        "metric": METRIC + " (served)", "value": main_run["value"], "unit": UNIT, "n_gpus": 1,
        "steps": 1, "warmup": 3, "ms_per_step": 1e3 * wall, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"{len(jobs)} jobs, Poisson arrivals at {args.rate}/s",
                   "graphs": f"{len(graphs)} pool graphs, n log-uniform in [1e3, 1e7]; R-MAT with "
                             "arcs/node U[4,32] or web-like; log2m in {4,6,8}",
                   "budget_bytes": 150 * 10**9, "max_active": args.max_active,
                   "arcs_per_job_mean": float(np.mean([graphs[gi].num_arcs for _, gi, _ in jobs])),
                   "serving": "continuous batching: one union launch per step for every running job"},
        "at_rate": main_run,
        "sustained": sustained,
        "one_at_a_time": {"value": units / alone_total, "unit": UNIT, "seconds": alone_total,
                          "note": "the stream's jobs run one after another through the "
                                  "single-instance API (create, run, results, destroy), each "
                                  "(graph, log2m) pair timed once"},
        "speedup_vs_one_at_a_time": main_run["value"] / (units / alone_total),
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# breadth-first visit of the web-like graph (the reference's ParFair)
# ---------------------------------------------------------------------------
def run_visit(args):
    """One step = one visit from node 0 of the web-like graph (every node it
    reaches, no filter), after a reset; the unit is the arc examined (each
    arc of every visited node: the reference's Unknown and Known events)."""
    import numpy as np
    import torch
    import hyperball_gb300 as hb

    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    torch.cuda.set_device(0)
    g = hb.Graph.weblike(1 << args.log2n)
    stream = torch.cuda.Stream()
    v = hb.ParFair(g, stream=stream.cuda_stream)
    for _ in range(args.warmup):
        v.reset()
        nodes, _, _, st = v.par_visit([0])
    off = np.asarray(g.offsets)
    arcs = int(np.sum(off[nodes.astype(np.int64) + 1] - off[nodes.astype(np.int64)]))
    secs = []
    for _ in range(args.steps):
        v.reset()
        torch.cuda.synchronize()
        t = time.perf_counter()
        _, _, _, st = v.par_visit([0])
        torch.cuda.synchronize()
        secs.append(time.perf_counter() - t)
    ms = 1e3 * sum(secs) / len(secs)
    device_ms = st["device_ms"]
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import hbo
        o = hbo.OracleVisit(g.offsets, g.successors)
        threads = os.cpu_count() or 1
        t = time.perf_counter()
        on = o.par_visit([0], threads=threads)[0]
        dt = time.perf_counter() - t
        if len(on) != st["visited"]:
            raise RuntimeError("the oracle's visit reached another number of nodes")
        cpu = {"value": arcs / dt, "unit": "arcs/s", "cores": threads, "kind": "port",
               "sample": f"fair parallel breadth-first visit (par_fair.rs restated) on {threads} threads, "
                         f"the same visit, {dt:.2f} s"}
    line = {
        "metric": "breadth-first visit arcs examined/s", "value": arcs / (device_ms / 1e3),
        "unit": "arcs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": device_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"weblike-2^{args.log2n} breadth-first visit from node 0",
                   "nodes": g.num_nodes, "arcs": g.num_arcs, "visited": st["visited"],
                   "levels": st["levels"], "arcs_examined": arcs,
                   "note": "value: device time of the visit's kernels (last step); e2e: the "
                           "whole call with the events (nodes, preds, distances) on the host"},
        "e2e": {"value": arcs / (ms / 1e3), "unit": "arcs/s", "h2d_bytes_per_step": 8,
                "d2h_bytes_per_step": 12 * st["visited"], "ms_per_step": ms},
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_sumsweep(args):
    """One step = ExactSumSweep RadiusDiameter (the radius, the diameter and
    their vertices) of the web-like graph with 2^log2n nodes (default 2^20)
    through the public call, graph and transpose from host memory."""
    import torch
    import hyperball_gb300 as hb

    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    torch.cuda.set_device(0)
    g = hb.Graph.weblike(1 << args.log2n)
    t = g.transpose()
    level = "radius_diameter"
    for _ in range(args.warmup):
        r = hb.exact_sum_sweep(g, t, level=level)
    secs, dev = [], []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = hb.exact_sum_sweep(g, t, level=level)
        secs.append(time.perf_counter() - t0)
        dev.append(r["device_ms"])
    ms = 1e3 * sum(secs) / len(secs)
    fields = ("diameter", "radius", "diametral_vertex", "radial_vertex", "radius_iterations",
              "diameter_iterations")
    cpu, parity = None, None
    if not args.no_cpu_baseline:
        from oracle import hbo
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        o = hbo.sum_sweep(g.offsets, g.successors, t.offsets, t.successors, level=level, threads=threads)
        dt = time.perf_counter() - t0
        if any(o[f] != r[f] for f in fields):
            raise RuntimeError("ExactSumSweep differs from the oracle")
        parity = {"oracle": "oracle/sum_sweep_oracle.cpp", "result": "match",
                  "checked": ", ".join(fields)}
        cpu = {"value": 1.0 / dt, "unit": "runs/s", "cores": threads, "kind": "port",
               "sample": f"ExactSumSweep restated (computer.rs), fair parallel visits on {threads} "
                         f"threads, one run, {dt:.1f} s"}
    line = {
        "metric": "ExactSumSweep RadiusDiameter runs/s", "value": 1e3 / ms,
        "unit": "runs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"weblike-2^{args.log2n} ExactSumSweep RadiusDiameter (directed)",
                   "nodes": g.num_nodes, "arcs": g.num_arcs, "diameter": r["diameter"],
                   "radius": r["radius"], "visits": r["sweeps"],
                   "diameter_iterations": r["diameter_iterations"],
                   "note": "value and e2e: the whole call from host CSR arrays (the largest "
                           "component from two device visits, the other components and the "
                           "component arcs on the host, visits and bounds on the device); "
                           "device_ms: the visits and bounds"},
        "device_ms": sum(dev) / len(dev),
        "e2e": {"value": 1e3 / ms, "unit": "runs/s",
                "h2d_bytes_per_step": 2 * (8 * (g.num_nodes + 1) + 4 * g.num_arcs),
                "d2h_bytes_per_step": 64, "ms_per_step": ms},
        "cpu_baseline": cpu, "parity": parity,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "served":
        return run_served(args)
    if args.workload == "visit":
        return run_visit(args)
    if args.workload == "sumsweep":
        return run_sumsweep(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
