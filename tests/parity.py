"""Lock-step comparison of the GPU HyperBall with the CPU oracle.

Mirrors the reference's in-crate test (src/algo/hyperball/hyperball_impl.rs:
1263-1322), which after every iteration asserts that both counter arrays of
the parallel HyperBall equal those of the sequential recurrence: here, after
every iteration, both GPU arrays must equal the oracle's byte for byte, the
iteration statistics must be identical, and the neighbourhood function and
per-node sums must agree within 1e-12 relative (only summation order differs).
"""
import numpy as np

NF_RTOL = 1e-12
SUM_RTOL = 1e-12


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.abs(a - b)
    scale = np.maximum(np.abs(a), np.abs(b))
    return np.where(scale > 0, d / np.where(scale > 0, scale, 1.0), d)


def assert_close(a, b, rtol, what):
    e = rel_err(a, b)
    if e.size and e.max() > rtol:
        i = int(np.argmax(e))
        raise AssertionError(f"{what}: rel err {e[i]:.3e} at {i} ({a[i]!r} vs {b[i]!r})")


def lockstep(hb, oracle, g, log2m, hash_kind=0, seed=0, transpose=None, sod=True, harm=True,
             transpose_on_device=False, buckets=None, max_iters=10_000, check_next=True,
             discounts=(), tma=False, far_rows=None, variant=None, graphs=True, warm_runs=0,
             weights=None, weight_seed=0):
    """Runs GPU and oracle side by side; returns (gpu, oracle, stats list)."""
    hasher = hb.JenkinsHasher(seed) if hash_kind == 1 else hb.DefaultHasher()
    logic = hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(log2m).build_hasher(hasher).build()
    if transpose is not None:
        b = hb.HyperBallBuilder.with_transpose(g, transpose, logic)
    else:
        b = hb.HyperBallBuilder.new(g, logic).transpose_on_device(transpose_on_device)
    b = b.sum_of_distances(sod).sum_of_inverse_distances(harm)
    if weights is not None:
        b = b.weights(weights, weight_seed)
    for f in discounts:
        b = b.discount_function(f)
    if buckets:
        b = b.degree_buckets(*buckets)
    b = b.tma_gather(tma, far_rows).union_variant(variant).cuda_graphs(graphs)
    gpu = b.build()
    has_t = transpose is not None or transpose_on_device
    t = transpose
    if t is None and transpose_on_device:
        t = g.transpose()
    orc = oracle.OracleHyperBall(
        g.offsets, g.successors, log2m, hash_kind=hash_kind, seed=seed,
        t_offsets=t.offsets if has_t else None, t_successors=t.successors if has_t else None,
        sod=sod, harm=harm, threads=1, discounts=discounts, weights=weights,
        weight_seed=weight_seed)
    for _ in range(warm_runs):
        gpu.run_until_done()  # the shapes of a finished run are replayed as CUDA graphs
    gpu.init()
    orc.init()
    np.testing.assert_array_equal(gpu.registers(0), orc.registers(0), "init current state")
    stats = []
    for it in range(max_iters):
        if it >= g.num_nodes:
            break
        sg = gpu.iterate()
        so = orc.iterate()
        stats.append((sg, so))
        for k in ("modified", "visited_arcs"):
            kg = "modified_counters" if k == "modified" else k
            assert sg[kg] == so[k], f"iteration {it}: {k} gpu {sg[kg]} oracle {so[k]}"
        for k in ("systolic", "local", "pre_local"):
            assert bool(sg[k]) == bool(so[k]), f"iteration {it}: mode {k}"
        ga, oa = gpu.registers(0), orc.registers(0)
        if not np.array_equal(ga, oa):
            bad = np.nonzero(np.any(ga != oa, axis=1))[0]
            raise AssertionError(f"iteration {it}: current state differs at {len(bad)} nodes, first {bad[:5]}")
        if check_next:
            np.testing.assert_array_equal(gpu.registers(1), orc.registers(1), f"iteration {it}: next state")
        assert_close(np.array([sg["neighborhood_function"]]), np.array([so["nf"]]), NF_RTOL,
                     f"iteration {it}: neighbourhood function")
        if so["modified"] == 0:
            break
    assert_close(gpu.neighborhood_function(), orc.neighborhood_function(), NF_RTOL, "NF vector")
    if sod:
        assert_close(gpu.sum_of_distances(), orc.sum_of_distances(), SUM_RTOL, "sum of distances")
    if harm:
        assert_close(gpu.harmonic_centralities(), orc.harmonic_centralities(), SUM_RTOL, "harmonic")
    for i in range(len(discounts)):
        assert_close(gpu.discounted_centrality(i), orc.discounted_centrality(i), SUM_RTOL, f"discount {i}")
    assert_close(gpu.reachable_nodes(), orc.reachable_nodes(), 0.0, "reachable nodes")
    return gpu, orc, stats
