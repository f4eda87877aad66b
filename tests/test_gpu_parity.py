"""GPU parity: the CUDA HyperBall against the CPU oracle, iteration by iteration.

Bit-exact counters (both arrays), identical modified / visited counts and
modes, neighbourhood function and per-node sums within 1e-12 relative.
"""
import numpy as np
import pytest

from conftest import cnr_basename, cnr_result
from parity import assert_close, lockstep

pytestmark = pytest.mark.gpu


def test_er_1e4_log2m6_systolic(hb, oracle):
    """The CPU-runnable config: ER n=10^4, 8 successors, SplitMix64 seed 0, log2m 6."""
    g = hb.Graph.erdos_renyi(10_000, 8, 0)
    t = g.transpose()
    gpu, orc, stats = lockstep(hb, oracle, g, 6, transpose=t)
    assert any(sg["systolic"] for sg, _ in stats), "systolic iterations expected"


def test_er_1e4_log2m6_standard_only(hb, oracle):
    g = hb.Graph.erdos_renyi(10_000, 8, 0)
    gpu, orc, stats = lockstep(hb, oracle, g, 6)
    assert not any(sg["systolic"] for sg, _ in stats)


@pytest.mark.parametrize("log2m", [4, 5, 7, 8, 9, 10])
def test_er_log2m(hb, oracle, log2m):
    g = hb.Graph.erdos_renyi(3000, 5, 11 + log2m)
    lockstep(hb, oracle, g, log2m, transpose=g.transpose())


@pytest.mark.parametrize("log2m", [4, 6, 8])
def test_jenkins_hash(hb, oracle, log2m):
    g = hb.Graph.erdos_renyi(4000, 6, 3)
    lockstep(hb, oracle, g, log2m, hash_kind=1, seed=42, transpose=g.transpose())


@pytest.mark.parametrize("log2m", [4, 5, 6, 7, 8, 9])
@pytest.mark.parametrize("far_rows", [1, 300])
def test_tma_far_gathers(hb, oracle, log2m, far_rows):
    """Successors farther than far_rows ids come by TMA gathers (four per arc
    lane, the rest by plain loads): the counters stay bit-exact, in standard,
    gather-all and systolic iterations and through the medium-node path."""
    g = hb.Graph.weblike(6000, cap=200, window=512, seed=log2m)
    lockstep(hb, oracle, g, log2m, transpose_on_device=True, tma=True, far_rows=far_rows)


def test_tma_far_gathers_rmat(hb, oracle):
    g = hb.Graph.rmat(14, 8, seed=6)
    lockstep(hb, oracle, g, 6, transpose_on_device=True, tma=True)


def test_tma_wait_timeout_reports_and_recovers(hb, oracle):
    """The far-gather mbarrier wait is bounded. With bytes added to every
    expected count the wait cannot complete: the iteration must return
    HB_ERR_TIMEOUT (after the kernel drained its copies), and the same handle
    must then run a clean, oracle-exact run after hb_init."""
    g = hb.Graph.weblike(6000, cap=200, window=512, seed=3)
    logic = hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(6).build()
    gpu = (hb.HyperBallBuilder.new(g, logic).transpose_on_device(True).sum_of_distances(True)
           .tma_gather(True, 1).cuda_graphs(False).build())
    gpu.debug_far_wait(polls=64, extra_tx_bytes=16)
    gpu.init()
    with pytest.raises(hb.HyperBallError) as ei:
        gpu.iterate()
    assert ei.value.code == hb.HB_ERR_TIMEOUT
    gpu.debug_far_wait(0, 0)
    gpu.run_until_done()
    orc = oracle.OracleHyperBall(g.offsets, g.successors, 6, sod=True,
                                 t_offsets=g.transpose().offsets,
                                 t_successors=g.transpose().successors)
    orc.run_until_done()
    assert gpu.iteration == orc.iteration
    np.testing.assert_array_equal(gpu.registers(0), orc.registers(0))
    assert_close(gpu.sum_of_distances(), orc.sum_of_distances(), 1e-12, "sum of distances")


N_VARIANTS = 10
STAGED = (5, 6, 7, 8)


@pytest.mark.parametrize("log2m", [4, 6, 8])
@pytest.mark.parametrize("variant", range(N_VARIANTS))
def test_union_variants(hb, oracle, log2m, variant):
    """Every union-kernel variant (prefetch into L1 or L2, 3 or 4 blocks per
    SM, the staged kernel with one or two loads in flight) gives the oracle's
    counters, in every kind of iteration."""
    assert hb.union_variant_count() == N_VARIANTS
    g = hb.Graph.weblike(20_000, cap=3000, window=256, seed=variant)
    lockstep(hb, oracle, g, log2m, transpose_on_device=True, variant=variant)


@pytest.mark.parametrize("log2m", [5, 7, 9, 10])
@pytest.mark.parametrize("variant", STAGED)
def test_staged_kernel_log2m(hb, oracle, log2m, variant):
    """The staged kernel at every chunk width (1 to 16 lanes per counter),
    light and medium items, standard iterations only (no transpose)."""
    g = hb.Graph.weblike(9000, cap=1500, window=128, seed=log2m)
    lockstep(hb, oracle, g, log2m, variant=variant, buckets=(16, 512))


def _hub_graph(hb, seed):
    """A web-like graph plus hubs of 32,768 to about 60,000 successors: the
    heavy kernel splits every node above 32,768 arcs into segments."""
    rng = np.random.default_rng(seed)
    base = hb.Graph.weblike(60_000, cap=500, window=256, seed=seed)
    off = np.asarray(base.offsets).astype(np.int64)
    suc = np.asarray(base.successors).astype(np.uint32)
    n = base.num_nodes
    rows = [suc[off[v]:off[v + 1]] for v in range(n)]
    for v, d in ((11, 59_000), (400, 40_000), (12_345, 32_769), (50_000, 32_000), (7, 16_384)):
        extra = rng.choice(n, size=d, replace=False).astype(np.uint32)
        rows[v] = np.unique(np.concatenate([rows[v], extra]))
    deg = np.array([len(r) for r in rows], dtype=np.uint64)
    offsets = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint64)
    return hb.Graph.from_csr(offsets, np.concatenate(rows).astype(np.uint32))


@pytest.mark.parametrize("log2m", [4, 6, 8, 10])
def test_heavy_nodes_split_into_segments(hb, oracle, log2m):
    """Heavy nodes above 32,768 arcs run as segments on several CTAs whose
    partial counters the last one merges: the oracle's counters in standard
    (merging every or only modified successors) and systolic iterations."""
    g = _hub_graph(hb, seed=log2m)
    assert int(np.max(np.diff(np.asarray(g.offsets).astype(np.int64)))) > 50_000
    lockstep(hb, oracle, g, log2m, transpose_on_device=True, buckets=(64, 4096))


@pytest.mark.parametrize("variant", STAGED)
def test_staged_kernel_filtered_rmat(hb, oracle, variant):
    """R-MAT leaves many counters unchanged, so standard iterations merge only
    modified successors (the filtered path of the staged kernel); items with
    more arcs than the staged ids read the rest from global memory."""
    g = hb.Graph.rmat(13, 16, seed=4)
    lockstep(hb, oracle, g, 6, variant=variant, buckets=(64, 4096))
    lockstep(hb, oracle, g, 8, transpose_on_device=True, variant=variant, buckets=(1024, 4096))


def test_autotuner_identical_results(hb):
    """The autotuner switches variants between iterations; the run equals a run
    on one fixed variant, bit for bit."""
    g = hb.Graph.weblike(1 << 19, seed=9)
    assert g.num_arcs >= 1 << 22  # large enough to be tuned
    logic = hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(6).build()

    def run(variant, runs):
        h = (hb.HyperBallBuilder.new(g, logic).transpose_on_device(True)
             .sum_of_distances(True).sum_of_inverse_distances(True).union_variant(variant).build())
        used = set()
        for _ in range(runs):
            h.run_until_done()
            used |= {s["union_variant"] for s in h.iteration_stats()}
        out = (h.registers(0), h.neighborhood_function(), h.sum_of_distances(),
               h.harmonic_centralities(), [s["modified_counters"] for s in h.iteration_stats()],
               h.union_variants_chosen())
        h.close()
        return out, used

    fixed, used0 = run(0, 1)
    assert used0 == {0}
    tuned, used = run(None, 2)
    assert len(used) > 1, used
    chosen = tuned[5]
    assert chosen[0] >= 0 and chosen[2] >= 0, chosen
    np.testing.assert_array_equal(tuned[0], fixed[0])
    np.testing.assert_array_equal(tuned[1], fixed[1])
    assert tuned[4] == fixed[4]
    np.testing.assert_array_equal(tuned[2], fixed[2])
    np.testing.assert_array_equal(tuned[3], fixed[3])


@pytest.mark.parametrize("graphs", [False, True])
def test_cuda_graph_iterations(hb, oracle, graphs):
    """After a first run, the iterations of the next run are replayed from
    captured CUDA graphs (standard, first systolic and systolic shapes;
    discount factors and 1/d from device memory) and match the oracle exactly
    as directly launched ones do."""
    g = hb.Graph.weblike(30_000, cap=2000, window=256, seed=4)
    gpu, orc, stats = lockstep(hb, oracle, g, 6, transpose_on_device=True, graphs=graphs,
                               discounts=(lambda d: 1.0 / d, lambda d: 0.5 ** d), warm_runs=1)
    replays = [sg["from_graph"] for sg, _ in stats]
    if graphs:
        assert all(replays), replays
        assert any(sg["systolic"] for sg, _ in stats)
        assert all(sg["kernel_launches"] > 0 for sg, _ in stats)
    else:
        assert not any(replays)


def test_degree_bucket_tuner(hb):
    """The bucket autotuner returns one of its candidate pairs, and a handle
    built with it gives the same registers and sums as the default buckets."""
    g = hb.Graph.weblike(1 << 16, cap=20_000, window=512, seed=3)
    logic = hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(6).build()
    small, medium, ms = hb.tune_degree_buckets(g, logic, iterations=3)
    assert small in (32, 64, 128, 256, 512, 1024) and medium in (4096, 16384, 65536) and ms > 0

    def run(buckets):
        b = hb.HyperBallBuilder.new(g, logic).transpose_on_device(True).sum_of_distances(True)
        if buckets:
            b = b.degree_buckets(*buckets)
        h = b.build()
        h.run_until_done()
        out = (h.registers(0), h.sum_of_distances(), h.neighborhood_function())
        h.close()
        return out

    tuned, default = run((small, medium)), run(None)
    np.testing.assert_array_equal(tuned[0], default[0])
    assert_close(tuned[1], default[1], 1e-12, "sum of distances")
    assert_close(tuned[2], default[2], 1e-12, "neighbourhood function")


def test_transpose_on_device(hb, oracle):
    g = hb.Graph.rmat(12, 8, seed=5)
    lockstep(hb, oracle, g, 6, transpose_on_device=True)


@pytest.mark.parametrize("buckets", [(0, 0), (1, 2), (4, 16), (1 << 30, 1 << 30)])
def test_degree_buckets(hb, oracle, buckets):
    """Every node through the group, warp or CTA path gives the same counters."""
    g = hb.Graph.weblike(20_000, cap=3000, window=64, seed=7)
    lockstep(hb, oracle, g, 6, transpose=g.transpose(), buckets=buckets)


def test_heavy_hub(hb, oracle):
    """A hub with thousands of successors goes through the CTA path (log2m 8)."""
    n = 6000
    rng = np.random.default_rng(0)
    rows = []
    for v in range(n):
        if v == 17:
            s = np.arange(n, dtype=np.uint32)  # includes a self-loop
        else:
            s = np.unique(rng.integers(0, n, size=rng.integers(0, 5)).astype(np.uint32))
        rows.append(s)
    off = np.zeros(n + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(r) for r in rows])
    g = hb.Graph.from_csr(off, np.concatenate(rows))
    lockstep(hb, oracle, g, 8, transpose=g.transpose(), buckets=(4, 64))


def test_discount_functions(hb, oracle):
    g = hb.Graph.erdos_renyi(2000, 4, 9)
    lockstep(hb, oracle, g, 6, transpose=g.transpose(),
             discounts=(lambda d: 1.0 / (d * d), lambda d: 0.5 ** d))


@pytest.mark.parametrize("log2m,hash_kind", [(4, 0), (6, 0), (8, 1)])
def test_node_weights(hb, oracle, log2m, hash_kind):
    """Node weights (HB:1165-1174): node v starts with w[v] added values
    instead of its own id. The reference draws them from a thread RNG (not
    reproducible); here value k of node v is SplitMix64 step k from
    weight_seed ^ v * golden, on the GPU (k_init) and in the oracle alike.
    Weights of 0 leave a counter empty; large ones fill many registers."""
    g = hb.Graph.erdos_renyi(3000, 5, 21 + log2m)
    rng = np.random.default_rng(log2m)
    w = rng.integers(0, 6, size=g.num_nodes).astype(np.uint64)
    w[::97] = 0
    w[5] = 3000
    for seed in (0, 12345):
        lockstep(hb, oracle, g, log2m, hash_kind=hash_kind, seed=42 * hash_kind,
                 transpose=g.transpose(), weights=w, weight_seed=seed)


def test_edge_cases(hb, oracle):
    # one node with a self-loop
    g = hb.Graph.from_csr(np.array([0, 1], dtype=np.uint64), np.array([0], dtype=np.uint32))
    lockstep(hb, oracle, g, 6)
    # no arcs at all
    g = hb.Graph.from_csr(np.zeros(51, dtype=np.uint64), np.zeros(0, dtype=np.uint32))
    lockstep(hb, oracle, g, 4, transpose=g.transpose())
    # a path: many iterations, ragged sizes (n not a multiple of 32)
    n = 77
    off = np.concatenate([np.arange(n, dtype=np.uint64), [n - 1]]).astype(np.uint64)
    g = hb.Graph.from_csr(off, np.arange(1, n, dtype=np.uint32))
    lockstep(hb, oracle, g, 5, transpose=g.transpose())


def test_run_api_matches_oracle(hb, oracle):
    g = hb.Graph.erdos_renyi(5000, 8, 0)
    t = g.transpose()
    logic = hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(6).build()
    gpu = (hb.HyperBallBuilder.with_transpose(g, t, logic)
           .sum_of_distances(True).sum_of_inverse_distances(True).build())
    orc = oracle.OracleHyperBall(g.offsets, g.successors, 6, t_offsets=t.offsets,
                                 t_successors=t.successors, sod=True, harm=True)
    # upper bound and threshold stops (HB:541, HB:572-577)
    for ub, thr in ((3, None), (1000, 0.01), (1000, None)):
        gpu.run(ub, thr)
        orc.run(ub, thr)
        assert gpu.iteration == orc.iteration
        np.testing.assert_array_equal(gpu.registers(), orc.registers())
        assert_close(gpu.neighborhood_function(), orc.neighborhood_function(), 1e-12, "nf")
        for name in ("sum_of_distances", "harmonic_centralities", "closeness_centrality",
                     "lin_centrality", "nieminen_centrality", "reachable_nodes"):
            assert_close(getattr(gpu, name)(), getattr(orc, name)(), 1e-12, name)
        # caller buffers and single-node lookups give the same values
        buf = np.full(g.num_nodes, np.nan)
        assert gpu.sum_of_distances(out=buf) is buf
        assert_close(buf, orc.sum_of_distances(), 1e-12, "sum_of_distances(out=)")
        reach = orc.reachable_nodes()
        for v in (0, 17, g.num_nodes - 1):
            assert_close(np.array([gpu.reachable_nodes_from(v)]), reach[v:v + 1], 1e-12, "from")
    with pytest.raises(ValueError):
        gpu.harmonic_centralities(out=np.zeros(g.num_nodes, dtype=np.float32))


def test_cached_memory_release(hb, oracle):
    """Handles reuse the library's pooled device memory; returning it to the
    device leaves later handles correct."""
    g = hb.Graph.rmat(11, 8, seed=9)
    first, _, _ = lockstep(hb, oracle, g, 6, transpose_on_device=True)
    hb.release_cached_memory(0)
    again, _, _ = lockstep(hb, oracle, g, 6, transpose_on_device=True)
    np.testing.assert_array_equal(first.registers(), again.registers())
    with pytest.raises(hb.InvalidArgumentError):
        hb.release_cached_memory(1 << 20)


def test_errors(hb):
    g = hb.Graph.erdos_renyi(100, 3, 1)
    logic = hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(6).build()
    h = hb.HyperBallBuilder.new(g, logic).build()
    with pytest.raises(hb.NotRunError):
        h.neighborhood_function()
    h.run_until_done()
    with pytest.raises(hb.NotRequestedError):
        h.sum_of_distances()
    with pytest.raises(hb.NotRequestedError):
        h.discounted_centrality(0)
    bad = hb.Graph.from_csr(np.array([0, 1], dtype=np.uint64), np.array([5], dtype=np.uint32))
    with pytest.raises(hb.InvalidArgumentError):
        hb.HyperBallBuilder.new(bad, logic).build()
    with pytest.raises(hb.InvalidArgumentError):
        hb.HyperBallBuilder.new(g, logic).union_variant(hb.union_variant_count()).build()


@pytest.mark.skipif(cnr_basename() is None, reason="cnr-2000 fixture not present")
def test_cnr2000_java_goldens(hb, oracle):
    """tests/test_hyperball.rs:221-302 on the GPU: log2m 8, Jenkins(42), to
    stabilisation; five centralities within 1e-6 of the Java results."""
    g = hb.Graph.load_bvgraph(cnr_basename())
    gt = hb.Graph.load_bvgraph(cnr_basename(transpose=True))
    logic = (hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(8)
             .build_hasher(hb.JenkinsHasher(42)).build())
    h = (hb.HyperBallBuilder.with_transpose(g, gt, logic)
         .sum_of_distances(True).sum_of_inverse_distances(True).build())
    h.run_until_done()
    for name, fn in (("sum_of_distances", h.sum_of_distances),
                     ("harmonic_centrality", h.harmonic_centralities),
                     ("lin_centrality", h.lin_centrality),
                     ("closeness_centrality", h.closeness_centrality),
                     ("nieminen_centrality", h.nieminen_centrality)):
        p = cnr_result(name)
        if p is None:
            pytest.skip("Java golden results not present")
        exp = np.fromfile(p, dtype=">f4").astype(np.float64)
        act = fn()
        d = np.abs(exp - act)
        rel = np.where(exp != 0, d / np.where(exp != 0, exp, 1.0), d)
        assert rel.max() < 1e-6, f"{name}: max rel {rel.max()}"


@pytest.mark.skipif(cnr_basename() is None, reason="cnr-2000 fixture not present")
def test_cnr2000_lockstep_log2m6(hb, oracle):
    """The reference's in-crate test (HB:1263-1322): cnr-2000, log2m 6, default
    hasher, systolic and local modes, both arrays checked every iteration."""
    g = hb.Graph.load_bvgraph(cnr_basename())
    gt = hb.Graph.load_bvgraph(cnr_basename(transpose=True))
    _, _, stats = lockstep(hb, oracle, g, 6, transpose=gt, sod=False, harm=False)
    assert any(sg["local"] for sg, _ in stats)
