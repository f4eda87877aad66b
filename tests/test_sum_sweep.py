"""ExactSumSweep: the oracle (a restatement of src/algo/exact_sum_sweep/) on
the cases of the reference's own tests (tests/test_exact_sum_sweep.rs,
tests/test_undir_sum_sweep.rs) and against the definition (one breadth-first
visit per node) on random graphs; then the device implementation
(hb_exact_sum_sweep) against the oracle, field by field."""
import numpy as np
import pytest

from oracle import hbo

NC = hbo.NOT_COMPUTED


def csr(n, arcs):
    """CSR of a graph on n nodes with the given arcs (rows sorted, duplicates
    removed, as the reference's BTreeGraph / VecGraph hold them)."""
    arcs = sorted(set((int(a), int(b)) for a, b in arcs))
    off = np.zeros(n + 1, dtype=np.uint64)
    for a, _ in arcs:
        off[a + 1] += 1
    off = np.cumsum(off).astype(np.uint64)
    suc = np.array([b for _, b in arcs], dtype=np.uint32)
    return off, suc


def transpose(n, arcs):
    return csr(n, [(b, a) for a, b in arcs])


def directed(n, arcs, level="all", radial=None):
    off, suc = csr(n, arcs)
    toff, tsuc = transpose(n, arcs)
    return hbo.sum_sweep(off, suc, toff, tsuc, level=level, radial=radial)


def undirected(n, arcs, level="all"):
    off, suc = csr(n, arcs)
    return hbo.sum_sweep(off, suc, level=level)


def random_arcs(n, p, seed, symmetric=False):
    rng = np.random.default_rng(seed)
    m = rng.random((n, n)) < p
    np.fill_diagonal(m, False)
    if symmetric:
        m = m | m.T
    a, b = np.nonzero(m)
    return list(zip(a.tolist(), b.tolist()))


# ---- the reference's directed cases (tests/test_exact_sum_sweep.rs) ----------

def test_directed_path():  # test_exact_sum_sweep.rs:24-51
    r = directed(3, [(0, 1), (1, 2), (2, 1), (1, 0)])
    assert list(r["forward_eccentricities"]) == [2, 1, 2]
    assert r["backward_eccentricities"][0] == 2
    assert (r["diameter"], r["radius"], r["radial_vertex"]) == (2, 1, 1)
    assert r["diametral_vertex"] in (0, 2)


def test_directed_many_scc():  # test_exact_sum_sweep.rs:53-82
    arcs = [(0, 1), (1, 0), (1, 2), (2, 1), (6, 2), (2, 6), (3, 4), (4, 3), (4, 5), (5, 4),
            (0, 3), (0, 4), (1, 5), (1, 4), (2, 5)]
    r = directed(7, arcs)
    assert (r["radius"], r["radial_vertex"]) == (2, 1)


def test_directed_lozenge():  # test_exact_sum_sweep.rs:84-104
    r = directed(4, [(0, 1), (1, 0), (0, 2), (1, 3), (2, 3)], level="radius")
    assert r["radius"] == 2 and r["radial_vertex"] in (0, 1)


def test_directed_many_paths_with_radial_vertices():  # test_exact_sum_sweep.rs:106-143
    arcs = [(0, 1), (1, 2), (2, 3), (3, 4), (5, 6), (6, 7), (7, 8), (8, 9), (9, 10), (10, 18),
            (11, 12), (13, 14), (14, 15), (15, 16), (16, 17)]
    radial = np.zeros(19, dtype=np.uint8)
    radial[[16, 8]] = 1
    r = directed(19, arcs, radial=radial)
    assert (r["diameter"], r["radius"], r["radial_vertex"]) == (6, 1, 16)
    assert r["diametral_vertex"] in (5, 18)


@pytest.mark.parametrize("size", [3, 5, 7])
def test_directed_cycle(size):  # test_exact_sum_sweep.rs:145-172
    r = directed(size, [(i, (i + 1) % size) for i in range(size)], level="radius_diameter")
    assert (r["diameter"], r["radius"]) == (size - 1, size - 1)


@pytest.mark.parametrize("size", [10, 50, 100])
def test_directed_clique(size):  # test_exact_sum_sweep.rs:174-209
    arcs = [(i, j) for i in range(size) for j in range(size) if i != j]
    picks = np.random.default_rng(size).integers(0, size, 3)
    radial = np.zeros(size, dtype=np.uint8)
    radial[picks] = 1
    r = directed(size, arcs, radial=radial)
    assert (r["forward_eccentricities"] == 1).all()
    assert r["radial_vertex"] in picks.tolist()


def test_directed_no_arcs():  # test_exact_sum_sweep.rs:211-225, 277-290
    for n in (100, 2):
        r = directed(n, [])
        assert (r["radius"], r["diameter"]) == (0, 0)


def test_directed_sparse():  # test_exact_sum_sweep.rs:227-237
    r = directed(66, [(10, 32), (10, 65), (65, 10), (21, 44)])
    assert (r["radius"], r["radial_vertex"]) == (1, 10)


def test_directed_no_radial_vertices():  # test_exact_sum_sweep.rs:239-265
    r = directed(2, [(0, 1)], radial=np.zeros(2, dtype=np.uint8))
    assert r["radius"] == NC


def test_empty_graph_has_no_output():  # test_exact_sum_sweep.rs:267-275
    assert directed(0, []) is None
    assert undirected(0, [], level="radius") is None


@pytest.mark.parametrize("d", [2, 3, 4])
def test_directed_random_against_definition(d):  # test_exact_sum_sweep.rs:292-331
    n = 100
    arcs = random_arcs(n, d / 100.0, seed=d)
    off, suc = csr(n, arcs)
    toff, tsuc = transpose(n, arcs)
    r = hbo.sum_sweep(off, suc, toff, tsuc)
    np.testing.assert_array_equal(r["forward_eccentricities"], hbo.eccentricities(off, suc))
    np.testing.assert_array_equal(r["backward_eccentricities"], hbo.eccentricities(toff, tsuc))


# ---- the selections' tie rules (tests/test_math.rs, utils/argmax.rs, argmin.rs) --

def _sel(v, t=None, keep=None, maximize=True):
    k = None if keep is None else [1 if keep(i, x) else 0 for i, x in enumerate(v)]
    return hbo.arg_select(v, t, k, maximize)


def test_argmax_cases():  # test_math.rs:13-70, argmax.rs doc examples
    assert _sel([]) is None
    assert _sel([0]) == 0
    assert _sel([2, 1, 5, 3]) == 2
    assert _sel([2, 5, 1, 3, 5]) == 1
    assert _sel([], [], lambda i, e: True) is None
    assert _sel([2, 1, 5, 3, 1], [5, 4, 3, 2, 1], lambda i, e: False) is None
    assert _sel([0], [0], lambda i, e: True) == 0
    assert _sel([1, 2, 3, 4, 5, 4, 3, 2, 1], list(range(1, 10)), lambda i, e: e < 4) == 6
    assert _sel([1, 2, 3, 2, 1], [1, 2, 3, 2, 1], lambda i, e: e < 3) == 1
    assert _sel([1, 2, 5, 2, 1, 2], [1, 2, 3, 4, 5, 2], lambda i, e: e < 4) == 3
    assert _sel([1, 2, 5, 2, 1, 2], [1, 1, 3, 2, 5, 2], lambda i, e: e < 4) == 3


def test_argmin_cases():  # test_math.rs:72-135
    assert _sel([], maximize=False) is None
    assert _sel([2**64 - 1], maximize=False) == 0
    assert _sel([2, 1, 5, 3], maximize=False) == 1
    assert _sel([2, 1, 5, 3, 1], maximize=False) == 1
    assert _sel([], [], lambda i, e: True, maximize=False) is None
    assert _sel([2, 1, 5, 3, 1], [5, 4, 3, 2, 1], lambda i, e: False, maximize=False) is None
    assert _sel([2**64 - 1], [2**64 - 1], lambda i, e: True, maximize=False) == 0
    assert _sel([1, 2, 3, 4, 5, 4, 3, 2, 1], list(range(9, 0, -1)), lambda i, e: e > 2, maximize=False) == 6
    assert _sel([1, 2, 3, 2, 1], [1, 2, 3, 2, 1], lambda i, e: e > 1, maximize=False) == 1


# ---- the reference's undirected cases (tests/test_undir_sum_sweep.rs) --------

def sym(arcs):
    return arcs + [(b, a) for a, b in arcs]


def test_undirected_path():  # test_undir_sum_sweep.rs:22-39
    r = undirected(3, [(0, 1), (1, 2), (2, 1), (1, 0)])
    assert list(r["forward_eccentricities"]) == [2, 1, 2]
    assert (r["diameter"], r["radius"], r["radial_vertex"]) == (2, 1, 1)


def test_undirected_star():  # test_undir_sum_sweep.rs:41-86
    r = undirected(9, sym([(0, 1), (1, 2), (0, 3), (3, 4), (0, 5), (5, 6), (0, 7), (7, 8)]))
    assert list(r["forward_eccentricities"]) == [2, 3, 4, 3, 4, 3, 4, 3, 4]
    assert (r["diameter"], r["radius"], r["radial_vertex"]) == (4, 2, 0)


def test_undirected_lozenge():  # test_undir_sum_sweep.rs:88-112
    r = undirected(4, sym([(0, 1), (0, 2), (1, 3), (2, 3)]), level="radius")
    assert r["radius"] == 2


@pytest.mark.parametrize("size", [3, 5, 7])
def test_undirected_cycle(size):  # test_undir_sum_sweep.rs:114-137
    r = undirected(size, sym([(i, (i + 1) % size) for i in range(size)]), level="radius_diameter")
    assert (r["diameter"], r["radius"]) == (size // 2, size // 2)


@pytest.mark.parametrize("size", [10, 50, 100])
def test_undirected_clique(size):  # test_undir_sum_sweep.rs:139-163
    r = undirected(size, [(i, j) for i in range(size) for j in range(size) if i != j])
    assert (r["forward_eccentricities"] == 1).all()
    assert (r["diameter"], r["radius"]) == (1, 1)


def test_undirected_no_arcs_and_sparse():  # test_undir_sum_sweep.rs:165-186
    r = undirected(100, [])
    assert (r["radius"], r["diameter"]) == (0, 0)
    r = undirected(66, sym([(10, 32), (10, 65), (21, 44)]), level="radius")
    assert r["radius"] == 1


@pytest.mark.parametrize("d", [2, 3, 4])
def test_undirected_random_against_definition(d):  # test_undir_sum_sweep.rs:195-225
    n = 100
    off, suc = csr(n, random_arcs(n, d / 100.0, seed=10 + d, symmetric=True))
    r = hbo.sum_sweep(off, suc)
    np.testing.assert_array_equal(r["forward_eccentricities"], hbo.eccentricities(off, suc))


@pytest.mark.parametrize("level", ["all", "all_forward", "radius_diameter", "diameter", "radius"])
def test_levels_agree_with_the_definition(level):
    """Every output level on graphs with many strongly connected components:
    the diameter is the largest eccentricity, the radius the smallest forward
    eccentricity of a radial vertex (the nodes that reach the largest
    component), and the reported vertices attain them."""
    for seed in range(6):
        n = 300
        arcs = random_arcs(n, 1.3 / n, seed=100 + seed)
        off, suc = csr(n, arcs)
        toff, tsuc = transpose(n, arcs)
        fe, be = hbo.eccentricities(off, suc), hbo.eccentricities(toff, tsuc)
        r = hbo.sum_sweep(off, suc, toff, tsuc, level=level)
        full = hbo.sum_sweep(off, suc, toff, tsuc, level="all")
        if level in ("all", "radius_diameter", "diameter", "all_forward"):
            assert r["diameter"] == fe.max() == be.max()
            assert fe[r["diametral_vertex"]] == r["diameter"] or be[r["diametral_vertex"]] == r["diameter"]
        if level != "diameter":
            assert r["radius"] == full["radius"]
            assert fe[r["radial_vertex"]] == r["radius"]
        if level in ("all", "all_forward"):
            np.testing.assert_array_equal(r["forward_eccentricities"], fe)
        if level == "all":
            np.testing.assert_array_equal(r["backward_eccentricities"], be)


@pytest.mark.parametrize("kind", ["weblike", "rmat", "undirected"])
def test_parallel_visits_give_the_same_result(kind):
    """The oracle with its visits as fair parallel visits on host threads
    (par_fair.rs, the visit the reference's ExactSumSweep runs; levels of
    4,096 nodes and more split among the threads) gives every field of the
    sequential run."""
    if kind == "weblike":
        g = hbo.OracleGraph.weblike(1 << 16)
    elif kind == "rmat":
        g = hbo.OracleGraph.rmat(15, 8, 0.57, 0.19, 0.19, seed=3)
    else:
        # an R-MAT graph with each arc also reversed
        e = hbo.OracleGraph.rmat(15, 8, 0.57, 0.19, 0.19, seed=5)
        n = e.num_nodes
        src = np.repeat(np.arange(n, dtype=np.uint64), np.diff(e.offsets.astype(np.int64)))
        dst = e.successors.astype(np.uint64)
        key = np.unique(np.concatenate([src * n + dst, dst * n + src]))
        key = key[key // n != key % n]
        off = np.zeros(n + 1, dtype=np.uint64)
        off[1:] = np.cumsum(np.bincount((key // n).astype(np.int64), minlength=n))
        suc = (key % n).astype(np.uint32)
    if kind != "undirected":
        t = g.transpose()
        args = (g.offsets, g.successors, t.offsets, t.successors)
    else:
        args = (off, suc)
    for level in ("radius_diameter", "radius"):
        one = hbo.sum_sweep(*args, level=level)
        for threads in (3, 8):
            assert hbo.sum_sweep(*args, level=level, threads=threads) == one, (level, threads)


# ---- the device implementation against the oracle ---------------------------

FIELDS = ("diameter", "radius", "diametral_vertex", "radial_vertex", "radius_iterations",
          "diameter_iterations", "forward_iterations", "all_iterations")


def device_vs_oracle(off, suc, toff=None, tsuc=None, level="all", radial=None):
    import hyperball_gb300 as hb
    g = hb.Graph.from_csr(off, suc)
    t = hb.Graph.from_csr(toff, tsuc) if toff is not None else None
    want = hbo.sum_sweep(off, suc, toff, tsuc, level=level, radial=radial)
    got = hb.exact_sum_sweep(g, t, level=level, radial_vertices=radial)
    for f in FIELDS:
        assert got[f] == want[f], (f, got[f], want[f])
    for f in ("forward_eccentricities", "backward_eccentricities"):
        assert (f in got) == (f in want), f
        if f in want:
            np.testing.assert_array_equal(got[f], want[f], err_msg=f)
    return got


REFERENCE_DIRECTED = [
    (3, [(0, 1), (1, 2), (2, 1), (1, 0)], "all", None),
    (7, [(0, 1), (1, 0), (1, 2), (2, 1), (6, 2), (2, 6), (3, 4), (4, 3), (4, 5), (5, 4), (0, 3),
         (0, 4), (1, 5), (1, 4), (2, 5)], "all", None),
    (4, [(0, 1), (1, 0), (0, 2), (1, 3), (2, 3)], "radius", None),
    (19, [(0, 1), (1, 2), (2, 3), (3, 4), (5, 6), (6, 7), (7, 8), (8, 9), (9, 10), (10, 18),
          (11, 12), (13, 14), (14, 15), (15, 16), (16, 17)], "all", [16, 8]),
    (7, [(i, (i + 1) % 7) for i in range(7)], "radius_diameter", None),
    (100, [], "all", None),
    (66, [(10, 32), (10, 65), (65, 10), (21, 44)], "all", None),
    (2, [(0, 1)], "all", []),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(REFERENCE_DIRECTED)))
def test_device_reference_directed_cases(case):
    n, arcs, level, radial = REFERENCE_DIRECTED[case]
    rad = None
    if radial is not None:
        rad = np.zeros(n, dtype=np.uint8)
        rad[list(radial)] = 1
    off, suc = csr(n, arcs)
    toff, tsuc = transpose(n, arcs)
    device_vs_oracle(off, suc, toff, tsuc, level=level, radial=rad)


@pytest.mark.gpu
@pytest.mark.parametrize("level", ["all", "all_forward", "radius_diameter", "diameter", "radius"])
@pytest.mark.parametrize("seed", range(4))
def test_device_random_directed(level, seed):
    """Sparse random graphs: many strongly connected components and arcs
    between them (every step of the algorithm, all_cc_upper_bound included)."""
    n = [300, 1000, 3000, 5000][seed]
    arcs = random_arcs(n, [1.2, 1.6, 2.5, 4.0][seed] / n, seed=200 + seed)
    off, suc = csr(n, arcs)
    toff, tsuc = transpose(n, arcs)
    device_vs_oracle(off, suc, toff, tsuc, level=level)


@pytest.mark.gpu
@pytest.mark.parametrize("level", ["all", "radius_diameter", "radius"])
def test_device_undirected(level):
    for seed, (n, d) in enumerate([(9, 0), (400, 1.5), (3000, 2.2)]):
        if n == 9:
            arcs = sym([(0, 1), (1, 2), (0, 3), (3, 4), (0, 5), (5, 6), (0, 7), (7, 8)])
        else:
            arcs = random_arcs(n, d / n, seed=300 + seed, symmetric=True)
        off, suc = csr(n, arcs)
        device_vs_oracle(off, suc, level=level)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["weblike", "rmat"])
def test_device_generated_graphs(kind):
    """Generated graphs with hubs above the visit's block-per-node bound
    (4,096 arcs) and, for R-MAT, thousands of components."""
    import hyperball_gb300 as hb
    g = hb.Graph.weblike(1 << 15, cap=20_000, window=512, seed=7) if kind == "weblike" else hb.Graph.rmat(13, 8, seed=3)
    t = g.transpose()
    off, suc = np.asarray(g.offsets), np.asarray(g.successors)
    if kind == "weblike":
        assert int(np.max(np.diff(off.astype(np.int64)))) > 4096
    device_vs_oracle(off, suc, np.asarray(t.offsets), np.asarray(t.successors), level="all")
    device_vs_oracle(off, suc, np.asarray(t.offsets), np.asarray(t.successors), level="radius")


@pytest.mark.gpu
def test_device_errors():
    import hyperball_gb300 as hb
    g0 = hb.Graph.from_csr(np.zeros(1, dtype=np.uint64), np.zeros(0, dtype=np.uint32))
    with pytest.raises(hb.HyperBallError, match="Trying to build All without all eccentricities computed"):
        hb.exact_sum_sweep(g0, g0)
    with pytest.raises(hb.HyperBallError, match="without the radius computed"):
        hb.exact_sum_sweep(g0, level="radius")
    g = hb.Graph.erdos_renyi(50, 3, 1)
    h = hb.Graph.erdos_renyi(60, 3, 1)
    with pytest.raises(hb.HyperBallError, match="transpose"):
        hb.exact_sum_sweep(g, h)


REFERENCE_UNDIRECTED = [
    (3, [(0, 1), (1, 2), (2, 1), (1, 0)], "all"),
    (9, sym([(0, 1), (1, 2), (0, 3), (3, 4), (0, 5), (5, 6), (0, 7), (7, 8)]), "all"),
    (4, sym([(0, 1), (0, 2), (1, 3), (2, 3)]), "radius"),
    (7, sym([(i, (i + 1) % 7) for i in range(7)]), "radius_diameter"),
    (10, [(i, j) for i in range(10) for j in range(10) if i != j], "all"),
    (100, [], "all"),
    (66, sym([(10, 32), (10, 65), (21, 44)]), "radius"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(REFERENCE_UNDIRECTED)))
def test_device_reference_undirected_cases(case):
    """The reference's undirected cases (tests/test_undir_sum_sweep.rs):
    one component, several of distinct sizes, and only singletons (a tie
    for the largest component)."""
    n, arcs, level = REFERENCE_UNDIRECTED[case]
    off, suc = csr(n, arcs)
    device_vs_oracle(off, suc, level=level)


def test_sweep_argument_errors_need_no_device():
    """Argument errors are reported before any device work (the reference's
    assertion message for an empty graph, a transpose of another size); with
    no device, a valid call fails loudly instead of computing on the host."""
    import hyperball_gb300 as hb
    g0 = hb.Graph.from_csr(np.zeros(1, dtype=np.uint64), np.zeros(0, dtype=np.uint32))
    with pytest.raises(hb.HyperBallError, match="Trying to build All without all eccentricities computed"):
        hb.exact_sum_sweep(g0, g0)
    with pytest.raises(hb.HyperBallError, match="Trying to build Radius without the radius computed"):
        hb.exact_sum_sweep(g0, level="radius")
    g = hb.Graph.erdos_renyi(50, 3, 1)
    with pytest.raises(hb.HyperBallError, match="transpose"):
        hb.exact_sum_sweep(g, hb.Graph.erdos_renyi(60, 3, 1))
    with pytest.raises(ValueError):
        hb.exact_sum_sweep(g, g.transpose(), radial_vertices=np.zeros(3, dtype=np.uint8))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if not has_gpu:
        with pytest.raises(hb.NoDeviceError):
            hb.exact_sum_sweep(g, g.transpose())
