"""Breadth-first visits: the device visit (hb_visit_*, the reference's
ParFair, src/algo/visits/breadth_first/par_fair.rs) against the CPU oracle
(the reference's sequential visit restated, oracle/visits_oracle.cpp), with
the cases of the reference's tests/test_bfv.rs: the simple graph visited from
every root in order, the two-root seed, cnr-2000 from every root starting at
10000. Distances must be equal; a predecessor must be a node one level
closer with an arc to the node (the parallel visit may pick any of them)."""
import numpy as np
import pytest

from conftest import cnr_basename

SIMPLE_ARCS = [(0, 0), (1, 0), (1, 2), (2, 1), (2, 3), (2, 4), (2, 5), (3, 4), (4, 3), (5, 5),
               (5, 6), (5, 7), (5, 8), (6, 7), (8, 7)]


def csr_from_arcs(arcs, n):
    rows = [[] for _ in range(n)]
    for a, b in arcs:
        rows[a].append(b)
    off = np.zeros(n + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(r) for r in rows])
    succ = np.array([x for r in rows for x in sorted(set(r))], dtype=np.uint32)
    return off, succ


def correct_dists(off, succ, start):
    """tests/test_bfv.rs:19-54, restated: BFS from start, start+1, ... (mod n)."""
    n = len(off) - 1
    visits = [-1] * n
    for i in range(n):
        s = (i + start) % n
        if visits[s] != -1:
            continue
        visits[s] = 0
        cur, d = [s], 1
        while cur:
            nxt = []
            for v in cur:
                for w in succ[off[v]:off[v + 1]]:
                    if visits[w] == -1:
                        visits[w] = d
                        nxt.append(int(w))
            cur, d = nxt, d + 1
    return visits


def test_oracle_simple_graph_and_seed(oracle):
    """The oracle gives the distances the reference's tests expect."""
    off, succ = csr_from_arcs(SIMPLE_ARCS, 9)
    v = oracle.OracleVisit(off, succ)
    d = v.visit_each(np.arange(9))
    assert list(d) == correct_dists(off, succ, 0) == [0, 0, 1, 2, 2, 2, 3, 3, 3]
    off2, succ2 = csr_from_arcs([(0, 1), (1, 2), (3, 2)], 4)
    v2 = oracle.OracleVisit(off2, succ2)
    nodes, preds, dists = v2.visit([0, 3])
    d2 = np.zeros(4, dtype=np.uint64)
    d2[nodes] = dists
    assert list(d2) == [0, 1, 1, 0]  # tests/test_bfv.rs:114-130


def test_oracle_random_graph_matches_test_definition(oracle, hb):
    g = hb.Graph.erdos_renyi(3000, 2, 5)
    off, succ = np.asarray(g.offsets), np.asarray(g.successors)
    start = 1234
    roots = (np.arange(g.num_nodes) + start) % g.num_nodes
    d = oracle.OracleVisit(off, succ).visit_each(roots)
    assert list(d) == correct_dists(off, succ, start)


@pytest.mark.parametrize("make", [lambda hb: hb.Graph.weblike(1 << 16, cap=5000, seed=3),
                                  lambda hb: hb.Graph.rmat(15, 8, seed=2),
                                  lambda hb: hb.Graph.erdos_renyi(40000, 3, 9)])
@pytest.mark.parametrize("threads", [1, 3, 8])
def test_oracle_parallel_visit_matches_sequential(oracle, hb, make, threads):
    """The oracle's fair parallel visit (par_fair.rs:226-323 on host threads;
    levels of 4,096 nodes and more are split among the threads) gives the
    sequential visit's distances and Known count, valid predecessors, the
    shared visited set, and the distance filter."""
    g = make(hb)
    off, succ = np.asarray(g.offsets), np.asarray(g.successors)
    seq, par = oracle.OracleVisit(off, succ), oracle.OracleVisit(off, succ)
    for roots in ([0], [5, 5, 17, 900]):
        seq.reset()
        par.reset()
        on, op, od = seq.visit(roots)
        pn, pp, pd = par.par_visit(roots, threads=threads)
        assert sorted(zip(pn.tolist(), pd.tolist())) == sorted(zip(on.tolist(), od.tolist()))
        assert par.known == seq.known
        assert np.all(np.diff(pd.astype(np.int64)) >= 0)  # level by level
        check_events(off, succ, pn, pp, pd, set(roots))
    # the visited set persists: nothing new from a visited node
    assert len(par.par_visit([int(pn[-1])], threads=threads)[0]) == 0
    # the filter: nodes farther than 2 neither reported nor marked
    seq.reset()
    par.reset()
    on, _, od = seq.visit([3], max_distance=2)
    pn, pp, pd = par.par_visit([3], max_distance=2, threads=threads)
    assert sorted(zip(pn.tolist(), pd.tolist())) == sorted(zip(on.tolist(), od.tolist()))
    rest_seq, rest_par = seq.visit([0])[0], par.par_visit([0], threads=threads)[0]
    assert sorted(rest_seq.tolist()) == sorted(rest_par.tolist())
    # distance 0: the roots only, no Known events; no roots: no events
    par.reset()
    pn, pp, pd = par.par_visit([4, 2, 4], max_distance=0, threads=threads)
    assert pn.tolist() == [4, 2] and pp.tolist() == [4, 2] and pd.tolist() == [0, 0]
    assert par.known == 0
    assert len(par.par_visit([], threads=threads)[0]) == 0 and par.known == 0


def test_oracle_parallel_visit_cnr2000_every_root(oracle, hb):
    """tests/test_bfv.rs:251-283 (the cnr-2000 test of the parallel visits):
    every root in order from 10,000; the oracle's parallel visit gives the
    sequential visit's distances."""
    base = cnr_basename()
    if base is None:
        pytest.skip("cnr-2000 not available (run tests/golden/make_fixtures.py)")
    g = hb.Graph.load_bvgraph(base)
    roots = (np.arange(g.num_nodes, dtype=np.uint64) + 10000) % g.num_nodes
    want = oracle.OracleVisit(g.offsets, g.successors).visit_each(roots)
    got = oracle.OracleVisit(g.offsets, g.successors).par_visit_each(roots, threads=4)
    np.testing.assert_array_equal(got, want)


def check_events(off, succ, nodes, preds, dists, roots_set):
    """Every predecessor is one level closer with an arc to the node; roots
    are their own predecessors at distance 0."""
    d = {int(a): int(b) for a, b in zip(nodes, dists)}
    assert len(d) == len(nodes), "a node was reported twice"
    for x, p, k in zip(nodes, preds, dists):
        x, p, k = int(x), int(p), int(k)
        if k == 0:
            assert p == x and x in roots_set
        else:
            assert d[p] == k - 1, (x, p, k)
            assert x in set(int(s) for s in succ[off[p]:off[p + 1]]), (x, p)


@pytest.mark.gpu
def test_simple_graph_and_seed(hb, oracle):
    off, succ = csr_from_arcs(SIMPLE_ARCS, 9)
    g = hb.Graph.from_csr(off, succ)
    v = hb.ParFair(g)
    assert list(v.visit_each(np.arange(9))) == [0, 0, 1, 2, 2, 2, 3, 3, 3]
    off2, succ2 = csr_from_arcs([(0, 1), (1, 2), (3, 2)], 4)
    v2 = hb.ParFair(hb.Graph.from_csr(off2, succ2))
    nodes, preds, dists, st = v2.par_visit([0, 3])
    d = np.zeros(4, dtype=np.int64)
    d[nodes] = dists
    assert list(d) == [0, 1, 1, 0]
    check_events(off2, succ2, nodes, preds, dists, {0, 3})
    # every node is visited now: another visit reports nothing
    assert len(v2.par_visit([1, 2])[0]) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("make", [lambda hb: hb.Graph.weblike(1 << 16, cap=5000, seed=3),
                                  lambda hb: hb.Graph.rmat(14, 8, seed=2),
                                  lambda hb: hb.Graph.erdos_renyi(20000, 3, 9)])
def test_visit_matches_oracle(hb, oracle, make):
    g = make(hb)
    off, succ = np.asarray(g.offsets), np.asarray(g.successors)
    v = hb.ParFair(g)
    o = oracle.OracleVisit(off, succ)
    for roots in ([0], [5, 5, 17, 900], [1]):
        nodes, preds, dists, st = v.par_visit(roots)
        on, op, od = o.visit(roots)
        # the same (node, distance) pairs; the reference's parallel order is free
        assert sorted(zip(nodes.tolist(), dists.tolist())) == sorted(zip(on.tolist(), od.tolist()))
        check_events(off, succ, nodes, preds, dists, set(roots))
        assert st["visited"] == len(on)
    # the distance filter: nodes farther than 2 are neither reported nor marked
    v.reset()
    o.reset()
    nodes, preds, dists, _ = v.par_visit([3], max_distance=2)
    on, op, od = o.visit([3], max_distance=2)
    assert sorted(zip(nodes.tolist(), dists.tolist())) == sorted(zip(on.tolist(), od.tolist()))
    assert dists.max(initial=0) <= 2
    nodes2, _, dists2, _ = v.par_visit([3])  # 3 is visited: nothing new from it
    assert len(nodes2) == 0
    far = v.par_visit([int(nodes[-1])] if len(nodes) else [0])
    on2 = o.visit([int(nodes[-1])] if len(nodes) else [0])[0]
    assert sorted(far[0].tolist()) == sorted(on2.tolist())


@pytest.mark.gpu
def test_known_arcs_and_heavy_nodes(hb, oracle):
    """A hub with 20,000 successors goes through the block-per-node path;
    Unknown plus Known events account for every arc of the visited nodes."""
    n = 30000
    rng = np.random.default_rng(1)
    rows = [np.unique(rng.integers(0, n, size=3)).astype(np.uint32) for _ in range(n)]
    rows[7] = np.arange(0, 20000, dtype=np.uint32)
    off = np.zeros(n + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(r) for r in rows])
    succ = np.concatenate(rows)
    v = hb.ParFair(hb.Graph.from_csr(off, succ))
    nodes, preds, dists, st = v.par_visit([7])
    on, op, od = oracle.OracleVisit(off, succ).visit([7])
    assert sorted(zip(nodes.tolist(), dists.tolist())) == sorted(zip(on.tolist(), od.tolist()))
    check_events(off, succ, nodes, preds, dists, {7})
    scanned = int(sum(off[x + 1] - off[x] for x in nodes.tolist()))
    assert st["known_arcs"] + (len(nodes) - 1) == scanned


@pytest.mark.gpu
def test_cnr2000_every_root(hb, oracle):
    """tests/test_bfv.rs:135-158: visit cnr-2000 from every root, starting at
    10000, and compare all distances."""
    base = cnr_basename()
    if base is None:
        pytest.skip("cnr-2000 not available (run tests/golden/make_fixtures.py)")
    g = hb.Graph.load_bvgraph(base)
    n = g.num_nodes
    roots = (np.arange(n, dtype=np.uint64) + 10000) % n
    d = hb.ParFair(g).visit_each(roots)
    od = oracle.OracleVisit(g.offsets, g.successors).visit_each(roots)
    np.testing.assert_array_equal(d.astype(np.uint64), od)


def test_visit_needs_a_device(product_lib, hb):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(hb.NoDeviceError):
        hb.ParFair(hb.Graph.erdos_renyi(100, 3, 1))
