"""The strongly connected components inside the ExactSumSweep restatement
(oracle/sum_sweep_oracle.cpp: Tarjan's algorithm as sccs/tarjan.rs numbers
it, and symm_seq.rs for symmetric graphs) on the cases of the reference's
tests/test_sccs.rs: the bucket graphs, a cycle, a complete graph, a tree,
the lozenge (which fixes Tarjan's numbering), cnr-2000's component count,
and symmetric random graphs. The device ExactSumSweep is compared with this
restatement in tests/test_sum_sweep.py, component numbering included."""
import numpy as np
import pytest

from conftest import cnr_basename
from oracle import hbo


def csr(arcs, n=None):
    """VecGraph::from_arcs: nodes 0..max id, rows sorted, duplicates removed."""
    n = (max(max(a, b) for a, b in arcs) + 1) if n is None else n
    key = np.unique(np.array([a * n + b for a, b in arcs], dtype=np.int64))
    off = np.zeros(n + 1, dtype=np.uint64)
    off[1:] = np.cumsum(np.bincount(key // n, minlength=n))
    return off, (key % n).astype(np.uint32)


def sizes_by_size(comp, nc):
    """sort_by_size / compute_sizes of the reference: component sizes, largest first."""
    return sorted(np.bincount(comp.astype(np.int64), minlength=nc).tolist(), reverse=True)


def test_buckets():  # test_sccs.rs:90-126
    arcs = [(0, 0), (1, 0), (1, 2), (2, 1), (2, 3), (2, 4), (2, 5), (3, 4), (4, 3), (5, 5), (5, 6),
            (5, 7), (5, 8), (6, 7), (8, 7)]
    nc, comp = hbo.sccs(*csr(arcs))
    assert comp[3] == comp[4]
    assert sizes_by_size(comp, nc) == [2, 2, 1, 1, 1, 1, 1]


def test_buckets_2():  # test_sccs.rs:129-142
    nc, comp = hbo.sccs(*csr([(0, 1), (1, 2), (2, 0), (1, 3)]))
    assert sizes_by_size(comp, nc) == [3, 1]


def test_cycle():  # test_sccs.rs:145-158
    nc, comp = hbo.sccs(*csr([(0, 1), (1, 2), (2, 3), (3, 0)]))
    assert sizes_by_size(comp, nc) == [4]


def test_complete_graph():  # test_sccs.rs:161-189
    nc, comp = hbo.sccs(*csr([(i, j) for i in range(5) for j in range(5) if i != j]))
    assert comp.tolist() == [0] * 5 and nc == 1


def test_tree():  # test_sccs.rs:192-204
    nc, _ = hbo.sccs(*csr([(0, 1), (0, 2), (1, 3), (1, 4), (2, 5), (2, 6)]))
    assert nc == 7


def test_lozenge_numbering():  # test_sccs.rs:245-254
    nc, comp = hbo.sccs(*csr([(0, 1), (1, 0), (0, 2), (1, 3), (2, 3)]))
    assert comp.tolist() == [2, 2, 1, 0] and nc == 3


def test_cnr2000_component_count(hb):  # test_sccs.rs:213-226
    base = cnr_basename()
    if base is None:
        pytest.skip("cnr-2000 not available (run tests/golden/make_fixtures.py)")
    g = hb.Graph.load_bvgraph(base)
    nc, comp = hbo.sccs(g.offsets, g.successors)
    assert nc == 100977
    # Tarjan's numbering is a reverse topological order: every arc between
    # components goes from a higher number to a lower one
    off = np.asarray(g.offsets).astype(np.int64)
    src = np.repeat(np.arange(g.num_nodes), np.diff(off))
    a, b = comp[src], comp[np.asarray(g.successors).astype(np.int64)]
    assert np.all(a >= b)


@pytest.mark.parametrize("n", [10, 40, 100, 3000])
def test_symmetric_components_match_tarjan(n):  # test_sccs.rs:257-276
    rng = np.random.default_rng(n)
    for p in (0.5 / n, 1.0 / n, 2.0 / n):
        m = rng.random((n, n)) < p if n <= 100 else None
        if m is None:
            k = rng.poisson(p * n * n)
            a, b = rng.integers(0, n, k), rng.integers(0, n, k)
        else:
            a, b = np.nonzero(m)
        arcs = set(zip(a.tolist(), b.tolist())) | set(zip(b.tolist(), a.tolist()))
        off, suc = csr(sorted(arcs), n)
        nt, ct = hbo.sccs(off, suc)
        ns, cs = hbo.sccs(off, suc, symmetric=True)
        assert ns == nt
        # the same partition; symm_seq.rs numbers components by smallest node
        assert len(set(zip(ct.tolist(), cs.tolist()))) == nt
        first = [int(np.flatnonzero(cs == c)[0]) for c in range(ns)]
        assert first == sorted(first)
