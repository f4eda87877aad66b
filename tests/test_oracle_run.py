"""CPU tests of the oracle's run control against the reference's semantics
(src/algo/hyperball/hyperball_impl.rs, "HB" below):

* run(upper_bound, threshold) caps the iterations at the number of nodes
  (HB:541), stops after the first iteration that modifies no counter
  (HB:559-570) and, with a threshold, after an iteration past the fourth whose
  relative increment is below 1 + threshold (HB:572-577);
* the neighbourhood function has one value per iteration plus the initial
  one, starts at the number of nodes and never decreases (HB:916-944);
* on a directed path every ball grows by one node per iteration, so the
  registers stop changing after the path's length.
"""
import numpy as np
import pytest


def _path(n):
    # 0 -> 1 -> ... -> n-1
    off = np.arange(n + 1, dtype=np.uint64)
    off[-1] = n - 1
    suc = np.arange(1, n, dtype=np.uint32)
    return off, suc


def test_run_stops_when_nothing_changes(oracle):
    off, suc = _path(12)
    # eight isolated nodes after the path: 20 nodes, so the cap is not what stops
    off = np.concatenate([off, np.full(8, off[-1], dtype=np.uint64)])
    o = oracle.OracleHyperBall(off, suc, 8, sod=True, harm=True, threads=1)
    o.run()
    # the farthest pair is 11 arcs apart: iterations 1..11 change counters, 12 does not
    assert o.iteration == 12
    nf = o.neighborhood_function()
    assert len(nf) == o.iteration + 1
    assert nf[0] == 20.0
    assert np.all(np.diff(nf) >= 0.0)


def test_run_caps_iterations_at_the_number_of_nodes(oracle):
    off, suc = _path(12)
    o = oracle.OracleHyperBall(off, suc, 8, threads=1)
    o.run(upper_bound=10**9)
    assert o.iteration <= 12
    o.run(upper_bound=3)
    assert o.iteration == 3
    assert len(o.neighborhood_function()) == 4


@pytest.mark.parametrize("threads", [1, 4])
def test_threshold_stops_after_the_fifth_iteration(oracle, threads):
    off, suc = _path(40)
    o = oracle.OracleHyperBall(off, suc, 6, threads=threads)
    # any relative increment is below 1 + 1e9: the check first applies after
    # the fifth iteration (0-based i > 3)
    o.run(threshold=1e9)
    assert o.iteration == 5
    o.run(threshold=0.0)
    # the neighbourhood function still grows on a 40-node path: no early stop
    assert o.iteration > 5


def test_path_counts_grow_with_the_ball(oracle):
    off, suc = _path(30)
    o = oracle.OracleHyperBall(off, suc, 10, sod=True, harm=True, threads=1)
    o.run()
    reach = o.reachable_nodes()
    # node v reaches the 30 - v nodes v..29; with 1024 registers the
    # estimate of a handful of elements is exact to well under one element
    want = 30.0 - np.arange(30)
    assert np.max(np.abs(reach - want) / want) < 0.05
    sod = o.sum_of_distances()
    # the last node reaches only itself: distance sum 0, closeness 0, lin 1
    assert sod[-1] == 0.0
    assert o.closeness_centrality()[-1] == 0.0
    assert o.lin_centrality()[-1] == 1.0
    # sum of distances from v is about sum_{d=1}^{29-v} d
    k = 29 - np.arange(30)
    exact = k * (k + 1) / 2.0
    mask = k > 0
    assert np.max(np.abs(sod[mask] - exact[mask]) / exact[mask]) < 0.15
