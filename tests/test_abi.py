"""CPU tests of the C-ABI library and the host-side layer (no GPU needed).

* The library loads and exports every function include/hyperball_gb300.h declares.
* Without a device every entry point that needs one fails loudly (no CPU path).
* Graph generators are deterministic; the web-like law has the stated mean.
"""
import ctypes
import hashlib
import os
import re

import numpy as np
import pytest

from conftest import REPO


def _declared():
    names = set()
    for hname in os.listdir(os.path.join(REPO, "include")):
        if not hname.endswith(".h"):
            continue
        src = open(os.path.join(REPO, "include", hname)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"\b(hb_[a-z0-9_]+)\s*\(", src))
    return names


def test_exports_every_declared_symbol(product_lib):
    names = _declared()
    assert len(names) > 30
    import hyperball_gb300 as hb

    bound = {n for n, _, _ in hb.EXPORTS}
    for n in names:
        assert hasattr(product_lib, n), f"library does not export {n}"
        assert n in bound, f"python binding lacks {n}"


def test_version(product_lib):
    assert b"sm_103a" in product_lib.hb_version()


def test_no_device_fails_loudly(hb):
    import ctypes.util

    if ctypes.util.find_library("cuda") is not None and os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    g = hb.Graph.erdos_renyi(100, 3, 0)
    logic = hb.HyperLogLogBuilder(100).log_2_num_reg(6).build()
    with pytest.raises(hb.HyperBallError):
        hb.HyperBallBuilder.new(g, logic).build()


def test_missing_library_fails_loudly(hb, tmp_path):
    """Without the built library the Python mirror raises: it has no other
    implementation to fall back on."""
    with pytest.raises(ImportError, match="no CPU fallback"):
        hb.load_library(str(tmp_path / "libhyperball_gb300.so"))


def test_invalid_arguments(hb):
    g = hb.Graph.erdos_renyi(100, 3, 0)
    with pytest.raises(hb.InvalidArgumentError):
        hb.HyperLogLogBuilder(100).log_2_num_reg(3).build()
    t = hb.Graph.erdos_renyi(99, 3, 0)
    logic = hb.HyperLogLogBuilder(100).log_2_num_reg(6).build()
    with pytest.raises(hb.InvalidArgumentError):
        hb.HyperBallBuilder.with_transpose(g, t, logic)
    with pytest.raises(hb.InvalidArgumentError):
        hb.Graph.from_csr(np.array([0, 2], dtype=np.uint64), np.array([0], dtype=np.uint32))
    with pytest.raises(hb.HyperBallError):
        hb.Graph.load_bvgraph("/nonexistent/graph")


def test_er_generator_matches_spec(hb):
    g = hb.Graph.erdos_renyi(10_000, 8, 0)
    assert g.num_arcs == 80_000
    deg = np.diff(g.offsets)
    assert np.all(deg == 8)
    for v in (0, 17, 9999):
        s = g.successors_of(v)
        assert v not in s and np.all(np.diff(s.astype(np.int64)) > 0)
    h1 = hashlib.sha256(g.successors.tobytes()).hexdigest()
    h2 = hashlib.sha256(hb.Graph.erdos_renyi(10_000, 8, 0).successors.tobytes()).hexdigest()
    assert h1 == h2


def test_weblike_generator(hb):
    g = hb.Graph.weblike(1 << 18, seed=2)
    deg = np.diff(g.offsets.astype(np.int64))
    # drawn degrees have mean 12; deduplication removes a few
    assert 9.0 < deg.mean() < 12.0
    assert deg.min() >= 0 and deg.max() <= 100_000
    v = 5000
    s = g.successors_of(v).astype(np.int64)
    assert np.all(np.diff(s) > 0) and v not in s
    # 4/5 of the draws fall within +-1024 (wrapped); deduplication of hub rows
    # removes mostly local draws, so the arc fraction is a little lower
    src = np.repeat(np.arange(g.num_nodes, dtype=np.int64), deg)
    d = np.abs(g.successors.astype(np.int64) - src)
    d = np.minimum(d, g.num_nodes - d)
    near = np.mean(d <= 1024)
    assert 0.6 < near < 0.85, near
    g2 = hb.Graph.weblike(1 << 18, seed=2)
    np.testing.assert_array_equal(g.successors, g2.successors)


def test_rmat_generator(hb):
    g = hb.Graph.rmat(12, 16, seed=1)
    assert g.num_nodes == 4096
    assert 0.5 * 16 * 4096 < g.num_arcs <= 16 * 4096
    for v in range(0, 4096, 97):
        s = g.successors_of(v).astype(np.int64)
        assert np.all(np.diff(s) > 0) and v not in s
    g2 = hb.Graph.rmat(12, 16, seed=1)
    np.testing.assert_array_equal(g.successors, g2.successors)


def test_transpose(hb):
    g = hb.Graph.erdos_renyi(500, 5, 3)
    t = g.transpose()
    pairs = set()
    for v in range(g.num_nodes):
        for s in g.successors_of(v):
            pairs.add((int(v), int(s)))
    tp = set()
    for v in range(t.num_nodes):
        for s in t.successors_of(v):
            tp.add((int(s), int(v)))
    assert pairs == tp


def test_tuning_entry_points_on_the_host(hb):
    """The variant count is host-only; the bucket tuner needs a device and
    fails loudly without one; bad arguments are rejected first."""
    import ctypes.util

    assert hb.union_variant_count() == 10
    lib = hb.load_library()
    sm, mm = ctypes.c_uint32(), ctypes.c_uint32()
    assert lib.hb_tune_degree_buckets(None, None, 3, ctypes.byref(sm), ctypes.byref(mm), None) == hb.HB_ERR_INVALID
    assert lib.hb_batch_graph_replays(None, None, None) == hb.HB_ERR_INVALID
    assert lib.hb_union_variant_chosen(None, None) == hb.HB_ERR_INVALID
    if ctypes.util.find_library("cuda") is not None and os.path.exists("/dev/nvidia0"):
        return
    g = hb.Graph.erdos_renyi(100, 3, 0)
    logic = hb.HyperLogLogBuilder(100).log_2_num_reg(6).build()
    with pytest.raises(hb.HyperBallError):
        hb.tune_degree_buckets(g, logic)
