"""CPU tests of the oracle against the reference's own fixtures and invariants.

* Java goldens: tests/test_hyperball.rs:221-302 (cnr-2000, log2m 8,
  Jenkins 42, five centralities within 1e-6).
* Sequential vs systolic/local engine, both arrays every iteration:
  src/algo/hyperball/hyperball_impl.rs:1263-1322.
* HyperLogLog arithmetic: merge is the register-wise max, count quirk,
  register size, SipHash round function (paper vector), statistical accuracy
  (tests/test_hyperloglog_counter.rs).
* The default node hash (Rust's DefaultHasher, SipHash-1-3 with zero keys)
  against CPython's SipHash-1-3 bytes hash under PYTHONHASHSEED=0.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, cnr_basename, cnr_result


def _java(name):
    return np.fromfile(cnr_result(name), dtype=">f4").astype(np.float64)


def _rel(exp, act):
    d = np.abs(exp - act)
    return np.where(exp != 0, d / np.where(exp != 0, exp, 1.0), d)


@pytest.fixture(scope="module")
def cnr(hb):
    if cnr_basename() is None:
        pytest.skip("cnr-2000 fixture not present")
    return hb.Graph.load_bvgraph(cnr_basename()), hb.Graph.load_bvgraph(cnr_basename(True))


def test_bvgraph_decoder(cnr):
    g, gt = cnr
    assert (g.num_nodes, g.num_arcs) == (325_557, 3_216_152)  # cnr-2000.properties
    t = g.transpose()
    np.testing.assert_array_equal(t.offsets, gt.offsets)
    np.testing.assert_array_equal(t.successors, gt.successors)
    for v in (0, 1, 1000, 325_556):
        s = g.successors_of(v)
        assert np.all(np.diff(s.astype(np.int64)) > 0)


def test_oracle_java_goldens(cnr, oracle):
    g, gt = cnr
    if cnr_result("sum_of_distances") is None:
        pytest.skip("Java results not present")
    o = oracle.OracleHyperBall(g.offsets, g.successors, 8, hash_kind=1, seed=42,
                               t_offsets=gt.offsets, t_successors=gt.successors,
                               sod=True, harm=True, threads=os.cpu_count() or 1)
    o.run_until_done()
    for name, fn in (("sum_of_distances", o.sum_of_distances),
                     ("harmonic_centrality", o.harmonic_centralities),
                     ("lin_centrality", o.lin_centrality),
                     ("closeness_centrality", o.closeness_centrality),
                     ("nieminen_centrality", o.nieminen_centrality)):
        exp = _java(name)
        assert _rel(exp, fn()).max() < 1e-6, name
    # the committed sample agrees with the files it was taken from
    doc = json.load(open(os.path.join(GOLDEN, "cnr2000_java_sample.json")))
    idx = np.array(doc["nodes"])
    for name, vals in doc["values"].items():
        raw = open(cnr_result(name), "rb").read()
        assert hashlib.sha256(raw).hexdigest() == doc["sha256"][name]
        np.testing.assert_array_equal(_java(name)[idx], np.array(vals))


def test_oracle_seq_vs_systolic_cnr(cnr, oracle):
    """HB:1263-1322 on cnr-2000, log2m 6, default hasher, 8 threads."""
    g, gt = cnr
    o = oracle.OracleHyperBall(g.offsets, g.successors, 6, t_offsets=gt.offsets,
                               t_successors=gt.successors, threads=os.cpu_count() or 1)
    s = oracle.SeqHyperBall(g.offsets, g.successors, 6)
    o.init()
    s.init()
    saw_local = False
    while True:
        st = o.iterate()
        s.iterate()
        saw_local |= bool(st["local"])
        np.testing.assert_array_equal(o.registers(1), s.registers(1))
        np.testing.assert_array_equal(o.registers(0), s.registers(0))
        if st["modified"] == 0:
            break
    assert saw_local


@pytest.mark.parametrize("log2m,threads", [(4, 1), (5, 3), (6, 4), (8, 2)])
def test_oracle_seq_vs_systolic_er(hb, oracle, log2m, threads):
    g = hb.Graph.erdos_renyi(3000, 4, log2m)
    t = g.transpose()
    o = oracle.OracleHyperBall(g.offsets, g.successors, log2m, t_offsets=t.offsets,
                               t_successors=t.successors, threads=threads, sod=True, harm=True)
    s = oracle.SeqHyperBall(g.offsets, g.successors, log2m)
    o.init()
    s.init()
    for _ in range(200):
        st = o.iterate()
        s.iterate()
        np.testing.assert_array_equal(o.registers(0), s.registers(0))
        np.testing.assert_array_equal(o.registers(1), s.registers(1))
        if st["modified"] == 0:
            break
    assert st["modified"] == 0


def test_oracle_digests(hb, oracle):
    """The oracle reproduces the committed per-iteration digests."""
    doc = json.load(open(os.path.join(GOLDEN, "oracle_digests.json")))
    import re

    for case in doc["cases"]:
        n, d, seed = map(int, re.findall(r"=(\d+)", case["graph"]))
        g = hb.Graph.erdos_renyi(n, d, seed)
        assert hashlib.sha256(g.successors.tobytes()).hexdigest() == case["graph_sha256"]
        t = g.transpose()
        o = oracle.OracleHyperBall(g.offsets, g.successors, case["log2m"],
                                   hash_kind=case["hash_kind"], seed=case["hash_seed"],
                                   t_offsets=t.offsets, t_successors=t.successors,
                                   sod=True, harm=True)
        o.init()
        for exp in case["iterations"]:
            st = o.iterate()
            assert st["modified"] == exp["modified"]
            assert st["visited_arcs"] == exp["visited_arcs"]
            assert abs(st["nf"] - exp["nf"]) <= 1e-12 * abs(exp["nf"])
            assert hashlib.sha256(o.registers(0).tobytes()).hexdigest() == exp["registers_sha256"]


# ---------------------------------------------------------------------------
# HyperLogLog arithmetic
# ---------------------------------------------------------------------------
def _regs_to_bytes(regs):
    """Packs 5-bit registers LSB-first into bytes (the reference layout)."""
    bits = 0
    for i, r in enumerate(regs):
        bits |= int(r) << (5 * i)
    nbytes = len(regs) * 5 // 8
    return np.frombuffer(bits.to_bytes(nbytes, "little"), dtype=np.uint8).copy()


def _bytes_to_regs(b, m):
    bits = int.from_bytes(bytes(b), "little")
    return [(bits >> (5 * i)) & 31 for i in range(m)]


@pytest.mark.parametrize("log2m", [4, 5, 6, 7, 8])
def test_broadword_merge_is_registerwise_max(oracle, log2m):
    """HLL:469-576 equals max() for every pair of values at every position."""
    L = oracle.lib()
    m = 1 << log2m
    rng = np.random.default_rng(log2m)
    wb = oracle.word_bits_for(log2m)
    pairs = [(a, b) for a in range(32) for b in range(32)]
    for start in range(0, len(pairs), m):
        chunk = pairs[start:start + m]
        x = rng.integers(0, 32, size=m)
        y = rng.integers(0, 32, size=m)
        for k, (a, b) in enumerate(chunk):
            x[k], y[k] = a, b
        xb, yb = _regs_to_bytes(x), _regs_to_bytes(y)
        assert L.hbo_hll_merge(log2m, 1000, wb, xb.ctypes.data, yb.ctypes.data) == 0
        assert _bytes_to_regs(xb, m) == [max(p, q) for p, q in zip(x, y)]


def test_merge_word_type_invariance(oracle):
    """u16, u32 and u64 words give the same bytes (little-endian layout)."""
    L = oracle.lib()
    rng = np.random.default_rng(1)
    for _ in range(50):
        x = rng.integers(0, 32, size=64)
        y = rng.integers(0, 32, size=64)
        outs = []
        for wb in (16, 32, 64):
            xb, yb = _regs_to_bytes(x), _regs_to_bytes(y)
            L.hbo_hll_merge(6, 1000, wb, xb.ctypes.data, yb.ctypes.data)
            outs.append(xb.tobytes())
        assert outs[0] == outs[1] == outs[2]


def test_count_i32_quirk(oracle):
    """HLL:178: a register holding 31 adds -2^-31 (Rust i32 shift) instead of +2^-31."""
    L = oracle.lib()
    m = 64
    regs = [31] * m
    b = _regs_to_bytes(regs)
    c_quirk = L.hbo_hll_count(6, 1000, 64, b.ctypes.data, 1)
    c_plain = L.hbo_hll_count(6, 1000, 64, b.ctypes.data, 0)
    alpha_m_m = 0.709 * m * m
    assert c_quirk == alpha_m_m / (-m * 2.0 ** -31)
    assert c_plain == alpha_m_m / (m * 2.0 ** -31)
    # all-zero counter: small-range correction m*ln(m/m) = 0
    z = _regs_to_bytes([0] * m)
    assert L.hbo_hll_count(6, 1000, 64, z.ctypes.data, 1) == 0.0


def test_register_size(oracle):
    L = oracle.lib()
    for n in (0, 1, 2, 10, 10_000, 1 << 26, 1 << 40, 2**64 - 1):
        assert L.hbo_register_size(n) == 5


def test_siphash_paper_vector(oracle):
    """SipHash-2-4, key 00..0f, message 00..0e -> a129ca6149be45e5 (Aumasson &
    Bernstein 2012, Appendix A); pins the round function used by SipHash-1-3."""
    L = oracle.lib()
    k0 = int.from_bytes(bytes(range(8)), "little")
    k1 = int.from_bytes(bytes(range(8, 16)), "little")
    msg = bytes(range(15))
    assert L.hbo_siphash(2, 4, k0, k1, msg, 15) == 0xa129ca6149be45e5


def test_division_by_iteration_number_is_correctly_rounded(oracle):
    """The device computes delta / (t+1) as Markstein's corrected product
    q0 = RN(a*rd), q1 = RN(q0 + fma(-q0, d, a)*rd); it must equal IEEE a/d
    for every divisor up to 4096 (far above any iteration count reached)."""
    assert oracle.lib().hbo_check_div_small_int(4096, 20000, 7) == 0


def test_sip13_is_siphash13_of_le_bytes(oracle):
    L = oracle.lib()
    for x in (0, 1, 12345, 2**63 + 7):
        assert L.hbo_hash(0, 0, x) == L.hbo_siphash(1, 3, 0, 0, x.to_bytes(8, "little"), 8)


def test_sip13_matches_cpython_siphash13(oracle):
    """The node hash against an independent SipHash-1-3. CPython hashes bytes
    with SipHash-1-3 (sys.hash_info.algorithm 'siphash13', no small-input
    cutoff), and with PYTHONHASHSEED=0 its 128-bit key is all zero bits: the
    key of Rust's DefaultHasher::new(), which the reference's HyperBall uses
    (hyperball_impl.rs:69, hyper_log_log_logic.rs:241-246). So in such an
    interpreter hash(x.to_bytes(8, 'little')) is the node hash of x, as a
    signed 64-bit value (CPython maps -1 to -2)."""
    import subprocess
    import sys
    rng = np.random.default_rng(11)
    xs = [0, 1, 2, 3, 255, 256, 65535, 1 << 20, (1 << 26) - 1, (1 << 32) + 1, 2**63, 2**64 - 1]
    xs += [int(v) for v in rng.integers(0, 1 << 26, size=500, dtype=np.uint64)]
    xs += [int(v) for v in rng.integers(0, 2**63, size=500, dtype=np.uint64) * 2 + 1]
    code = ("import sys; h = sys.hash_info; print(h.algorithm, h.cutoff); "
            "[print(hash(int(t).to_bytes(8, 'little'))) for t in sys.stdin.read().split()]")
    env = dict(os.environ, PYTHONHASHSEED="0")
    out = subprocess.run([sys.executable, "-c", code], input=" ".join(map(str, xs)), env=env,
                         capture_output=True, text=True, check=True).stdout.split("\n")
    algorithm, cutoff = out[0].split()
    if algorithm != "siphash13" or cutoff != "0":
        pytest.skip(f"this interpreter hashes bytes with {algorithm} (cutoff {cutoff})")
    L = oracle.lib()
    checked = 0
    for x, line in zip(xs, out[1:]):
        py = int(line)
        if py == -2:
            continue  # SipHash output -1 or -2: CPython returns -2 for both
        assert L.hbo_hash(0, 0, x) == py & (2**64 - 1), x
        checked += 1
    assert checked == len(xs)


def _splitmix(seed, xs):
    """Stand-in element hasher for the statistical tests (xxh3 with a seed in
    the reference; any well-mixed 64-bit hash serves the accuracy bound)."""
    z = (np.asarray(xs, dtype=np.uint64) + np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15))
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


@pytest.mark.parametrize("log2m", [4, 6, 8, 12])
def test_hll_accuracy(oracle, log2m):
    """tests/test_hyperloglog_counter.rs:21-64 and :126-185: >= 90 of 100 trials
    within 2 * rel_std, for single counters and for merged halves."""
    import ctypes

    L = oracle.lib()
    rsd = {4: 1.106, 5: 1.070, 6: 1.054, 7: 1.046}.get(log2m, 1.04) / np.sqrt(1 << log2m)
    P = ctypes.POINTER(ctypes.c_uint64)
    with np.errstate(over="ignore"):
        for size in (1, 10, 100, 1000, 100_000):
            ok_single = ok_merge = 0
            incr = (1 << 32) // size
            xs = (np.arange(size, dtype=np.int64) * incr + np.iinfo(np.int64).min).view(np.uint64)
            for trial in range(100):
                h = np.ascontiguousarray(_splitmix(trial, xs))
                c = L.hbo_hll_count_hashes(log2m, size, h.ctypes.data_as(P), size, None, 0)
                ok_single += abs(size - c) / size < 2 * rsd
                a, b = h[: size // 2].copy(), h[size // 2:].copy()
                c2 = L.hbo_hll_count_hashes(log2m, size, a.ctypes.data_as(P), len(a),
                                            b.ctypes.data_as(P), len(b))
                ok_merge += abs(size - c2) / size < 2 * rsd
            assert ok_single >= 90, (size, ok_single)
            assert ok_merge >= 90, (size, ok_merge)
