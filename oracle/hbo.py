"""ctypes wrapper of the CPU oracle library — test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
the checker; the product never imports it.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_P = ctypes.POINTER
_lib = None


class Stats(ctypes.Structure):
    _fields_ = [
        ("iteration", ctypes.c_uint64),
        ("modified", ctypes.c_uint64),
        ("visited_arcs", ctypes.c_uint64),
        ("nf", ctypes.c_double),
        ("relative_increment", ctypes.c_double),
        ("systolic", ctypes.c_int32),
        ("local", ctypes.c_int32),
        ("pre_local", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


DISCOUNT_FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_uint64, ctypes.c_void_p)


def lib():
    global _lib
    if _lib is None:
        build_oracle.build()
        L = ctypes.CDLL(build_oracle.LIB)
        V = ctypes.c_void_p
        sig = {
            "hbo_create": (V, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint32),
                               _P(ctypes.c_uint64), _P(ctypes.c_uint32), ctypes.c_int,
                               ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                               ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                               _P(ctypes.c_uint64), ctypes.c_uint64]),
            "hbo_add_discount": (ctypes.c_int, [V, DISCOUNT_FN, V]),
            "hbo_destroy": (None, [V]),
            "hbo_init": (ctypes.c_int, [V]),
            "hbo_iterate": (ctypes.c_int, [V, _P(Stats)]),
            "hbo_run": (ctypes.c_int, [V, ctypes.c_uint64, ctypes.c_double, ctypes.c_int]),
            "hbo_iteration": (ctypes.c_uint64, [V]),
            "hbo_words_per_counter": (ctypes.c_uint64, [V]),
            "hbo_word_bytes": (ctypes.c_int, [V]),
            "hbo_last_stats": (None, [V, _P(Stats)]),
            "hbo_get_array": (None, [V, ctypes.c_int, V]),
            "hbo_nf_len": (ctypes.c_uint64, [V]),
            "hbo_get_nf": (None, [V, _P(ctypes.c_double)]),
            "hbo_get_sod": (ctypes.c_int, [V, _P(ctypes.c_double)]),
            "hbo_get_harm": (ctypes.c_int, [V, _P(ctypes.c_double)]),
            "hbo_get_discounted": (ctypes.c_int, [V, ctypes.c_uint64, _P(ctypes.c_double)]),
            "hbo_get_reachable": (None, [V, ctypes.c_uint64, _P(ctypes.c_double)]),
            "hbo_seq_create": (V, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint32),
                                   ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_int]),
            "hbo_seq_init": (None, [V]),
            "hbo_seq_iterate": (None, [V]),
            "hbo_seq_get_array": (None, [V, ctypes.c_int, V]),
            "hbo_seq_destroy": (None, [V]),
            "hbo_hash": (ctypes.c_uint64, [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]),
            "hbo_siphash": (ctypes.c_uint64, [ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                              ctypes.c_uint64, ctypes.c_char_p, ctypes.c_uint64]),
            "hbo_register_size": (ctypes.c_int, [ctypes.c_uint64]),
            "hbo_hll_merge": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint64, ctypes.c_int, V, V]),
            "hbo_hll_count": (ctypes.c_double, [ctypes.c_int, ctypes.c_uint64, ctypes.c_int, V,
                                                ctypes.c_int]),
            "hbo_hll_add": (None, [ctypes.c_int, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_uint64, V, ctypes.c_uint64]),
            "hbo_hll_add_hash": (None, [ctypes.c_int, ctypes.c_uint64, V, ctypes.c_uint64]),
            "hbo_hll_params": (None, [ctypes.c_int, ctypes.c_uint64, _P(ctypes.c_double),
                                      _P(ctypes.c_uint64)]),
            "hbo_last_error": (ctypes.c_char_p, []),
            "hbo_check_div_small_int": (ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_uint64,
                                                          ctypes.c_uint64]),
            "hbo_hll_count_hashes": (ctypes.c_double, [ctypes.c_int, ctypes.c_uint64,
                                                       _P(ctypes.c_uint64), ctypes.c_uint64,
                                                       _P(ctypes.c_uint64), ctypes.c_uint64]),
            "hbo_gen_er": (V, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64]),
            "hbo_gen_rmat": (V, [ctypes.c_int, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_uint64]),
            "hbo_gen_weblike": (V, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double,
                                    ctypes.c_uint64, ctypes.c_uint64]),
            "hbo_graph_transpose": (V, [V]),
            "hbo_transpose_csr": (V, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint32)]),
            "hbo_graph_nodes": (ctypes.c_uint64, [V]),
            "hbo_graph_arcs": (ctypes.c_uint64, [V]),
            "hbo_graph_offsets": (V, [V]),
            "hbo_graph_successors": (V, [V]),
            "hbo_graph_free": (None, [V]),
            "hbo_visit_create": (V, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint32)]),
            "hbo_visit_destroy": (None, [V]),
            "hbo_visit_reset": (None, [V]),
            "hbo_sum_sweep": (ctypes.c_int, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint32),
                                             _P(ctypes.c_uint64), _P(ctypes.c_uint32), ctypes.c_int,
                                             V, _P(ctypes.c_uint64), _P(ctypes.c_uint64),
                                             _P(ctypes.c_uint64)]),
            "hbo_eccentricities": (None, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint32),
                                          _P(ctypes.c_uint64)]),
            "hbo_sccs_tarjan": (ctypes.c_uint64, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint32),
                                                  _P(ctypes.c_uint64)]),
            "hbo_sccs_symm": (ctypes.c_uint64, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint32),
                                                _P(ctypes.c_uint64)]),
            "hbo_arg_select": (ctypes.c_uint64, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint64),
                                                 _P(ctypes.c_uint8), ctypes.c_int]),
            "hbo_visit_each": (None, [V, _P(ctypes.c_uint64), ctypes.c_uint64, _P(ctypes.c_uint64)]),
            "hbo_par_visit_each": (None, [V, _P(ctypes.c_uint64), ctypes.c_uint64, ctypes.c_uint32,
                                          _P(ctypes.c_uint64)]),
            "hbo_visit_run": (ctypes.c_uint64, [V, _P(ctypes.c_uint64), ctypes.c_uint64,
                                                ctypes.c_uint64, _P(ctypes.c_uint64),
                                                _P(ctypes.c_uint64), _P(ctypes.c_uint64),
                                                ctypes.c_uint64, _P(ctypes.c_uint64)]),
            "hbo_par_visit_run": (ctypes.c_uint64, [V, _P(ctypes.c_uint64), ctypes.c_uint64,
                                                    ctypes.c_uint64, ctypes.c_uint32,
                                                    _P(ctypes.c_uint64), _P(ctypes.c_uint64),
                                                    _P(ctypes.c_uint64), ctypes.c_uint64,
                                                    _P(ctypes.c_uint64)]),
            "hbo_sum_sweep_par": (ctypes.c_int, [ctypes.c_uint64, _P(ctypes.c_uint64), _P(ctypes.c_uint32),
                                                 _P(ctypes.c_uint64), _P(ctypes.c_uint32), ctypes.c_int,
                                                 V, _P(ctypes.c_uint64), _P(ctypes.c_uint64),
                                                 _P(ctypes.c_uint64), ctypes.c_uint32]),
        }
        for k, (r, a) in sig.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


class OracleGraph:
    """A CSR graph made by the seeded generators compiled into the oracle's
    library (the same source as the product's): `offsets` (u64, n+1) and
    `successors` (u32, m) are views of memory this object owns."""

    def __init__(self, handle):
        if not handle:
            raise MemoryError("graph generation failed")
        self._h = ctypes.c_void_p(handle)
        L = lib()
        self.num_nodes = int(L.hbo_graph_nodes(self._h))
        self.num_arcs = int(L.hbo_graph_arcs(self._h))
        self.offsets = self._view(L.hbo_graph_offsets(self._h), self.num_nodes + 1, ctypes.c_uint64)
        self.successors = self._view(L.hbo_graph_successors(self._h), self.num_arcs, ctypes.c_uint32)

    @staticmethod
    def _view(ptr, count, ctype):
        if count == 0 or not ptr:
            return np.zeros(count, dtype=np.dtype(ctype))
        return np.ctypeslib.as_array(ctypes.cast(ptr, _P(ctype)), shape=(count,))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().hbo_graph_free(self._h)
            self._h = None

    @staticmethod
    def erdos_renyi(n, d, seed):
        return OracleGraph(lib().hbo_gen_er(n, d, seed))

    @staticmethod
    def rmat(scale, edges_per_node, a=0.57, b=0.19, c=0.19, seed=1):
        return OracleGraph(lib().hbo_gen_rmat(scale, edges_per_node, a, b, c, seed))

    @staticmethod
    def weblike(n, cap=100_000, shift=1.266, window=1024, seed=2):
        return OracleGraph(lib().hbo_gen_weblike(n, cap, shift, window, seed))

    def transpose(self):
        return OracleGraph(lib().hbo_graph_transpose(self._h))

    @staticmethod
    def transpose_of(offsets, successors):
        """The transpose of a CSR held in numpy arrays (rows sorted)."""
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        suc = np.ascontiguousarray(successors, dtype=np.uint32)
        return OracleGraph(lib().hbo_transpose_csr(len(off) - 1, off.ctypes.data_as(_P(ctypes.c_uint64)),
                                                   suc.ctypes.data_as(_P(ctypes.c_uint32))))


def word_bits_for(log2m):
    """Widest word the reference's `ensure!` (HLL:399-403) accepts."""
    bits = (1 << log2m) * 5
    for w in (64, 32, 16):
        if bits % w == 0:
            return w
    return 16


SOD, HARM, NO_QUIRK = 1, 2, 4


class OracleHyperBall:
    """The reference HyperBall restated on the CPU (oracle/hyperball_oracle.cpp)."""

    def __init__(self, offsets, successors, log2m, hash_kind=0, seed=0, t_offsets=None,
                 t_successors=None, sod=False, harm=False, threads=1, granularity=0,
                 num_elements=0, word_bits=None, quirk=True, weights=None, weight_seed=0,
                 discounts=()):
        L = lib()
        self._off = np.ascontiguousarray(offsets, dtype=np.uint64)
        self._suc = np.ascontiguousarray(successors, dtype=np.uint32)
        self.n = len(self._off) - 1
        self._toff = None if t_offsets is None else np.ascontiguousarray(t_offsets, dtype=np.uint64)
        self._tsuc = None if t_successors is None else np.ascontiguousarray(t_successors, dtype=np.uint32)
        self._w = None if weights is None else np.ascontiguousarray(weights, dtype=np.uint64)
        wb = word_bits or word_bits_for(log2m)
        flags = (SOD if sod else 0) | (HARM if harm else 0) | (0 if quirk else NO_QUIRK)
        p = lambda a, t: a.ctypes.data_as(_P(t)) if a is not None else None
        self._h = L.hbo_create(self.n, p(self._off, ctypes.c_uint64), p(self._suc, ctypes.c_uint32),
                               p(self._toff, ctypes.c_uint64), p(self._tsuc, ctypes.c_uint32),
                               log2m, hash_kind, seed, num_elements, wb, flags, threads,
                               granularity, p(self._w, ctypes.c_uint64), weight_seed)
        if not self._h:
            raise ValueError(L.hbo_last_error().decode())
        self._cbs = []
        for fn in discounts:
            cb = DISCOUNT_FN(lambda d, _c, f=fn: float(f(int(d))))
            self._cbs.append(cb)
            L.hbo_add_discount(self._h, cb, None)
        self.counter_bytes = (1 << log2m) * 5 // 8

    def __del__(self):
        if getattr(self, "_h", None):
            lib().hbo_destroy(self._h)
            self._h = None

    def init(self):
        lib().hbo_init(self._h)

    def iterate(self):
        s = Stats()
        lib().hbo_iterate(self._h, ctypes.byref(s))
        return s.as_dict()

    def run(self, upper_bound=2**64 - 1, threshold=None):
        lib().hbo_run(self._h, upper_bound, 0.0 if threshold is None else threshold,
                      0 if threshold is None else 1)

    def run_until_done(self):
        self.run()

    @property
    def iteration(self):
        return int(lib().hbo_iteration(self._h))

    def registers(self, which=0):
        out = np.zeros((self.n, self.counter_bytes), dtype=np.uint8)
        lib().hbo_get_array(self._h, which, out.ctypes.data)
        return out

    def neighborhood_function(self):
        k = lib().hbo_nf_len(self._h)
        out = np.zeros(k, dtype=np.float64)
        lib().hbo_get_nf(self._h, out.ctypes.data_as(_P(ctypes.c_double)))
        return out

    def sum_of_distances(self):
        out = np.zeros(self.n, dtype=np.float64)
        if lib().hbo_get_sod(self._h, out.ctypes.data_as(_P(ctypes.c_double))) != 0:
            raise ValueError("sum of distances not requested")
        return out

    def harmonic_centralities(self):
        out = np.zeros(self.n, dtype=np.float64)
        if lib().hbo_get_harm(self._h, out.ctypes.data_as(_P(ctypes.c_double))) != 0:
            raise ValueError("harmonic centralities not requested")
        return out

    def discounted_centrality(self, i):
        out = np.zeros(self.n, dtype=np.float64)
        if lib().hbo_get_discounted(self._h, i, out.ctypes.data_as(_P(ctypes.c_double))) != 0:
            raise ValueError("no such discount function")
        return out

    def reachable_nodes(self):
        out = np.zeros(self.n, dtype=np.float64)
        lib().hbo_get_reachable(self._h, self.n, out.ctypes.data_as(_P(ctypes.c_double)))
        return out

    # derived accessors, HB:674-732
    def closeness_centrality(self):
        d = self.sum_of_distances()
        with np.errstate(divide="ignore"):
            return np.where(d == 0.0, 0.0, 1.0 / np.where(d == 0.0, 1.0, d))

    def lin_centrality(self):
        d = self.sum_of_distances()
        c = self.reachable_nodes()
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(d == 0.0, 1.0, c * c / np.where(d == 0.0, 1.0, d))

    def nieminen_centrality(self):
        d = self.sum_of_distances()
        c = self.reachable_nodes()
        return (c * c) - d


class SeqHyperBall:
    """SeqHyperBall of HB:1230-1261 (merges every successor, no modes)."""

    def __init__(self, offsets, successors, log2m, hash_kind=0, seed=0):
        L = lib()
        self._off = np.ascontiguousarray(offsets, dtype=np.uint64)
        self._suc = np.ascontiguousarray(successors, dtype=np.uint32)
        self.n = len(self._off) - 1
        self.counter_bytes = (1 << log2m) * 5 // 8
        self._h = L.hbo_seq_create(self.n, self._off.ctypes.data_as(_P(ctypes.c_uint64)),
                                   self._suc.ctypes.data_as(_P(ctypes.c_uint32)), log2m, hash_kind,
                                   seed, word_bits_for(log2m))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().hbo_seq_destroy(self._h)
            self._h = None

    def init(self):
        lib().hbo_seq_init(self._h)

    def iterate(self):
        lib().hbo_seq_iterate(self._h)

    def registers(self, which=0):
        out = np.zeros((self.n, self.counter_bytes), dtype=np.uint8)
        lib().hbo_seq_get_array(self._h, which, out.ctypes.data)
        return out


class OracleVisit:
    """The reference's sequential breadth-first visit (seq.rs:113-224)
    restated: visit(roots) returns the Unknown events (node, pred, distance)
    in event order; the visited set persists until reset(). par_visit is the
    fair parallel visit with predecessors (par_fair.rs:226-323) on host
    threads, on the same visited set. Both leave the number of Known events
    in `known`."""

    def __init__(self, offsets, successors):
        self._off = np.ascontiguousarray(offsets, dtype=np.uint64)
        self._suc = np.ascontiguousarray(successors, dtype=np.uint32)
        self.n = len(self._off) - 1
        self._h = lib().hbo_visit_create(self.n, self._off.ctypes.data_as(_P(ctypes.c_uint64)),
                                         self._suc.ctypes.data_as(_P(ctypes.c_uint32)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().hbo_visit_destroy(self._h)
            self._h = None

    def reset(self):
        lib().hbo_visit_reset(self._h)

    def visit(self, roots, max_distance=None):
        r = np.ascontiguousarray(roots, dtype=np.uint64)
        cap = self.n
        nodes = np.zeros(cap, dtype=np.uint64)
        preds = np.zeros(cap, dtype=np.uint64)
        dists = np.zeros(cap, dtype=np.uint64)
        known = ctypes.c_uint64()
        md = 2**64 - 1 if max_distance is None else int(max_distance)
        P = lambda a: a.ctypes.data_as(_P(ctypes.c_uint64))
        k = lib().hbo_visit_run(self._h, P(r), len(r), md, P(nodes), P(preds), P(dists), cap,
                                ctypes.byref(known))
        self.known = known.value
        return nodes[:k], preds[:k], dists[:k]

    def par_visit(self, roots, max_distance=None, threads=None):
        r = np.ascontiguousarray(roots, dtype=np.uint64)
        cap = self.n
        nodes = np.zeros(cap, dtype=np.uint64)
        preds = np.zeros(cap, dtype=np.uint64)
        dists = np.zeros(cap, dtype=np.uint64)
        known = ctypes.c_uint64()
        md = 2**64 - 1 if max_distance is None else int(max_distance)
        th = (os.cpu_count() or 1) if threads is None else max(1, int(threads))
        P = lambda a: a.ctypes.data_as(_P(ctypes.c_uint64))
        k = lib().hbo_par_visit_run(self._h, P(r), len(r), md, th, P(nodes), P(preds), P(dists), cap,
                                    ctypes.byref(known))
        self.known = known.value
        return nodes[:k], preds[:k], dists[:k]

    def visit_each(self, roots):
        r = np.ascontiguousarray(roots, dtype=np.uint64)
        d = np.zeros(self.n, dtype=np.uint64)
        lib().hbo_visit_each(self._h, r.ctypes.data_as(_P(ctypes.c_uint64)), len(r),
                             d.ctypes.data_as(_P(ctypes.c_uint64)))
        return d

    def par_visit_each(self, roots, threads=None):
        r = np.ascontiguousarray(roots, dtype=np.uint64)
        d = np.zeros(self.n, dtype=np.uint64)
        th = (os.cpu_count() or 1) if threads is None else max(1, int(threads))
        lib().hbo_par_visit_each(self._h, r.ctypes.data_as(_P(ctypes.c_uint64)), len(r), th,
                                 d.ctypes.data_as(_P(ctypes.c_uint64)))
        return d



SWEEP_LEVELS = {"all": 0, "all_forward": 1, "radius_diameter": 2, "diameter": 3, "radius": 4}
NOT_COMPUTED = 2**64 - 1


def sum_sweep(offsets, successors, t_offsets=None, t_successors=None, level="all", radial=None,
              threads=1):
    """ExactSumSweep restated (src/algo/exact_sum_sweep/computer.rs): a
    directed graph with its transpose, or a symmetric graph without one.
    threads > 1 runs its visits as fair parallel visits on that many host
    threads (the results are the same).
    Returns the output level's fields (eccentricities as uint64 arrays;
    iterations and the radius of a graph without radial vertices as
    NOT_COMPUTED = 2^64 - 1), or None when the level's outputs were not all
    computed (an empty graph: the reference's output builders panic)."""
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    suc = np.ascontiguousarray(successors, dtype=np.uint32)
    n = len(off) - 1
    P64 = lambda a: a.ctypes.data_as(_P(ctypes.c_uint64))
    P32 = lambda a: a.ctypes.data_as(_P(ctypes.c_uint32))
    undirected = t_offsets is None
    if not undirected:
        toff = np.ascontiguousarray(t_offsets, dtype=np.uint64)
        tsuc = np.ascontiguousarray(t_successors, dtype=np.uint32)
    rad = None if radial is None else np.ascontiguousarray(radial, dtype=np.uint8)
    fe = np.zeros(max(n, 1), dtype=np.uint64)
    be = np.zeros(max(n, 1), dtype=np.uint64)
    res = np.zeros(8, dtype=np.uint64)
    lv = SWEEP_LEVELS[level]
    r = lib().hbo_sum_sweep_par(n, P64(off), P32(suc), None if undirected else P64(toff),
                                None if undirected else P32(tsuc), lv,
                                None if rad is None else rad.ctypes.data, P64(fe), P64(be), P64(res),
                                max(1, int(threads)))
    if r != 0:
        return None
    out = {"diameter": int(res[0]), "radius": int(res[1]), "diametral_vertex": int(res[2]),
           "radial_vertex": int(res[3]), "radius_iterations": int(res[4]),
           "diameter_iterations": int(res[5]), "forward_iterations": int(res[6]),
           "all_iterations": int(res[7])}
    eff = 1 if undirected and lv == 0 else lv
    if eff in (0, 1):
        out["forward_eccentricities"] = fe[:n].copy()
    if eff == 0:
        out["backward_eccentricities"] = be[:n].copy()
    return out


def arg_select(values, tie=None, keep=None, maximize=True):
    """The restatement's argmax / argmin (utils/argmax.rs, argmin.rs): the
    index of the largest (maximize) or smallest (value, tie) among the kept
    indices, the first among equals; None when nothing is kept."""
    v = np.ascontiguousarray(values, dtype=np.uint64)
    n = len(v)
    t = np.zeros(max(n, 1), dtype=np.uint64) if tie is None else np.ascontiguousarray(tie, dtype=np.uint64)
    k = np.ones(max(n, 1), dtype=np.uint8) if keep is None else np.ascontiguousarray(keep, dtype=np.uint8)
    if n == 0:
        v = np.zeros(1, dtype=np.uint64)
    r = lib().hbo_arg_select(n, v.ctypes.data_as(_P(ctypes.c_uint64)), t.ctypes.data_as(_P(ctypes.c_uint64)),
                             k.ctypes.data_as(_P(ctypes.c_uint8)), 1 if maximize else 0)
    return None if r == 2**64 - 1 else int(r)


def sccs(offsets, successors, symmetric=False):
    """The components ExactSumSweep's restatement uses: Tarjan's numbering
    (sccs/tarjan.rs) or, for a symmetric graph, symm_seq.rs's. Returns
    (number of components, component of every node as uint64)."""
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    suc = np.ascontiguousarray(successors, dtype=np.uint32)
    n = len(off) - 1
    comp = np.zeros(max(n, 1), dtype=np.uint64)
    f = lib().hbo_sccs_symm if symmetric else lib().hbo_sccs_tarjan
    nc = f(n, off.ctypes.data_as(_P(ctypes.c_uint64)), suc.ctypes.data_as(_P(ctypes.c_uint32)),
           comp.ctypes.data_as(_P(ctypes.c_uint64)))
    return int(nc), comp[:n].copy()


def eccentricities(offsets, successors):
    """Forward eccentricity of every node, one breadth-first visit each."""
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    suc = np.ascontiguousarray(successors, dtype=np.uint32)
    n = len(off) - 1
    e = np.zeros(max(n, 1), dtype=np.uint64)
    lib().hbo_eccentricities(n, off.ctypes.data_as(_P(ctypes.c_uint64)),
                             suc.ctypes.data_as(_P(ctypes.c_uint32)),
                             e.ctypes.data_as(_P(ctypes.c_uint64)))
    return e[:n]
