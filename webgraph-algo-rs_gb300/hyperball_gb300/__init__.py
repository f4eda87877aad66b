"""Python mirror of the reference HyperBall API over the GB300 C ABI.

The reference (Rust crate webgraph-algo 0.1.0) drives HyperBall as

    let logic = HyperLogLogBuilder::new(n).log_2_num_reg(8)
        .build_hasher(JenkinsHasherBuilder::new(42)).build()?;     // HLL:234-428
    let mut hb = HyperBallBuilder::with_transpose(&g, &gt, &dcf, a0, a1)
        .sum_of_distances(true).sum_of_inverse_distances(true)
        .build(pl);                                                 // HB:204-403
    hb.run_until_done(&threads, pl)?;                               // HB:614-621
    let sod = hb.sum_of_distances()?;                               // HB:639-647

and this module keeps that shape, names and error behaviour:

    logic = HyperLogLogBuilder(n).log_2_num_reg(8).build_hasher(JenkinsHasher(42)).build()
    hb = (HyperBallBuilder.with_transpose(g, gt, logic)
          .sum_of_distances(True).sum_of_inverse_distances(True).build())
    hb.run_until_done()
    sod = hb.sum_of_distances()

Counters live on the GPU; there is no CPU path. Loading the library never
needs a GPU, but building a HyperBall without one raises NoDeviceError.
"""
import ctypes
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(_HERE)
LIB_PATH = os.path.join(_PKG, "lib", "libhyperball_gb300.so")

HB_OK = 0
HB_ERR_INVALID = 1
HB_ERR_NOT_RUN = 2
HB_ERR_NOT_REQUESTED = 3
HB_ERR_OOM = 4
HB_ERR_CUDA = 5
HB_ERR_TIMEOUT = 6
HB_ERR_IO = 7
HB_ERR_NO_DEVICE = 8

HB_HASH_SIP13 = 0
HB_HASH_JENKINS = 1

HB_SUM_OF_DISTANCES = 1 << 0
HB_SUM_OF_INVERSE_DISTANCES = 1 << 1
HB_TRANSPOSE_ON_DEVICE = 1 << 2
HB_NO_I32_SHIFT_QUIRK = 1 << 3
HB_TMA_GATHER = 1 << 4
HB_NO_GRAPHS = 1 << 5

HB_CURRENT_STATE = 0
HB_NEXT_STATE = 1

HB_JOB_QUEUED = 0
HB_JOB_RUNNING = 1
HB_JOB_DONE = 2
HB_JOB_FAILED = 3


class HyperBallError(RuntimeError):
    """Base error; `code` is the C status."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class InvalidArgumentError(HyperBallError, ValueError):
    pass


class NotRunError(HyperBallError):
    pass


class NotRequestedError(HyperBallError):
    pass


class NoDeviceError(HyperBallError):
    pass


_ERRORS = {
    HB_ERR_INVALID: InvalidArgumentError,
    HB_ERR_NOT_RUN: NotRunError,
    HB_ERR_NOT_REQUESTED: NotRequestedError,
    HB_ERR_NO_DEVICE: NoDeviceError,
}


class GraphView(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_uint64),
        ("num_arcs", ctypes.c_uint64),
        ("offsets", ctypes.POINTER(ctypes.c_uint64)),
        ("successors", ctypes.POINTER(ctypes.c_uint32)),
    ]


class Options(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("log2m", ctypes.c_int32),
        ("hash_kind", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("hash_seed", ctypes.c_uint64),
        ("num_elements", ctypes.c_uint64),
        ("flags", ctypes.c_uint32),
        ("far_rows", ctypes.c_uint32),
        ("arc_granularity", ctypes.c_uint64),
        ("weights", ctypes.POINTER(ctypes.c_uint64)),
        ("weight_seed", ctypes.c_uint64),
        ("stream", ctypes.c_void_p),
        ("small_max_degree", ctypes.c_uint32),
        ("medium_max_degree", ctypes.c_uint32),
        ("union_variant", ctypes.c_uint32),
    ]


class ServerOptions(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("device", ctypes.c_int32),
        ("hbm_budget_bytes", ctypes.c_uint64),
        ("max_active", ctypes.c_uint32),
        ("keep_registers", ctypes.c_uint32),
        ("setup_threads", ctypes.c_uint32),
        ("union_sm_reserve", ctypes.c_uint32),
    ]


class JobInfo(ctypes.Structure):
    _fields_ = [
        ("state", ctypes.c_int32),
        ("error", ctypes.c_int32),
        ("iterations", ctypes.c_uint64),
        ("visited_arcs", ctypes.c_uint64),
        ("register_updates", ctypes.c_uint64),
        ("footprint_bytes", ctypes.c_uint64),
        ("queue_ms", ctypes.c_double),
        ("run_ms", ctypes.c_double),
        ("latency_ms", ctypes.c_double),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class VisitStats(ctypes.Structure):
    _fields_ = [("visited", ctypes.c_uint64), ("levels", ctypes.c_uint64),
                ("known_arcs", ctypes.c_uint64), ("device_ms", ctypes.c_double)]


class SweepResult(ctypes.Structure):
    _fields_ = [("diameter", ctypes.c_uint64), ("radius", ctypes.c_uint64),
                ("diametral_vertex", ctypes.c_uint64), ("radial_vertex", ctypes.c_uint64),
                ("radius_iterations", ctypes.c_uint64), ("diameter_iterations", ctypes.c_uint64),
                ("forward_iterations", ctypes.c_uint64), ("all_iterations", ctypes.c_uint64),
                ("sweeps", ctypes.c_uint64), ("device_ms", ctypes.c_double)]


class IterStats(ctypes.Structure):
    _fields_ = [
        ("iteration", ctypes.c_uint64),
        ("modified_counters", ctypes.c_uint64),
        ("visited_arcs", ctypes.c_uint64),
        ("scanned_nodes", ctypes.c_uint64),
        ("neighborhood_function", ctypes.c_double),
        ("relative_increment", ctypes.c_double),
        ("systolic", ctypes.c_int32),
        ("local", ctypes.c_int32),
        ("pre_local", ctypes.c_int32),
        ("union_variant", ctypes.c_int32),
        ("union_ms", ctypes.c_double),
        ("iteration_ms", ctypes.c_double),
        ("scanned_arcs", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64),
        ("from_graph", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


DISCOUNT_FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_uint64, ctypes.c_void_p)

# (name, restype, argtypes) of every exported entry point of include/hyperball_gb300.h
_P = ctypes.POINTER
_H = ctypes.c_void_p
EXPORTS = [
    ("hb_options_default", None, [_P(Options)]),
    ("hb_create", ctypes.c_int, [_P(GraphView), _P(GraphView), _P(Options), _P(_H)]),
    ("hb_add_discount_function", ctypes.c_int, [_H, DISCOUNT_FN, ctypes.c_void_p]),
    ("hb_destroy", None, [_H]),
    ("hb_run", ctypes.c_int, [_H, ctypes.c_uint64, ctypes.c_double]),
    ("hb_run_until_stable", ctypes.c_int, [_H, ctypes.c_uint64]),
    ("hb_run_until_done", ctypes.c_int, [_H]),
    ("hb_init", ctypes.c_int, [_H]),
    ("hb_iterate", ctypes.c_int, [_H, _P(IterStats)]),
    ("hb_num_iterations", ctypes.c_uint64, [_H]),
    ("hb_get_iteration_stats", ctypes.c_int, [_H, ctypes.c_uint64, _P(IterStats)]),
    ("hb_get_neighborhood_function", ctypes.c_int,
     [_H, _P(ctypes.c_double), ctypes.c_size_t, _P(ctypes.c_size_t)]),
    ("hb_get_sum_of_distances", ctypes.c_int, [_H, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_get_harmonic_centralities", ctypes.c_int, [_H, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_get_discounted_centrality", ctypes.c_int,
     [_H, ctypes.c_size_t, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_get_closeness_centrality", ctypes.c_int, [_H, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_get_lin_centrality", ctypes.c_int, [_H, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_get_nieminen_centrality", ctypes.c_int, [_H, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_get_reachable_nodes", ctypes.c_int, [_H, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_reachable_nodes_from", ctypes.c_int, [_H, ctypes.c_uint64, _P(ctypes.c_double)]),
    ("hb_get_registers", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    ("hb_counter_layout", ctypes.c_int, [_H, _P(ctypes.c_uint64), _P(ctypes.c_int)]),
    ("hb_union_variant_count", ctypes.c_int, []),
    ("hb_tune_degree_buckets", ctypes.c_int,
     [ctypes.POINTER(GraphView), ctypes.POINTER(Options), ctypes.c_uint32, _P(ctypes.c_uint32),
      _P(ctypes.c_uint32), _P(ctypes.c_double)]),
    ("hb_union_variant_chosen", ctypes.c_int, [_H, _P(ctypes.c_int32)]),
    ("hb_last_error", ctypes.c_char_p, [_H]),
    ("hb_global_last_error", ctypes.c_char_p, []),
    ("hb_graph_load_bvgraph", ctypes.c_int, [ctypes.c_char_p, _P(_H)]),
    ("hb_graph_generate_er", ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, _P(_H)]),
    ("hb_graph_generate_rmat", ctypes.c_int,
     [ctypes.c_int, ctypes.c_uint64, ctypes.c_double, ctypes.c_double, ctypes.c_double,
      ctypes.c_uint64, _P(_H)]),
    ("hb_graph_generate_weblike", ctypes.c_int,
     [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64, _P(_H)]),
    ("hb_graph_transpose", ctypes.c_int, [_H, _P(_H)]),
    ("hb_graph_from_csr", ctypes.c_int, [_P(GraphView), _P(_H)]),
    ("hb_graph_get_view", GraphView, [_H]),
    ("hb_graph_free", None, [_H]),
    ("hb_version", ctypes.c_char_p, []),
    ("hb_kernel_launches", ctypes.c_uint64, [_H]),
    ("hb_release_cached_memory", ctypes.c_int, [ctypes.c_int]),
    ("hb_batch_create", ctypes.c_int,
     [_P(GraphView), ctypes.c_uint32, _P(ctypes.c_int32), _P(Options), _P(_H)]),
    ("hb_batch_run_until_done", ctypes.c_int, [_H]),
    ("hb_batch_num_graphs", ctypes.c_uint32, [_H]),
    ("hb_batch_num_iterations", ctypes.c_uint64, [_H, ctypes.c_uint32]),
    ("hb_batch_get_neighborhood_function", ctypes.c_int,
     [_H, ctypes.c_uint32, _P(ctypes.c_double), ctypes.c_size_t, _P(ctypes.c_size_t)]),
    ("hb_batch_get_sum_of_distances", ctypes.c_int,
     [_H, ctypes.c_uint32, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_batch_get_harmonic_centralities", ctypes.c_int,
     [_H, ctypes.c_uint32, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_batch_get_registers", ctypes.c_int, [_H, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t]),
    ("hb_batch_stats", ctypes.c_int,
     [_H, _P(ctypes.c_uint64), _P(ctypes.c_uint64), _P(ctypes.c_uint64), _P(ctypes.c_double)]),
    ("hb_batch_graph_replays", ctypes.c_int, [_H, _P(ctypes.c_uint64), _P(ctypes.c_uint64)]),
    ("hb_batch_destroy", None, [_H]),
    ("hb_server_options_default", None, [_P(ServerOptions)]),
    ("hb_server_create", ctypes.c_int, [_P(ServerOptions), _P(_H)]),
    ("hb_server_submit", ctypes.c_int, [_H, _P(GraphView), _P(Options), _P(ctypes.c_uint64)]),
    ("hb_server_submit_borrowed", ctypes.c_int, [_H, _P(GraphView), _P(Options), _P(ctypes.c_uint64)]),
    ("hb_server_wait", ctypes.c_int, [_H, ctypes.c_uint64, ctypes.c_double]),
    ("hb_server_job_info", ctypes.c_int, [_H, ctypes.c_uint64, _P(JobInfo)]),
    ("hb_server_get_neighborhood_function", ctypes.c_int,
     [_H, ctypes.c_uint64, _P(ctypes.c_double), ctypes.c_size_t, _P(ctypes.c_size_t)]),
    ("hb_server_get_sum_of_distances", ctypes.c_int,
     [_H, ctypes.c_uint64, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_server_get_harmonic_centralities", ctypes.c_int,
     [_H, ctypes.c_uint64, _P(ctypes.c_double), ctypes.c_size_t]),
    ("hb_server_get_registers", ctypes.c_int, [_H, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t]),
    ("hb_server_release", ctypes.c_int, [_H, ctypes.c_uint64]),
    ("hb_server_destroy", None, [_H]),
    ("hb_job_footprint", ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]),
    ("hb_server_last_error", ctypes.c_char_p, []),
    ("hb_server_stats", ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.POINTER(ctypes.c_double)]),
    ("hb_server_step_times", ctypes.c_int, [_H] + [ctypes.POINTER(ctypes.c_double)] * 5),
    ("hb_device_transpose", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_void_p]),
    ("hb_device_transpose_noalloc", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_void_p]),
    ("hb_debug_far_wait", ctypes.c_int, [_H, ctypes.c_uint32, ctypes.c_uint32]),
    ("hb_debug_fail_allocations", ctypes.c_int, [ctypes.c_int64]),
    ("hb_visit_create", ctypes.c_int, [ctypes.POINTER(GraphView), ctypes.c_int, ctypes.c_void_p,
                                       ctypes.POINTER(ctypes.c_void_p)]),
    ("hb_visit_destroy", None, [_H]),
    ("hb_visit_reset", ctypes.c_int, [_H]),
    ("hb_visit_run", ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t,
                                    ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(VisitStats)]),
    ("hb_visit_each", ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    ("hb_visit_last_error", ctypes.c_char_p, [_H]),
    ("hb_exact_sum_sweep", ctypes.c_int, [ctypes.POINTER(GraphView), ctypes.POINTER(GraphView),
                                          ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.POINTER(SweepResult)]),
    ("hb_sweep_last_error", ctypes.c_char_p, []),
]

_lib = None


def tune_degree_buckets(graph, logic, iterations=3, device=0, stream=None):
    """hb_tune_degree_buckets: the (small_max, medium_max) degree-bucket pair
    whose union kernels ran the given standard iterations fastest on this
    graph, and that time in ms. Pass the pair to
    HyperBallBuilder.degree_buckets(); every pair gives identical results."""
    lib = load_library()
    o = Options()
    lib.hb_options_default(ctypes.byref(o))
    o.log2m = logic.log2m
    o.hash_kind = logic.hasher.kind
    o.hash_seed = logic.hasher.seed
    o.num_elements = logic.num_elements
    o.device = int(device)
    o.stream = stream
    gv = graph.view()
    sm, mm, ms = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
    _check(lib.hb_tune_degree_buckets(ctypes.byref(gv), ctypes.byref(o), int(iterations),
                                      ctypes.byref(sm), ctypes.byref(mm), ctypes.byref(ms)))
    return int(sm.value), int(mm.value), float(ms.value)


def union_variant_count():
    """Variants of the union kernels the autotuner chooses from."""
    return int(load_library().hb_union_variant_count())


def load_library(path=None):
    """Loads the in-tree shared library (building nothing). Raises if missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            "libhyperball_gb300.so not built (run __graft_entry__.build()); "
            "there is no CPU fallback")
    lib = ctypes.CDLL(p)
    for name, res, args in EXPORTS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _check(code, handle=None):
    if code == HB_OK:
        return
    lib = load_library()
    msg = (lib.hb_last_error(handle) if handle else lib.hb_global_last_error()) or b""
    raise _ERRORS.get(code, HyperBallError)(code, msg.decode(errors="replace"))


# ---------------------------------------------------------------------------
# graphs
# ---------------------------------------------------------------------------
class _Owned:
    """Array-interface holder that keeps the owner of the memory alive."""

    def __init__(self, owner, ptr, n, typestr):
        self.owner = owner
        self.__array_interface__ = {"data": (ptr, True), "shape": (n,), "typestr": typestr,
                                    "version": 3}


class Graph:
    """Host CSR graph (u64 offsets, u32 successors) owned by the library.

    Stands in for webgraph's RandomAccessGraph; `offsets` is also the
    cumulative outdegree function the reference passes as `D: Succ`."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle) if not isinstance(handle, ctypes.c_void_p) else handle
        lib = load_library()
        v = lib.hb_graph_get_view(self._h)
        self.num_nodes = int(v.num_nodes)
        self.num_arcs = int(v.num_arcs)
        self._off_ptr = ctypes.cast(v.offsets, ctypes.c_void_p).value
        self._suc_ptr = ctypes.cast(v.successors, ctypes.c_void_p).value

    # Views keep the graph alive through their base object, so an array taken
    # from a temporary Graph never outlives the memory it points to.
    @property
    def offsets(self):
        return np.asarray(_Owned(self, self._off_ptr, self.num_nodes + 1, "<u8"))

    @property
    def successors(self):
        if self.num_arcs == 0:
            return np.zeros(0, dtype=np.uint32)
        return np.asarray(_Owned(self, self._suc_ptr, self.num_arcs, "<u4"))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            load_library().hb_graph_free(h)
            self._h = None

    def view(self):
        return GraphView(self.num_nodes, self.num_arcs,
                         self.offsets.ctypes.data_as(_P(ctypes.c_uint64)),
                         self.successors.ctypes.data_as(_P(ctypes.c_uint32)))

    def outdegree(self, node):
        return int(self.offsets[node + 1] - self.offsets[node])

    def successors_of(self, node):
        return self.successors[self.offsets[node]:self.offsets[node + 1]]

    @staticmethod
    def _make(fn, *args):
        h = ctypes.c_void_p()
        _check(fn(*args, ctypes.byref(h)))
        return Graph(h)

    @staticmethod
    def load_bvgraph(basename):
        return Graph._make(load_library().hb_graph_load_bvgraph, os.fsencode(basename))

    @staticmethod
    def erdos_renyi(n, d, seed):
        return Graph._make(load_library().hb_graph_generate_er, n, d, seed)

    @staticmethod
    def rmat(scale, edges_per_node, a=0.57, b=0.19, c=0.19, seed=1):
        return Graph._make(load_library().hb_graph_generate_rmat, scale, edges_per_node, a, b, c, seed)

    @staticmethod
    def weblike(n, cap=100_000, shift=1.266, window=1024, seed=2):
        return Graph._make(load_library().hb_graph_generate_weblike, n, cap, shift, window, seed)

    @staticmethod
    def from_csr(offsets, successors):
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        suc = np.ascontiguousarray(successors, dtype=np.uint32)
        v = GraphView(len(off) - 1, len(suc), off.ctypes.data_as(_P(ctypes.c_uint64)),
                      suc.ctypes.data_as(_P(ctypes.c_uint32)))
        return Graph._make(load_library().hb_graph_from_csr, ctypes.byref(v))

    def transpose(self):
        return Graph._make(load_library().hb_graph_transpose, self._h)


class CsrView:
    """A CSR graph in caller-owned host memory (for instance pinned buffers),
    passed to hb_create without a copy into a library-owned Graph. The caller
    keeps the buffers alive while a builder or HyperBall uses the view."""

    def __init__(self, num_nodes, num_arcs, offsets_ptr, successors_ptr, owner=None):
        self.num_nodes = int(num_nodes)
        self.num_arcs = int(num_arcs)
        self._off_ptr = int(offsets_ptr)
        self._suc_ptr = int(successors_ptr)
        self._owner = owner

    def view(self):
        return GraphView(self.num_nodes, self.num_arcs,
                         ctypes.cast(self._off_ptr, _P(ctypes.c_uint64)),
                         ctypes.cast(self._suc_ptr, _P(ctypes.c_uint32)))


# ---------------------------------------------------------------------------
# HyperLogLog logic descriptor (HyperLogLogBuilder, HLL:234-428)
# ---------------------------------------------------------------------------
class DefaultHasher:
    """Rust std DefaultHasher (SipHash-1-3, zero keys)."""
    kind = HB_HASH_SIP13
    seed = 0


class JenkinsHasher:
    """JenkinsHasherBuilder::new(seed) of the reference's tests."""
    kind = HB_HASH_JENKINS

    def __init__(self, seed):
        self.seed = seed


class HyperLogLog:
    def __init__(self, log2m, hasher, num_elements):
        self.log2m = log2m
        self.hasher = hasher
        self.num_elements = num_elements

    @property
    def num_registers(self):
        return 1 << self.log2m

    @property
    def counter_bytes(self):
        return (1 << self.log2m) * 5 // 8


class HyperLogLogBuilder:
    def __init__(self, n):
        self._n = n
        self._log2m = 4
        self._hasher = DefaultHasher()

    def log_2_num_reg(self, log2m):
        self._log2m = log2m
        return self

    def rsd(self, rsd):
        return self.log_2_num_reg(math.ceil(math.log2((1.106 / rsd) ** 2)))

    def num_elements(self, n):
        self._n = n
        return self

    def build_hasher(self, hasher):
        self._hasher = hasher
        return self

    def word_type(self, _dtype):
        # The device layout is byte-identical for every word type.
        return self

    def build(self):
        if self._log2m < 4:
            raise InvalidArgumentError(
                HB_ERR_INVALID,
                "the logarithm of the number of registers per counter should be at least 4; "
                f"got {self._log2m}")
        return HyperLogLog(self._log2m, self._hasher, self._n)


# ---------------------------------------------------------------------------
# HyperBallBuilder / HyperBall (HB:26-757)
# ---------------------------------------------------------------------------
class HyperBallBuilder:
    DEFAULT_GRANULARITY = 16 * 1024

    def __init__(self, graph, transpose, logic):
        self._graph = graph
        self._transpose = transpose
        self._logic = logic
        self._sod = False
        self._harm = False
        self._disc = []
        self._gran = self.DEFAULT_GRANULARITY
        self._weights = None
        self._weight_seed = 0
        self._transpose_on_device = False
        self._stream = None
        self._device = 0
        self._small = None
        self._medium = None
        self._quirk = True
        self._tma = False
        self._far_rows = None
        self._variant = None
        self._graphs = True

    @staticmethod
    def new(graph, logic):
        """HyperBallBuilder::new (HB:152-181): no transpose, no systolic iterations."""
        return HyperBallBuilder(graph, None, logic)

    @staticmethod
    def with_transpose(graph, transpose, logic):
        """HyperBallBuilder::with_transpose (HB:204-256)."""
        if transpose.num_nodes != graph.num_nodes:
            raise InvalidArgumentError(
                HB_ERR_INVALID, "the transpose should have same number of nodes of the graph")
        if transpose.num_arcs != graph.num_arcs:
            raise InvalidArgumentError(
                HB_ERR_INVALID, "the transpose should have same number of arcs of the graph")
        return HyperBallBuilder(graph, transpose, logic)

    @staticmethod
    def with_hyper_log_log(graph, transpose, log2m, weights=None):
        """HyperBallBuilder::with_hyper_log_log (HB:91-133), default hasher."""
        if weights is not None and len(weights) != graph.num_nodes:
            raise InvalidArgumentError(
                HB_ERR_INVALID, "weights should have length equal to the graph's number of nodes")
        n = int(np.sum(weights)) if weights is not None else graph.num_nodes
        logic = HyperLogLogBuilder(n).log_2_num_reg(log2m).build()
        b = HyperBallBuilder(graph, transpose, logic)
        return b.weights(weights)

    def sum_of_distances(self, flag):
        self._sod = bool(flag)
        return self

    def sum_of_inverse_distances(self, flag):
        self._harm = bool(flag)
        return self

    def arc_granularity(self, g):
        self._gran = int(g)
        return self

    def weights(self, weights, seed=0):
        if weights is not None:
            w = np.ascontiguousarray(weights, dtype=np.uint64)
            if len(w) != self._graph.num_nodes:
                raise InvalidArgumentError(HB_ERR_INVALID, "weights length mismatch")
            self._weights = w
        else:
            self._weights = None
        self._weight_seed = seed
        return self

    def discount_function(self, fn):
        self._disc.append(fn)
        return self

    def no_discount_function(self):
        self._disc = []
        return self

    # GB300 extensions (no reference counterpart)
    def transpose_on_device(self, flag=True):
        self._transpose_on_device = bool(flag)
        return self

    def stream(self, cuda_stream_ptr):
        self._stream = cuda_stream_ptr
        return self

    def device(self, ordinal):
        self._device = int(ordinal)
        return self

    def degree_buckets(self, small_max, medium_max):
        """Nodes of out-degree up to small_max run one lane group each, up to
        medium_max one 8-lane team each, above one CTA each (defaults 64 and
        4096; tune_degree_buckets picks them per graph). The results do not
        depend on them."""
        self._small, self._medium = int(small_max), int(medium_max)
        return self

    def i32_shift_quirk(self, flag):
        self._quirk = bool(flag)
        return self

    def tma_gather(self, flag=True, far_rows=None):
        """Far successors (more than far_rows ids from their node, default
        8192) by TMA gathers instead of plain loads (the default); the
        results are the same."""
        self._tma = bool(flag)
        self._far_rows = far_rows
        return self

    def cuda_graphs(self, flag=True):
        """Replay repeated iteration shapes as CUDA graphs (the default) or
        launch every iteration directly; the results are the same."""
        self._graphs = bool(flag)
        return self

    def union_variant(self, index):
        """A fixed variant of the union kernels (0 .. union_variant_count() - 1)
        instead of the autotuner's choice (None); every variant gives the same
        results."""
        self._variant = None if index is None else int(index)
        return self

    def build(self):
        return HyperBall(self)


class HyperBall:
    def __init__(self, b):
        lib = load_library()
        self._lib = lib
        self._b = b
        self.num_nodes = b._graph.num_nodes
        o = Options()
        lib.hb_options_default(ctypes.byref(o))
        o.log2m = b._logic.log2m
        o.hash_kind = b._logic.hasher.kind
        o.hash_seed = b._logic.hasher.seed
        o.num_elements = b._logic.num_elements
        flags = 0
        if b._sod:
            flags |= HB_SUM_OF_DISTANCES
        if b._harm:
            flags |= HB_SUM_OF_INVERSE_DISTANCES
        if b._transpose is None and b._transpose_on_device:
            flags |= HB_TRANSPOSE_ON_DEVICE
        if not b._quirk:
            flags |= HB_NO_I32_SHIFT_QUIRK
        if b._tma:
            flags |= HB_TMA_GATHER
        if not b._graphs:
            flags |= HB_NO_GRAPHS
        if b._far_rows is not None:
            o.far_rows = int(b._far_rows)
        o.flags = flags
        o.arc_granularity = b._gran
        o.device = b._device
        o.stream = b._stream
        if b._small is not None:
            o.small_max_degree = b._small
        if b._medium is not None:
            o.medium_max_degree = b._medium
        if b._variant is not None:
            o.union_variant = b._variant
        if b._weights is not None:
            o.weights = b._weights.ctypes.data_as(_P(ctypes.c_uint64))
            o.weight_seed = b._weight_seed
        self._gv = b._graph.view()
        self._tv = b._transpose.view() if b._transpose is not None else None
        h = ctypes.c_void_p()
        _check(lib.hb_create(ctypes.byref(self._gv),
                             ctypes.byref(self._tv) if self._tv is not None else None,
                             ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self._disc_refs = []
        for fn in b._disc:
            cb = DISCOUNT_FN(lambda d, _ctx, f=fn: float(f(int(d))))
            self._disc_refs.append(cb)
            _check(lib.hb_add_discount_function(h, cb, None), h)
        cb = ctypes.c_uint64()
        rs = ctypes.c_int()
        _check(lib.hb_counter_layout(h, ctypes.byref(cb), ctypes.byref(rs)), h)
        self.counter_bytes = int(cb.value)
        self.register_size = int(rs.value)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.hb_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- running ---------------------------------------------------------
    def run(self, upper_bound, threshold=None):
        t = float("nan") if threshold is None else float(threshold)
        _check(self._lib.hb_run(self._h, min(int(upper_bound), 2**64 - 1), t), self._h)

    def run_until_stable(self, upper_bound):
        _check(self._lib.hb_run_until_stable(self._h, min(int(upper_bound), 2**64 - 1)), self._h)

    def run_until_done(self):
        _check(self._lib.hb_run_until_done(self._h), self._h)

    def init(self):
        _check(self._lib.hb_init(self._h), self._h)

    def debug_far_wait(self, polls=0, extra_tx_bytes=0):
        """Test hook (hb_debug_far_wait): bounds the TMA far-gather waits to
        `polls` polls and adds bytes that never arrive to every expected
        count, so the timeout path runs. (0, 0) restores the defaults."""
        _check(self._lib.hb_debug_far_wait(self._h, int(polls), int(extra_tx_bytes)), self._h)

    def iterate(self):
        s = IterStats()
        _check(self._lib.hb_iterate(self._h, ctypes.byref(s)), self._h)
        return s.as_dict()

    @property
    def iteration(self):
        return int(self._lib.hb_num_iterations(self._h))

    def iteration_stats(self):
        out = []
        for i in range(self.iteration):
            s = IterStats()
            _check(self._lib.hb_get_iteration_stats(self._h, i, ctypes.byref(s)), self._h)
            out.append(s.as_dict())
        return out

    # -- results ---------------------------------------------------------
    def neighborhood_function(self):
        ln = ctypes.c_size_t()
        _check(self._lib.hb_get_neighborhood_function(self._h, None, 0, ctypes.byref(ln)), self._h)
        out = np.zeros(ln.value, dtype=np.float64)
        _check(self._lib.hb_get_neighborhood_function(
            self._h, out.ctypes.data_as(_P(ctypes.c_double)), ln.value, ctypes.byref(ln)), self._h)
        return out

    def _vec(self, fn, *pre, out=None):
        # out: an optional C-contiguous float64 array of num_nodes elements
        # to fill (for instance page-locked memory), else a new array
        if out is None:
            out = np.zeros(self.num_nodes, dtype=np.float64)
        elif (out.dtype != np.float64 or out.shape != (self.num_nodes,)
              or not out.flags.c_contiguous or not out.flags.writeable):
            raise ValueError("out must be a writable C-contiguous float64 array of num_nodes elements")
        _check(fn(self._h, *pre, out.ctypes.data_as(_P(ctypes.c_double)), self.num_nodes), self._h)
        return out

    def sum_of_distances(self, out=None):
        return self._vec(self._lib.hb_get_sum_of_distances, out=out)

    def harmonic_centralities(self, out=None):
        return self._vec(self._lib.hb_get_harmonic_centralities, out=out)

    def discounted_centrality(self, index, out=None):
        return self._vec(self._lib.hb_get_discounted_centrality, index, out=out)

    def closeness_centrality(self, out=None):
        return self._vec(self._lib.hb_get_closeness_centrality, out=out)

    def lin_centrality(self, out=None):
        return self._vec(self._lib.hb_get_lin_centrality, out=out)

    def nieminen_centrality(self, out=None):
        return self._vec(self._lib.hb_get_nieminen_centrality, out=out)

    def reachable_nodes(self, out=None):
        return self._vec(self._lib.hb_get_reachable_nodes, out=out)

    def reachable_nodes_from(self, node):
        v = ctypes.c_double()
        _check(self._lib.hb_reachable_nodes_from(self._h, node, ctypes.byref(v)), self._h)
        return v.value

    def kernel_launches(self):
        """CUDA kernels the library launched for this instance so far."""
        return int(self._lib.hb_kernel_launches(self._h))

    def union_variants_chosen(self):
        """The union-kernel variant kept for standard iterations merging every
        successor, standard iterations merging modified successors, and
        systolic iterations (-1: still being timed)."""
        c = (ctypes.c_int32 * 3)()
        _check(self._lib.hb_union_variant_chosen(self._h, c), self._h)
        return list(c)

    def registers(self, which=HB_CURRENT_STATE, out=None):
        """Raw counter bytes (num_nodes x counter_bytes), reference layout;
        `out` is an optional C-contiguous uint8 array of that shape to fill."""
        shape = (self.num_nodes, self.counter_bytes)
        if out is None:
            out = np.zeros(shape, dtype=np.uint8)
        elif out.dtype != np.uint8 or out.shape != shape or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous uint8 array of num_nodes x counter_bytes")
        _check(self._lib.hb_get_registers(self._h, which, out.ctypes.data, out.nbytes), self._h)
        return out


# ---------------------------------------------------------------------------
# batches (no reference counterpart): many independent instances in one pass
# ---------------------------------------------------------------------------
class HyperBallBatch:
    """Independent HyperBall instances run together: graphs[i] with log2m[i];
    the hasher and the requested outputs are shared. For each graph the
    results equal those of HyperBallBuilder(...).build().run_until_done()."""

    def __init__(self, graphs, log2ms, hasher=None, sum_of_distances=False,
                 sum_of_inverse_distances=False, transpose_on_device=True, device=0,
                 stream=None):
        lib = load_library()
        self._lib = lib
        self._graphs = list(graphs)
        if len(log2ms) != len(self._graphs):
            raise InvalidArgumentError(HB_ERR_INVALID, "one log2m per graph")
        hasher = hasher or DefaultHasher()
        o = Options()
        lib.hb_options_default(ctypes.byref(o))
        o.hash_kind = hasher.kind
        o.hash_seed = hasher.seed
        o.device = device
        o.stream = stream
        flags = 0
        if sum_of_distances:
            flags |= HB_SUM_OF_DISTANCES
        if sum_of_inverse_distances:
            flags |= HB_SUM_OF_INVERSE_DISTANCES
        if transpose_on_device:
            flags |= HB_TRANSPOSE_ON_DEVICE
        o.flags = flags
        self._views = (GraphView * len(self._graphs))(*[g.view() for g in self._graphs])
        self._log2m = (ctypes.c_int32 * len(self._graphs))(*[int(x) for x in log2ms])
        self.num_nodes = [g.num_nodes for g in self._graphs]
        self.counter_bytes = [(1 << int(x)) * 5 // 8 for x in log2ms]
        h = ctypes.c_void_p()
        _check(lib.hb_batch_create(self._views, len(self._graphs), self._log2m, ctypes.byref(o),
                                   ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.hb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __len__(self):
        return len(self._graphs)

    def run_until_done(self):
        _check(self._lib.hb_batch_run_until_done(self._h))

    def iterations(self, i):
        return int(self._lib.hb_batch_num_iterations(self._h, i))

    def neighborhood_function(self, i):
        n = ctypes.c_size_t()
        _check(self._lib.hb_batch_get_neighborhood_function(self._h, i, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.float64)
        _check(self._lib.hb_batch_get_neighborhood_function(
            self._h, i, out.ctypes.data_as(_P(ctypes.c_double)), n.value, ctypes.byref(n)))
        return out

    def _vec(self, fn, i):
        out = np.zeros(self.num_nodes[i], dtype=np.float64)
        _check(fn(self._h, i, out.ctypes.data_as(_P(ctypes.c_double)), self.num_nodes[i]))
        return out

    def sum_of_distances(self, i):
        return self._vec(self._lib.hb_batch_get_sum_of_distances, i)

    def harmonic_centralities(self, i):
        return self._vec(self._lib.hb_batch_get_harmonic_centralities, i)

    def registers(self, i):
        out = np.zeros((self.num_nodes[i], self.counter_bytes[i]), dtype=np.uint8)
        _check(self._lib.hb_batch_get_registers(self._h, i, out.ctypes.data, out.size))
        return out

    def stats(self):
        it, vis, upd, ms = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_double()
        _check(self._lib.hb_batch_stats(self._h, ctypes.byref(it), ctypes.byref(vis),
                                        ctypes.byref(upd), ctypes.byref(ms)))
        rep, total = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._lib.hb_batch_graph_replays(self._h, ctypes.byref(rep), ctypes.byref(total)))
        return {"iterations": it.value, "visited_arcs": vis.value, "register_updates": upd.value,
                "union_ms": ms.value, "graph_replays": rep.value, "group_iterations": total.value}


# ---------------------------------------------------------------------------
# served jobs (no reference counterpart)
# ---------------------------------------------------------------------------
def _scheck(code):
    if code == HB_OK:
        return
    msg = load_library().hb_server_last_error() or b""
    raise _ERRORS.get(code, HyperBallError)(code, msg.decode(errors="replace"))


class HyperBallServer:
    """Continuous admission of HyperBall jobs against a device-memory budget;
    every job returns what HyperBallBuilder(...).build().run_until_done()
    returns for its graph alone."""

    def __init__(self, hbm_budget_bytes=150 * 10**9, max_active=16, keep_registers=False,
                 device=0, setup_threads=0, union_sm_reserve=None):
        lib = load_library()
        self._lib = lib
        o = ServerOptions()
        lib.hb_server_options_default(ctypes.byref(o))
        o.hbm_budget_bytes = int(hbm_budget_bytes)
        o.max_active = int(max_active)
        o.keep_registers = 1 if keep_registers else 0
        o.device = int(device)
        o.setup_threads = int(setup_threads)
        if union_sm_reserve is not None:
            o.union_sm_reserve = int(union_sm_reserve)
        h = ctypes.c_void_p()
        _scheck(lib.hb_server_create(ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self._nodes = {}
        self._borrowed = {}

    def stats(self):
        """Stepping statistics (hb_server_stats, hb_server_step_times):
        steps, their wall time on the stepping thread, the device time of the
        union parts, the job-steps (jobs per step, summed), and where the
        steps' time went (device time before, in and after the union parts;
        host time launching and waiting)."""
        st, sm, um, js = ctypes.c_uint64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
        lm = ctypes.c_double()
        _scheck(self._lib.hb_server_stats(self._h, ctypes.byref(st), ctypes.byref(sm),
                                          ctypes.byref(um), ctypes.byref(js), ctypes.byref(lm)))
        pre, uni, post, host, wait = (ctypes.c_double() for _ in range(5))
        _scheck(self._lib.hb_server_step_times(self._h, ctypes.byref(pre), ctypes.byref(uni),
                                               ctypes.byref(post), ctypes.byref(host),
                                               ctypes.byref(wait)))
        return {"steps": st.value, "step_ms": sm.value, "union_ms": um.value,
                "job_steps": js.value, "launch_ms": lm.value,
                "device_ms": {"pre": pre.value, "union": uni.value, "post": post.value},
                "host_ms": host.value, "wait_ms": wait.value}

    def submit(self, graph, log2m, hasher=None, sum_of_distances=False,
               sum_of_inverse_distances=False, transpose_on_device=True, borrow=False):
        """Queues a job. borrow=True skips the copy of the graph: the graph
        object is then kept alive by the server until the job is released."""
        hasher = hasher or DefaultHasher()
        o = Options()
        self._lib.hb_options_default(ctypes.byref(o))
        o.log2m = int(log2m)
        o.hash_kind = hasher.kind
        o.hash_seed = hasher.seed
        o.num_elements = graph.num_nodes
        o.flags = ((HB_SUM_OF_DISTANCES if sum_of_distances else 0)
                   | (HB_SUM_OF_INVERSE_DISTANCES if sum_of_inverse_distances else 0)
                   | (HB_TRANSPOSE_ON_DEVICE if transpose_on_device else 0))
        v = graph.view()
        job = ctypes.c_uint64()
        submit = self._lib.hb_server_submit_borrowed if borrow else self._lib.hb_server_submit
        _scheck(submit(self._h, ctypes.byref(v), ctypes.byref(o), ctypes.byref(job)))
        self._nodes[job.value] = (graph.num_nodes, (1 << int(log2m)) * 5 // 8)
        if borrow:
            self._borrowed[job.value] = graph
        return job.value

    def wait(self, job, timeout=None):
        _scheck(self._lib.hb_server_wait(self._h, job, -1.0 if timeout is None else float(timeout)))

    def info(self, job):
        i = JobInfo()
        _scheck(self._lib.hb_server_job_info(self._h, job, ctypes.byref(i)))
        return i.as_dict()

    def neighborhood_function(self, job):
        n = ctypes.c_size_t()
        _scheck(self._lib.hb_server_get_neighborhood_function(self._h, job, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.float64)
        _scheck(self._lib.hb_server_get_neighborhood_function(
            self._h, job, out.ctypes.data_as(_P(ctypes.c_double)), n.value, ctypes.byref(n)))
        return out

    def _vec(self, fn, job):
        out = np.zeros(self._nodes[job][0], dtype=np.float64)
        _scheck(fn(self._h, job, out.ctypes.data_as(_P(ctypes.c_double)), len(out)))
        return out

    def sum_of_distances(self, job):
        return self._vec(self._lib.hb_server_get_sum_of_distances, job)

    def harmonic_centralities(self, job):
        return self._vec(self._lib.hb_server_get_harmonic_centralities, job)

    def registers(self, job):
        n, cb = self._nodes[job]
        out = np.zeros((n, cb), dtype=np.uint8)
        _scheck(self._lib.hb_server_get_registers(self._h, job, out.ctypes.data, out.size))
        return out

    def release(self, job):
        _scheck(self._lib.hb_server_release(self._h, job))
        self._nodes.pop(job, None)
        self._borrowed.pop(job, None)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.hb_server_destroy(self._h)
            self._h = None
        self._borrowed = {}

    def __del__(self):
        self.close()


def job_footprint(num_nodes, num_arcs, log2m):
    """Device bytes a server reserves for a job of this size."""
    return int(load_library().hb_job_footprint(num_nodes, num_arcs, log2m))


def release_cached_memory(device=0):
    """Returns the device memory the library keeps for reuse (freed by
    closed handles) to the device."""
    _check(load_library().hb_release_cached_memory(device))


# ---------------------------------------------------------------------------
# breadth-first visits (src/algo/visits/breadth_first/par_fair.rs)
# ---------------------------------------------------------------------------
def debug_fail_allocations(after):
    """Test hook (hb_debug_fail_allocations): the (after + 1)-th device
    allocation of a handle from now fails once with HB_ERR_OOM; -1 turns
    it off."""
    load_library().hb_debug_fail_allocations(int(after))


SWEEP_LEVELS = {"all": 0, "all_forward": 1, "radius_diameter": 2, "diameter": 3, "radius": 4}
SWEEP_NONE = 2**64 - 1


def exact_sum_sweep(graph, transpose=None, level="all", radial_vertices=None, device=0,
                    stream=None):
    """ExactSumSweep (src/algo/exact_sum_sweep/) on the device:
    OutputLevel::compute_directed(graph, transpose, radial_vertices) with a
    transpose, compute_undirected(graph) of a symmetric graph without one.
    `level`: "all", "all_forward", "radius_diameter", "diameter", "radius".
    Returns the output's fields as a dict (forward / backward eccentricities
    as uint64 arrays where the level computes them; a radius without radial
    vertices and iteration counts the level does not compute are
    SWEEP_NONE = 2^64 - 1), plus "sweeps" (visits run) and "device_ms"."""
    lib = load_library()
    lv = SWEEP_LEVELS[level]
    g = graph.view()
    t = transpose.view() if transpose is not None else None
    n = graph.num_nodes
    rad = None
    if radial_vertices is not None:
        rad = np.ascontiguousarray(radial_vertices, dtype=np.uint8)
        if rad.shape != (n,):
            raise ValueError("radial_vertices must have one entry per node")
    eff = 1 if (transpose is None and lv == 0) else lv
    fe = np.zeros(max(n, 1), dtype=np.uint64) if eff in (0, 1) else None
    be = np.zeros(max(n, 1), dtype=np.uint64) if eff == 0 else None
    res = SweepResult()
    code = lib.hb_exact_sum_sweep(ctypes.byref(g), ctypes.byref(t) if t is not None else None, lv,
                                  rad.ctypes.data if rad is not None else None, int(device), stream,
                                  fe.ctypes.data if fe is not None else None,
                                  be.ctypes.data if be is not None else None, ctypes.byref(res))
    if code:
        msg = (lib.hb_sweep_last_error() or b"").decode(errors="replace")
        raise _ERRORS.get(code, HyperBallError)(code, msg)
    out = {f: getattr(res, f) for f, _ in SweepResult._fields_}
    if fe is not None:
        out["forward_eccentricities"] = fe[:n]
    if be is not None:
        out["backward_eccentricities"] = be[:n]
    return out


class ParFair:
    """The fair parallel breadth-first visit of the reference (ParFairPred /
    ParFairNoPred, par_fair.rs:92-124) on the device. The reference reports
    a visit through a callback; par_visit returns its Unknown events as
    arrays (nodes, preds, distances), level by level. The visited set
    persists across visits until reset(). `granularity` is accepted for
    parity with ParFair::new; the device balances work by warps."""

    def __init__(self, graph, granularity=1, device=0, stream=None):
        lib = load_library()
        self._lib = lib
        self._graph = graph  # the view below points into it
        self.num_nodes = graph.num_nodes
        self.granularity = int(granularity)
        h = ctypes.c_void_p()
        v = graph.view()
        code = lib.hb_visit_create(ctypes.byref(v), int(device), stream, ctypes.byref(h))
        if code:
            msg = (lib.hb_visit_last_error(None) or b"").decode(errors="replace")
            raise _ERRORS.get(code, HyperBallError)(code, msg)
        self._h = h

    def _check(self, code):
        if code:
            msg = (self._lib.hb_visit_last_error(self._h) or b"").decode(errors="replace")
            raise _ERRORS.get(code, HyperBallError)(code, msg)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.hb_visit_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def reset(self):
        """Parallel::reset (par_fair.rs:322-324)."""
        self._check(self._lib.hb_visit_reset(self._h))

    def par_visit(self, roots, max_distance=None):
        """One visit from `roots` (visited roots skipped); nodes farther than
        max_distance are neither reported nor marked. Returns (nodes, preds,
        distances) as uint32 arrays, and the visit's statistics."""
        r = np.ascontiguousarray(np.asarray(roots, dtype=np.uint64).reshape(-1))
        n = max(self.num_nodes, 1)
        nodes = np.zeros(n, dtype=np.uint32)
        preds = np.zeros(n, dtype=np.uint32)
        dists = np.zeros(n, dtype=np.uint32)
        st = VisitStats()
        md = 2**64 - 1 if max_distance is None else int(max_distance)
        self._check(self._lib.hb_visit_run(self._h, r.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                           len(r), md, nodes.ctypes.data, preds.ctypes.data,
                                           dists.ctypes.data, n, ctypes.byref(st)))
        k = st.visited
        return nodes[:k], preds[:k], dists[:k], {"visited": st.visited, "levels": st.levels,
                                                 "known_arcs": st.known_arcs,
                                                 "device_ms": st.device_ms}

    def visit_each(self, roots, dist=None, pred=None):
        """visit([root]) for each root in order (tests/test_bfv.rs:89-101):
        dist[node] (and pred[node]) for every node a visit reaches."""
        r = np.ascontiguousarray(np.asarray(roots, dtype=np.uint64).reshape(-1))
        if dist is None:
            dist = np.zeros(self.num_nodes, dtype=np.uint32)
        pp = pred.ctypes.data if pred is not None else None
        self._check(self._lib.hb_visit_each(self._h, r.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                            len(r), dist.ctypes.data, pp, self.num_nodes))
        return dist

