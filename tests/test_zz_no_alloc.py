"""hb_device_transpose_noalloc (fixed device scratch, no allocation) against
hb_device_transpose (allocating) and the host transpose. Collected last so it
also runs after every other test in the same process."""
import ctypes

import numpy as np
import pytest

import hyperball_gb300 as hb

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

NOALLOC_MAX_NODES = 1 << 20


def _device_csr(g):
    off = np.asarray(g.offsets).view(np.int64).copy()
    succ = np.asarray(g.successors).view(np.int32).copy()
    if len(succ) == 0:
        succ = np.zeros(1, dtype=np.int32)
    return torch.from_numpy(off).cuda(), torch.from_numpy(succ).cuda()


def _transpose(fn, n, m, d_off, d_succ, stream=None):
    t_off = torch.full((n + 1,), -1, dtype=torch.int64, device="cuda")
    t_succ = torch.full((max(m, 1),), -1, dtype=torch.int32, device="cuda")
    rc = fn(d_off.data_ptr(), d_succ.data_ptr(), n, m, t_off.data_ptr(), t_succ.data_ptr(), stream)
    torch.cuda.synchronize()
    msg = hb.load_library().hb_global_last_error()
    return rc, msg, t_off.cpu().numpy().view(np.uint64), t_succ.cpu().numpy().view(np.uint32)[:m]


def _sorted_rows(off, succ):
    n = len(off) - 1
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(off.astype(np.int64)))
    return succ[np.lexsort((succ, rows))]


@pytest.mark.parametrize("make", [lambda: hb.Graph.weblike(1 << 16, seed=5),
                                  lambda: hb.Graph.erdos_renyi(20000, 7, 11)])
def test_noalloc_matches_allocating_transpose(make):
    lib = hb.load_library()
    g = make()
    n, m = g.num_nodes, g.num_arcs
    ref = g.transpose()
    ref_off, ref_succ = np.asarray(ref.offsets), np.asarray(ref.successors)
    d_off, d_succ = _device_csr(g)
    # two calls in a row of each, interleaved
    calls = [lib.hb_device_transpose, lib.hb_device_transpose_noalloc,
             lib.hb_device_transpose_noalloc, lib.hb_device_transpose]
    for fn in calls:
        rc, msg, t_off, t_succ = _transpose(fn, n, m, d_off, d_succ)
        assert rc == hb.HB_OK, msg
        np.testing.assert_array_equal(t_off, ref_off)
        np.testing.assert_array_equal(_sorted_rows(t_off, t_succ), ref_succ)


def test_noalloc_on_a_stream_and_at_the_size_limit():
    lib = hb.load_library()
    # a ring at exactly the largest accepted size
    n = NOALLOC_MAX_NODES
    off = np.arange(n + 1, dtype=np.uint64)
    succ = ((np.arange(n, dtype=np.uint64) + 1) % n).astype(np.uint32)
    g = hb.Graph.from_csr(off, succ)
    d_off, d_succ = _device_csr(g)
    s = torch.cuda.Stream()
    rc, msg, t_off, t_succ = _transpose(lib.hb_device_transpose_noalloc, n, n, d_off, d_succ,
                                        ctypes.c_void_p(s.cuda_stream))
    assert rc == hb.HB_OK, msg
    np.testing.assert_array_equal(t_off, off)
    np.testing.assert_array_equal(t_succ, ((np.arange(n) - 1) % n).astype(np.uint32))


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = hb.load_library()
    d_off = torch.zeros(4, dtype=torch.int64, device="cuda")
    d_succ = torch.zeros(4, dtype=torch.int32, device="cuda")
    n = NOALLOC_MAX_NODES + 1
    rc = lib.hb_device_transpose_noalloc(d_off.data_ptr(), d_succ.data_ptr(), n, 0,
                                         d_off.data_ptr(), d_succ.data_ptr(), None)
    assert rc == hb.HB_ERR_INVALID
    assert b"at most 1048576" in lib.hb_global_last_error()


class _CurrentPool:
    """The current memory pool of device 0 through the driver API (the pool
    cudaMallocAsync draws from): its used-memory high watermark can be reset
    and read, so a call that allocated from it, even briefly, shows."""
    USED_MEM_CURRENT, USED_MEM_HIGH = 7, 8  # CUmemPool_attribute

    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(dev), 0) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetMemPool(ctypes.byref(self.pool), dev) == 0

    def _get(self, attr):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def reset_high(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def used_high(self):
        return self._get(self.USED_MEM_HIGH)


def test_noalloc_allocates_no_device_memory():
    lib = hb.load_library()
    g = hb.Graph.weblike(1 << 18, seed=9)
    n, m = g.num_nodes, g.num_arcs
    d_off, d_succ = _device_csr(g)
    t_off = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    t_succ = torch.empty(m, dtype=torch.int32, device="cuda")
    args = (d_off.data_ptr(), d_succ.data_ptr(), n, m, t_off.data_ptr(), t_succ.data_ptr(), None)
    pool = _CurrentPool()
    # the allocating transpose shows up in the pool's watermark ...
    torch.cuda.synchronize()
    pool.reset_high()
    assert lib.hb_device_transpose(*args) == hb.HB_OK
    assert pool.used_high() > 0
    # ... the fixed-scratch one does not, and the free device memory stays put
    lib.hb_device_transpose_noalloc(*args)  # first call on the device: address lookup
    torch.cuda.synchronize()
    pool.reset_high()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        assert lib.hb_device_transpose_noalloc(*args) == hb.HB_OK
    torch.cuda.synchronize()
    assert pool.used_high() == 0
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_invalid_graphs_and_handles_empty_ones():
    lib = hb.load_library()
    # successor out of range: refused before any kernel indexes with it
    off = torch.tensor([0, 1, 2], dtype=torch.int64, device="cuda")
    succ = torch.tensor([1, 7], dtype=torch.int32, device="cuda")
    for fn in (lib.hb_device_transpose, lib.hb_device_transpose_noalloc):
        rc, msg, _, _ = _transpose(fn, 2, 2, off, succ)
        assert rc == hb.HB_ERR_INVALID and b"successors" in msg
    # no arcs
    off0 = torch.zeros(4, dtype=torch.int64, device="cuda")
    for fn in (lib.hb_device_transpose, lib.hb_device_transpose_noalloc):
        rc, msg, t_off, _ = _transpose(fn, 3, 0, off0, succ)
        assert rc == hb.HB_OK, msg
        np.testing.assert_array_equal(t_off, np.zeros(4, dtype=np.uint64))
