"""Failures made on the host, never on the device: a device allocation
failing during creation (hb_debug_fail_allocations stands for a cudaMalloc
failure) is reported as HB_ERR_OOM, releases what the failed creation held,
and leaves the library able to run an oracle-exact HyperBall right after."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_allocation_failures_during_creation(hb, oracle):
    g = hb.Graph.weblike(20_000, cap=2000, window=256, seed=4)
    logic = hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(6).build()

    def build():
        return (hb.HyperBallBuilder.new(g, logic).transpose_on_device(True)
                .sum_of_distances(True).sum_of_inverse_distances(True).build())

    failed = 0
    for k in (0, 1, 2, 5, 10, 20, 30):
        hb.debug_fail_allocations(k)
        try:
            h = build()
        except hb.HyperBallError as e:
            assert e.code == hb.HB_ERR_OOM, e
            assert "injected" in str(e)
            failed += 1
        else:
            h.close()
        finally:
            hb.debug_fail_allocations(-1)
    assert failed >= 5
    # a clean creation afterwards equals the oracle
    h = build()
    h.run_until_done()
    t = g.transpose()
    orc = oracle.OracleHyperBall(g.offsets, g.successors, 6, sod=True, harm=True,
                                 t_offsets=t.offsets, t_successors=t.successors)
    orc.run_until_done()
    assert h.iteration == orc.iteration
    np.testing.assert_array_equal(h.registers(0), orc.registers(0))
    h.close()
