"""Served HyperBall: jobs admitted against a device-memory budget overlap on
the device, and every job's results equal the same graph run alone (registers
bit-exact, iteration count, neighbourhood function and per-node sums to 1e-12)."""
import numpy as np
import pytest

import hyperball_gb300 as hb

RTOL = 1e-12


def _jobs():
    return [
        (hb.Graph.erdos_renyi(2000, 5, 21), 4),
        (hb.Graph.rmat(11, 16, seed=23), 6),
        (hb.Graph.weblike(6000, seed=25), 8),
        (hb.Graph.erdos_renyi(1500, 12, 27), 6),
        (hb.Graph.rmat(10, 8, seed=29), 8),
        (hb.Graph.weblike(3000, seed=31), 4),
        (hb.Graph.erdos_renyi(500, 3, 33), 8),
        (hb.Graph.rmat(12, 16, seed=35), 6),
    ]


def _alone(g, log2m):
    logic = hb.HyperLogLogBuilder(g.num_nodes).log_2_num_reg(log2m).build()
    h = (hb.HyperBallBuilder.new(g, logic).transpose_on_device(True)
         .sum_of_distances(True).sum_of_inverse_distances(True).build())
    h.run_until_done()
    out = dict(iterations=h.iteration, registers=h.registers(), nf=h.neighborhood_function(),
               sod=h.sum_of_distances(), harm=h.harmonic_centralities())
    h.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("max_active,borrow", [(1, False), (3, False), (16, False), (16, True)])
def test_served_jobs_equal_jobs_alone(max_active, borrow):
    jobs = _jobs()
    s = hb.HyperBallServer(max_active=max_active, keep_registers=True)
    ids = [s.submit(g, l2m, sum_of_distances=True, sum_of_inverse_distances=True, borrow=borrow)
           for g, l2m in jobs]
    for j in ids:
        s.wait(j, timeout=600)
    for j, (g, l2m) in zip(ids, jobs):
        want = _alone(g, l2m)
        info = s.info(j)
        assert info["state"] == hb.HB_JOB_DONE and info["iterations"] == want["iterations"]
        assert info["latency_ms"] >= info["run_ms"] > 0
        np.testing.assert_array_equal(s.registers(j), want["registers"])
        np.testing.assert_allclose(s.neighborhood_function(j), want["nf"], rtol=RTOL)
        np.testing.assert_allclose(s.sum_of_distances(j), want["sod"], rtol=RTOL)
        np.testing.assert_allclose(s.harmonic_centralities(j), want["harm"], rtol=RTOL)
        s.release(j)
    st = s.stats()
    assert st["steps"] > 0 and st["job_steps"] >= st["steps"]
    dev = st["device_ms"]
    assert dev["union"] == pytest.approx(st["union_ms"]) and dev["union"] > 0
    assert dev["pre"] >= 0 and dev["post"] >= 0 and st["wait_ms"] > 0
    assert dev["pre"] + dev["union"] + dev["post"] <= st["step_ms"] * 1.05
    s.close()


@pytest.mark.gpu
def test_budget_admission_serialises_jobs_that_do_not_fit_together():
    jobs = _jobs()[:4]
    big = max(hb.job_footprint(g.num_nodes, g.num_arcs, l2m) for g, l2m in jobs)
    # room for one job at a time
    s = hb.HyperBallServer(hbm_budget_bytes=big, max_active=8)
    ids = [s.submit(g, l2m, sum_of_distances=True) for g, l2m in jobs]
    for j in ids:
        s.wait(j, timeout=600)
    infos = [s.info(j) for j in ids]
    assert all(i["state"] == hb.HB_JOB_DONE for i in infos)
    # later jobs queued while earlier ones held the budget
    assert infos[-1]["queue_ms"] >= infos[0]["run_ms"] * 0.5
    for j, (g, l2m) in zip(ids, jobs):
        np.testing.assert_allclose(s.sum_of_distances(j), _alone(g, l2m)["sod"], rtol=RTOL)
    s.close()


def test_server_rejects_jobs_larger_than_the_budget(product_lib):
    s = hb.HyperBallServer(hbm_budget_bytes=1 << 20)
    g = hb.Graph.erdos_renyi(100000, 8, 1)
    with pytest.raises(hb.InvalidArgumentError):
        s.submit(g, 8)
    with pytest.raises(hb.InvalidArgumentError):
        s.wait(12345)
    s.close()


def test_server_reports_failures_loudly_without_a_device(product_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    s = hb.HyperBallServer()
    j = s.submit(hb.Graph.erdos_renyi(200, 4, 2), 6)
    with pytest.raises(hb.NoDeviceError):
        s.wait(j, timeout=60)
    assert s.info(j)["state"] == hb.HB_JOB_FAILED
    with pytest.raises(hb.NotRunError):
        s.neighborhood_function(j)
    s.close()
