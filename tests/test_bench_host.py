"""Host logic of bench.py on the CPU: replica aggregation over two gloo ranks,
the union-kernel byte model, the clock summary and the reference arm."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    r = bench.Ranks(world, "gloo")
    r.barrier()
    # rank k took 1 + k seconds; every rank must see the slowest
    slowest = r.max(1.0 + rank)
    out[rank] = (slowest, bench.job_value(world, 3, 1000, slowest))
    r.barrier()
    r.close()


def test_replicas_take_max_over_ranks_gloo():
    world = 2
    out = mp.Manager().dict()
    mp.start_processes(_replica, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    assert out[0] == out[1] == (2.0, world * 3 * 1000 / 2.0)


def test_single_process_ranks_are_noops():
    r = bench.Ranks(1, "gloo")
    r.barrier()
    assert r.max(3.5) == 3.5
    r.close()
    assert bench.job_value(1, 2, 10, 4.0) == 5.0


def test_union_model_bytes():
    n = 1000
    stats = [
        {"scanned_nodes": 1000, "scanned_arcs": 8000, "visited_arcs": 7900, "modified_counters": 900},
        {"scanned_nodes": 300, "scanned_arcs": 2000, "visited_arcs": 500, "modified_counters": 0},
    ]
    w, f = bench.COUNTER_BYTES, 16 + 16 * bench.N_SUMS
    got = bench.union_model_bytes(stats, n)
    assert got[0] == 8 * 1001 + 4 * 8000 + w * min(n, 7900) + 2 * w * 1000 + n // 4
    assert got[1] == 8 * 301 + 4 * 2000 + w * min(900, 500) + 2 * w * 300 + n // 4
    ext = bench.union_model_bytes(stats, n, with_sums=True)
    assert ext[0] == got[0] + f * 900 and ext[1] == got[1]


def test_clock_summary():
    rows = [
        ["0", "1980", "2070", "900.1", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
        ["0", "2070", "2070", "1300.0", "0x4", "Not Active", "Not Active", "Not Active", "Active"],
        ["0", "2010", "2070", "1200.0", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
    ]
    c = bench.ClockSampler.summarise(rows)
    assert c["sm_mhz"] == 2010 and c["sm_max_mhz"] == 2070
    assert c["reasons"] == ["sw_power_cap"] and c["samples"] == 3
    assert bench.ClockSampler.summarise([]) is None


def test_reference_arm_line():
    """`--impl reference` runs the CPU restatement and prints the contract line."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--log2n", "12", "--steps", "2", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["value"] > 0 and line["unit"] == bench.UNIT
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    # the same config keys as the GPU arm's line, filled from the CPU run
    assert set(line["config"]) == {"workload", "nodes", "graph", "log2m", "hash", "mode",
                                   "outputs", "l2", "arcs", "iterations", "parallelism"}
    assert line["config"]["arcs"] > 0 and line["config"]["iterations"] > 0


def test_reference_arm_loads_only_oracle_libraries():
    """The CPU arm builds its graph with the generators compiled into the
    oracle's library: no library of the product is mapped in that process."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--log2n', '11', "
            "'--steps', '1', '--warmup', '1']\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\n"
            "except SystemExit:\n    pass\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('MAPS', 'libhyperball_gb300' in maps, 'libhb_oracle' in maps)\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert "MAPS False True" in r.stdout


@pytest.mark.parametrize("workload,metric,config_keys", [
    ("visit", "breadth-first visit arcs examined/s",
     {"workload", "nodes", "arcs", "visited", "levels", "arcs_examined"}),
    ("sumsweep", "ExactSumSweep RadiusDiameter runs/s",
     {"workload", "nodes", "arcs", "diameter", "radius", "diameter_iterations"}),
])
def test_reference_arm_of_the_visit_and_sumsweep_workloads(workload, metric, config_keys):
    """The CPU arm of the breadth-first visit and ExactSumSweep workloads: the
    oracle's fair parallel visits on every host thread, the GPU arm's metric
    and config keys, and no library of the product in the process."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--workload', "
            f"'{workload}', '--log2n', '15', '--steps', '1', '--warmup', '1']\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\n"
            "except SystemExit:\n    pass\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('MAPS', 'libhyperball_gb300' in maps, 'libhb_oracle' in maps)\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr
    out = r.stdout.strip().splitlines()
    assert out[-1] == "MAPS False True"
    line = json.loads(out[-2])
    assert line["impl"] == "reference" and line["metric"] == metric and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["cpu_baseline"]["cores"] == (os.cpu_count() or 1)
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert set(line["config"]) == config_keys


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--log2n", "10", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert r.returncode == 0 and r.stdout.strip() == ""


@pytest.mark.gpu
def test_bench_small_gpu():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--log2n", "16",
                        "--steps", "2", "--warmup", "3", "--no-cpu-baseline", "--e2e-steps", "1"],
                       capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["value"] > 0 and line["gpu_launches"] > 0
    assert 0 < line["roofline"]["frac"]
    assert line["e2e"]["h2d_bytes_per_step"] > 0
