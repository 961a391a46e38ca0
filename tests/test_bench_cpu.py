"""bench.py's host side on CPU: the reference arm (the oracle port on the host
cores) at one and two ranks, and the max-over-ranks reduction its timings use
(gloo process group, world size 2, 127.0.0.1 rendezvous)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def test_reference_arm_one_rank():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--workload", "rho0.5_108k", "--steps", "2", "--warmup", "1"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["config"]["pairs_half"] == 4212000  # 108,000 particles, rho 0.5, search 3.3


def test_reference_arm_large_system_samples_a_sixteenth():
    """The default workload's reference arm: the 8,001,504-particle system,
    each step the gather over its first 500,094 rows."""
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--steps", "2", "--warmup", "0"], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    d = _json_lines(r.stdout)[0]
    assert d["config"]["N"] == 8001504 and d["config"]["rows_per_step"] == 500094
    # the rows' full-list entries / 2: about 75 half pairs per particle at rho 1
    assert 70 * 500094 < d["config"]["pairs_half"] < 80 * 500094
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"]


def test_reference_arm_two_ranks_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--workload", "rho0.5_108k", "--gpus", "2", "--steps", "2",
           "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout  # rank 0 alone reports; rank 1 exits 0 without work
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2


def _dist_worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist("gloo")
    d.barrier()
    q.put((rank, d.max(1.0 + rank), d.sum(1.0 + rank)))
    d.close()


def test_dist_max_and_sum_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_dist_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank sees the slowest rank's time and the job total
    assert got == [(0, 2.0, 3.0), (1, 2.0, 3.0)]


def test_bench_helpers():
    """Host helpers behind the bench line: the roofline figures read from the
    committed ncu summaries, the per-step byte model and the clock merge."""
    sys.path.insert(0, str(ROOT))
    import bench
    for layout, alg in (("aos", 43_200_000), ("soa", 41_472_000)):
        name = f"force_mixed_gather_{layout}_108k_rho0.5.txt"
        traffic = bench.profiled_traffic(name)
        l1 = bench.profiled_metric(
            name, "l1tex__data_pipe_lsu_wavefronts.avg.pct_of_peak_sustained_elapsed")
        assert traffic is not None and 0.8 < traffic / alg < 1.1, (layout, traffic)
        assert l1 is not None and 0 < l1 <= 100
        assert bench.pair_kernel_bytes("gather", layout, 4_212_000, 108_000) == alg
    assert bench.profiled_metric("force_mixed_gather_aos_108k_rho0.5.txt", "no_such_metric") is None
    # one MD step: the force call's gather over 2P entries plus 104 B and the
    # drift's 112 B per particle, plus the rows written by rebuilds
    assert bench.md_step_bytes(10, 2, 0.0) == 4 * 20 + 216 * 2
    assert bench.md_step_bytes(10, 2, 0.5) == 4 * 20 + 216 * 2 + 4 * 20 * 0.5
    merged = bench.merge_clocks([
        {"sm_mhz": 2070, "sm_min_mhz": 2000, "sm_max_mhz": 2070, "reasons": [], "samples": 5},
        {"sm_mhz": 2050, "sm_min_mhz": 1950, "sm_max_mhz": 2070, "reasons": ["sw_power_cap"],
         "samples": 3},
        {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}])
    assert merged["samples"] == 8 and merged["sm_min_mhz"] == 1950
    assert merged["reasons"] == ["sw_power_cap"] and merged["sm_mhz"] == 2060


def test_ncu_summary_extractor():
    """The summary extractor behind profiles/: a long-form metrics capture
    and a launch list, as ncu writes them with --csv."""
    sys.path.insert(0, str(ROOT))
    from lj_gpu_gb300 import ncu_summary as ns
    head = '"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream",' \
           '"Block Size","Grid Size","Device","CC","Section Name","Metric Name","Metric Unit",' \
           '"Metric Value"'
    def row(i, kern, metric, unit, value):
        return f'"{i}","1","python","h","{kern}","1","7","(256, 1, 1)","(10, 1, 1)","0",' \
               f'"10.3","Command line profiler metrics","{metric}","{unit}","{value}"'
    text = "\n".join(["==PROF== Connected", head,
                      row(0, "k_a(int)", "dram__bytes_read.sum", "Mbyte", "1.5"),
                      row(0, "k_a(int)", "dram__bytes_write.sum", "Kbyte", "2"),
                      row(0, "k_a(int)", "gpu__time_duration.sum", "us", "10"),
                      row(1, "k_b(int)", "gpu__time_duration.sum", "ms", "0.03"),
                      row(2, "k_a(int)", "gpu__time_duration.sum", "ns", "10000")])
    s = ns.summarise_raw(text, kernel="k_a")
    assert "traffic_bytes_per_launch: 1502000" in s and "k_b" not in s
    t = ns.summarise_launches(text)
    assert "| `k_a` | 2 | 0.020 | 10.0 | 40.0 % |" in t
    assert "| `k_b` | 1 | 0.030 | 30.0 | 60.0 % |" in t
