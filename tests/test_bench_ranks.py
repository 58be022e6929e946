"""bench.py's multi-rank path on CPU (gloo, world size 2): the whole-job time is
the slowest rank's, the rate counts every rank's units, and the reference arm
runs on rank 0 only.  The GPU legs are replicas: no collective in the timed
region, so the host logic is all there is to test without GPUs."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    t = bench.max_over_ranks(0.25 + 0.5 * rank, dist, "cpu")
    q.put((rank, t, bench.whole_job_rate(100, t, ws)))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in out] == [0, 1]
    for _, t, rate in out:
        assert t == 0.75                  # the slower rank's time on both
        assert rate == 100 * 2 / 0.75     # units of both ranks over it


def test_single_rank_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5, None, "cpu") == 1.5
    assert bench.whole_job_rate(30, 1.5, 1) == 20.0


def test_reference_arm_rank0_only():
    sys.path.insert(0, ROOT)
    import bench

    class A:
        quick = True
        steps = 1
    assert bench.run_reference(A(), 2, 1) is None


def test_committed_traffic_per_workload():
    """The roofline's traffic comes from the committed capture of the
    benchmarked workload's dominant kernel, and is absent for a workload
    without one."""
    sys.path.insert(0, ROOT)
    import bench
    t256 = bench.committed_traffic("euler256")
    t512 = bench.committed_traffic("euler512")
    assert t256 is not None and 4e8 < t256 < 7e8          # one 512^3 F3 launch (algorithmic 624 MB)
    assert t512 is not None and 3e9 < t512 < 5e9          # one 1024^3 F3 launch (algorithmic 4.76 GB)
    assert bench.committed_traffic("tilt64") is None


def test_reference_arm_json_contract():
    """`bench.py --impl reference` on the CPU (the oracle on the host cores, the
    small workload): one JSON line with the contract's keys, the reference's
    own metric and an e2e without host-device copies."""
    import json
    import subprocess
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--quick",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("{")][-1]
    d = json.loads(line)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "iters/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]
