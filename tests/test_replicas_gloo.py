"""The multi-GPU contract of this path is replicas only: every rank runs an
independent evolution, and the job's throughput is all ranks' work over the
slowest rank's time.  That reduction and the reference arm's rank handling are
exercised here on CPU with world_size 2 over gloo (no GPU)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=ws)
    try:
        # each rank timed its own replica: rank r took 1 + r seconds
        value, slowest = bench.replica_throughput(1000, 3, 10, 1.0 + rank, ws)
        out.put((rank, value, slowest))
    finally:
        dist.destroy_process_group()


def test_replica_throughput_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, slowest in got:
        assert slowest == 2.0
        # 2 ranks x 1000 points x 3 RHS x 10 steps over the slowest 2 s
        assert value == pytest.approx(30000.0)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    value, slowest = bench.replica_throughput(500, 3, 4, 0.5, 1)
    assert slowest == 0.5 and value == pytest.approx(12000.0)


def test_reference_arm_rank_handling():
    # rank 1 of 2 exits 0 without work or output; rank 0 times the CPU
    # restatement and prints the reference line
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
    env.update(RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0
