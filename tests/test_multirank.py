"""The bench's multi-GPU form is replicas only: each rank runs its own
replicate of the workload with its own seed, the job's time is the slowest
rank's, and rank 0 alone prints.  The host side of that, with two `gloo`
ranks on the CPU (no GPU needed)."""
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


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + rank, torch, world, "cpu")
        out.put((rank, bench.replica_seed(rank), ms, bench.job_rate(1000, world, ms)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_max_time_and_distinct_seeds():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res[0][1] != res[1][1]                       # own seeds
    assert res[0][2] == res[1][2] == 11.0               # the slowest rank's time
    assert res[0][3] == res[1][3] == 2000 / 0.011       # every rank's units


def test_reference_arm_under_two_ranks_prints_once():
    """`bench.py --impl reference` under torchrun: rank 0 times the CPU
    port and prints one JSON line, rank 1 exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--cpu-scale", "0.002", "--days", "30"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
