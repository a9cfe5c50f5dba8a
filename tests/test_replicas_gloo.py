"""The N > 1 bench path on CPU: the render path does not shard (each GPU
renders its own frame as an independent replica), so the only cross-rank
step is the timing — every rank agrees on the slowest rank's time and the
whole-job rate counts every rank's paths over it. Checked here with two
gloo ranks; the reference arm under torchrun prints one line from rank 0
and the other rank exits 0 without work."""

import json
import os
import socket
import subprocess
import sys

import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = 1.0 + rank  # rank 1 is the slow replica
        rate, used = bench.replica_throughput(1000, 4, seconds, world, "cpu")
        out[rank] = (rate, used)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replicas_agree_on_the_slowest_rank():
    world = 2
    port = free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    slowest = float(world)
    for rank in range(world):
        rate, used = out[rank]
        assert used == slowest
        assert rate == 1000 * 4 * world / slowest


def test_one_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert not dist.is_initialized()
    assert bench.replica_throughput(10, 3, 2.0, 1, "cpu") == (15.0, 2.0)


def test_reference_arm_under_torchrun_prints_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--size", "64"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
