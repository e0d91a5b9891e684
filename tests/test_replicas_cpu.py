"""Replicas on N > 1 GPUs (one independent pipe per rank, no collective on the data path): the
bench's aggregation takes the slowest rank's time and counts every rank's frames. Checked with
two gloo ranks on the CPU, and the reference arm's ranks other than 0 exit without work."""

import os
import socket
import subprocess
import sys
from pathlib import Path

import torch
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench

    ms, value = bench.replica_throughput([12.5, 20.0][rank], 640, world, device="cpu")
    out.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for _, ms, value in res:
        assert ms == 20.0  # the slowest rank
        assert abs(value - 2 * 640 / 20e-3) < 1e-6  # all ranks' frames over the slowest time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replica_throughput(8.0, 64, 1, device="cpu") == (8.0, 64 / 8e-3)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
