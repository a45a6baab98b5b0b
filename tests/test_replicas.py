"""The bench's multi-GPU mode is replicas only: every rank runs its own copy
of the workload and nothing is exchanged on the data path.  On CPU, two
gloo ranks check the one collective of the timing: each rank receives the
slowest rank's time and the whole-job throughput.  The reference arm prints
on rank 0 only; the other ranks exit 0 without work."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        total, value = bench.replica_value(torch, dist, times[rank], 1000, 10, world)
        queue.put((rank, total, value))
    finally:
        dist.destroy_process_group()


def test_replica_value_single_rank():
    import torch
    sys.path.insert(0, str(ROOT))
    import bench
    total, value = bench.replica_value(torch, None, 100.0, 1000, 10, 1)
    assert total == 100.0
    assert value == pytest.approx(1000 * 10 / 0.1 / 1e6)


def test_replica_value_takes_the_slowest_rank():
    import torch.multiprocessing as mp
    world, times = 2, [120.0, 150.0]
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, times, queue)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        got = sorted(queue.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [r for r, _, _ in got] == [0, 1]
    for _, total, value in got:
        assert total == 150.0
        assert value == pytest.approx(1000 * 10 * world / 0.150 / 1e6)
    assert all(p.exitcode == 0 for p in procs)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
