"""The multi-process path of bench.py on the CPU: one process per GPU runs its own replica (the march
shards by frames with no data-path collective); the whole-job rate is timed by the slowest rank,
taken with an all-reduce MAX.  Exercised here with two gloo ranks."""
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    slowest = bench.reduce_max(times[rank], dist, "cpu")
    rate = bench.whole_job_rate(world, 1000, slowest)
    q.put((rank, slowest, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [2.0, 2.5]
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [2.5, 2.5]
    assert all(abs(g[2] - 2 * 1000 / 2.5) < 1e-9 for g in got)


def test_reduce_max_single_process():
    sys.path.insert(0, REPO)
    import bench
    assert bench.reduce_max(3.25, None, "cpu") == 3.25
    assert bench.whole_job_rate(1, 500, 2.0) == 250.0


@pytest.mark.parametrize("rank", ["1", "3"])
def test_reference_arm_other_ranks_exit_quietly(rank):
    # Under torchrun only rank 0 times the CPU reference and prints; the other ranks exit 0 at once.
    env = dict(os.environ, RANK=rank, WORLD_SIZE="4", LOCAL_RANK=rank)
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--gpus", "4",
                          "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == ""
