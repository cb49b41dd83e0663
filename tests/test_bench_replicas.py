"""The N > 1 path of bench.py on CPU: two gloo ranks, each an independent replica; the job's
time is the slowest rank's, its value the points of all replicas over that time, and only
rank 0 runs the reference arm."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r times 1 + r ms for the headline and 5 - r ms for a second arm
        got = bench.reduce_max(dist, [1.0 + rank, 5.0 - rank])
        out.put((rank, got, bench.whole_job(1000, world, got[0]), bench.is_rank0()))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, value, r0 in res:
        assert got == [2.0, 5.0]
        assert value == pytest.approx(2 * 1000 / 2e-3)
        assert r0 == (rank == 0)


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")

    class Args:
        steps, warmup, gpus = 1, 3, 2
    assert bench.run_reference(Args()) == 0   # returns at once: no oracle run on rank 1
    assert bench.reduce_max(None, [3, 4.5]) == [3.0, 4.5]
