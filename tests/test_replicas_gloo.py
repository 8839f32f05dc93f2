"""The replicas-only multi-GPU rule of bench.py on two CPU ranks (gloo): every
rank times its own replica, the job is timed by the slowest rank, and all ranks
report the same whole-job rate world * DOF * stages / max time."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seconds = 1.0 + rank  # rank 1 is the slower replica
    t = bench.max_over_ranks(seconds, world, device="cpu")
    q.put((rank, t, bench.replica_rate(world, 1000, 5, t)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_timed_by_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.0, 2.0]
    assert [o[2] for o in out] == [2 * 1000 * 5 / 2.0] * 2


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_rate(1, 100, 5, 2.0) == 250.0
