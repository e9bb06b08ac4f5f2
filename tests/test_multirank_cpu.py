"""bench.py under two ranks on CPU (gloo): the max-over-ranks timing and the
reference arm's rank > 0 exit.  No GPU: the replicas themselves are covered by
the single-GPU tests; this checks the multi-process host logic."""
import argparse
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, values, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    got = bench._barrier_max(values[rank], world)
    dist.barrier()
    q.put((rank, got))
    dist.destroy_process_group()


def test_max_over_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    values = [1.25, 3.5]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, values, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 3.5, 1: 3.5}


def test_reference_arm_other_ranks_exit(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(workload="uniform256", proteomes=None, k=6, steps=1, warmup=1,
                              ref_seconds=1.0, gpus=2)
    assert bench.run_reference(args) == 0  # no work, no output on rank 1
