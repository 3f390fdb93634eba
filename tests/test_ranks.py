"""The multi-GPU bench path (replicas only: every rank builds its own survey,
no data-path collective) on CPU: two gloo ranks agree on the slowest rank's
times, and the whole-job figure divides them by the replica count."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import ROOT  # noqa: F401  (puts the repository root on sys.path)
import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks([1.0 + rank, 10.0 - rank], dist)
    q.put((rank, got, bench.whole_job_seconds_per_build(got[0], world)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, job in out:
        assert got == [2.0, 10.0], rank
        assert job == 1.0


def test_single_rank_values_pass_through():
    assert bench.max_over_ranks([0.25, 3.0]) == [0.25, 3.0]
    assert bench.whole_job_seconds_per_build(0.3, 1) == 0.3
