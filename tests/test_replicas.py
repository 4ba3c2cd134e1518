"""Replica aggregation across two gloo ranks on CPU (the bench's N>1 host logic)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    from qsi_subspace_ed_gb300.replicas import aggregate

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units, ms = aggregate(1000.0 * (rank + 1), 10.0 + 5.0 * rank)
    q.put((rank, units, ms))
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
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
    assert out == [(0, 3000.0, 15.0), (1, 3000.0, 15.0)]


def test_single_process_passthrough():
    from qsi_subspace_ed_gb300.replicas import aggregate

    assert aggregate(5.0, 2.0) == (5.0, 2.0)
