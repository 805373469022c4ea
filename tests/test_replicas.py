"""Replica aggregation over torch.distributed with the gloo backend, world size 2 (CPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from gom_release_gb300.replicas import aggregate, throughput, world as world_env
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert world_env() == (world, rank, rank)
    units = 1000.0 * (rank + 1)
    secs = 2.0 if rank == 0 else 4.0
    total, slowest = aggregate(units, secs)
    out[rank] = (total, slowest, throughput(units, secs))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_throughput():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        total, slowest, thr = out[r]
        assert total == 3000.0 and slowest == 4.0
        assert thr == pytest.approx(750.0)
