"""The multi-GPU path is replicas only: each rank runs an independent engine, the job's time is
the slowest rank's. These CPU tests run the host-side logic of bench.py on world_size-2 gloo
process groups (no GPU)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    out[rank] = (bench.reduce_max(1.5 + rank, "cpu", world), bench.replica_seed(rank))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replica_ranks_reduce_max_and_own_seeds(world):
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
        res = dict(out)
    assert all(res[r][0] == 1.5 + world - 1 for r in range(world))
    seeds = [res[r][1] for r in range(world)]
    assert len(set(seeds)) == world


def test_single_rank_reduce_is_identity():
    import bench

    assert bench.reduce_max(3.25, "cpu", 1) == 3.25
