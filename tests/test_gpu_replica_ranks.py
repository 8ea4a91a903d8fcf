"""The multi-GPU form is replicas only: each rank drives its own engine with its own Langevin
stream, and the ranks exchange nothing but the timing reduction. Two spawned processes (a gloo
group for that reduction) each run three MD steps of a small mixed-engine context on this GPU,
as two ranks of `bench.py --gpus 2` would on two GPUs; their kernels never wait on one another.
Each rank's trajectory equals the same replica stepped alone in this process (1e-12 relative: the
FP64 atomics of the force sums may add in another order), and the two ranks' trajectories
differ (distinct seeds)."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DELT, T = 0.25e-3, 300.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(seed):
    import importlib

    pkg = importlib.import_module("pimd-f90_gb300")
    W = pkg.waterbox
    c = W.make_config("ttm3f_512x32", nw=32, P=4)
    L = c["params"]["box"][0]
    rc = min(9.0, L / 2 - 0.01)
    p = dict(c["params"], rc=rc, rc1=0.8 * rc, alpha=3.5 / rc, nmax=8, polar_maxiter=40, polar_eps=1e-8)
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    P = p["nbeads"]
    eng.nm_init(P, W.KB_AMU * T * P / W.HBAR, DELT)
    eng.langevin_init(DELT / 2, 0, 0.1, P * T)
    mp_ = eng.md_params(DELT, c["massO"], c["massH"], langevin=1, seed=seed)
    R, Pm, G = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    for t in range(1, 4):
        eng.md_step(mp_, R, Pm, G, t)
    eng.close()
    return R, Pm


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    R, Pm = _replica(bench.replica_seed(rank))
    t = bench.reduce_max(1.0 + rank, "cpu", world)
    out[rank] = (R, Pm, t)
    dist.barrier()
    dist.destroy_process_group()


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_two_replica_ranks_are_independent(engine_lib):
    import torch.multiprocessing as mp

    import bench

    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
        res = dict(out)
    for r in range(world):
        R, Pm = _replica(bench.replica_seed(r))
        assert rel(res[r][0], R) < 1e-12 and rel(res[r][1], Pm) < 1e-12
        assert res[r][2] == 1.0 + world - 1
    assert rel(res[0][1], res[1][1]) > 1e-6
