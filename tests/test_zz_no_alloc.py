"""The allocation-free neighbour-list entry point (pimd_neighbors_noalloc).

It exists for callers that must not let the library allocate device memory (drivers owning all
GPU memory through their own pool, fixed per-GPU budgets, CUDA-graph recording). This file is
collected last so that a failure here stops a -x run only after every other test has run.
Two calls in a row on different beads are checked pair for pair against the engine's own
neighbour list (pimd_get_neighbors, which the allocating context provides): integer output,
so the comparison is exact.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_neighbors_match_engine(pkg, engine_lib):
    import torch

    L = pkg.engine.load()
    c = pkg.waterbox.make_config("ttm3f_512x32", nw=256, P=2)
    p = dict(c["params"], polar_maxiter=2, polar_eps=0.0)
    eng = pkg.ForceEngine(p)
    eng.full_bead_forces(c["RRt"], c["RRc"])
    box = (ctypes.c_double * 3)(*p["box"])
    cap = 64 * 256
    dev = torch.device("cuda", 0)
    ij = torch.full((cap, 2), -1, dtype=torch.int32, device=dev)
    n = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for bead in (0, 1):  # two calls in a row, different inputs, shared scratch
        RR = torch.from_numpy(np.ascontiguousarray(c["RRt"][bead])).to(dev)
        rc = L.pimd_neighbors_noalloc(RR.data_ptr(), p["natoms"], box, p["rc"], ij.data_ptr(), cap, n.data_ptr(),
                                      stream.cuda_stream)
        assert rc == 0
        torch.cuda.synchronize(dev)
        ref = eng.neighbors(bead)
        assert int(n.item()) == len(ref)
        assert np.array_equal(ij[: len(ref)].cpu().numpy(), ref)
    # a capacity below the pair count: the first cap pairs are written, nothing past them, and
    # *npairs still reports the full total
    small = len(ref) // 3
    ij.fill_(-7)
    torch.cuda.synchronize(dev)
    free0 = torch.cuda.mem_get_info(dev)[0]
    rc = L.pimd_neighbors_noalloc(RR.data_ptr(), p["natoms"], box, p["rc"], ij.data_ptr(), small, n.data_ptr(),
                                  stream.cuda_stream)
    assert rc == 0
    torch.cuda.synchronize(dev)
    assert int(n.item()) == len(ref)
    got = ij.cpu().numpy()
    assert np.array_equal(got[:small], ref[:small])
    assert (got[small:] == -7).all()
    # a warmed-up call takes no device memory (the free amount is unchanged)
    assert torch.cuda.mem_get_info(dev)[0] == free0
    eng.close()


def test_noalloc_rejects_oversize(pkg, engine_lib):
    L = pkg.engine.load()
    box = (ctypes.c_double * 3)(100.0, 100.0, 100.0)
    # 16385 molecules exceed the static scratch; rejected before any device access
    rc = L.pimd_neighbors_noalloc(1, 3 * 16385, box, 9.0, 1, 10, 1, None)
    assert rc == 1


def test_noalloc_rejects_bad_box(pkg, engine_lib):
    L = pkg.engine.load()
    for bad in ((0.0, 10.0, 10.0), (10.0, float("nan"), 10.0), (10.0, 10.0, float("inf")), (-5.0, 10.0, 10.0)):
        box = (ctypes.c_double * 3)(*bad)
        # rejected on the host before any device access
        assert L.pimd_neighbors_noalloc(1, 9, box, 3.0, 1, 10, 1, None) == 1
