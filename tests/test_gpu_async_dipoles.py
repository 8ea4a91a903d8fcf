"""The mixed engine's asynchronous real-space dipole field (tuning knob dd_async, TTM3-F): the
tensor-core field pass and the real-space gather of a dipole iteration run side by side, and
whichever finishes a unit of 128 dipole sites last runs its SOR update. It changes no arithmetic:
the same FP32 fields enter the same FP64 update, so the dipoles, iteration counts and forces
equal the synchronous order's (1e-9 relative: FP64 atomics of the force sums and of the
convergence sums add in another order). Cases: unit boundaries that split a block of four
molecules (202 H2O), a unit base below the first M site (100 H2O), odd and even iteration
counts (polar_eps 0, so every bead runs to polar_maxiter), perturbed beads, the eager host loop
and the CUDA-graph step, and agreement with the oracle. Also:
the field pass started on a programmatic event of the real-space field (tuning knob dd_jpev)
equals the full join."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DELT, T = 0.25e-3, 300.0


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def case(pkg, nw, P, **kw):
    c = pkg.waterbox.make_config("ttm3f_512x32", nw=nw, P=P)
    L = c["params"]["box"][0]
    rc = min(9.0, L / 2 - 0.01)
    p = dict(c["params"], rc=rc, rc1=0.8 * rc, alpha=3.5 / rc, nmax=8, polar_maxiter=40, polar_eps=1e-8)
    p.update(kw)
    return c, p


def forces(pkg, c, p, async_on):
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    assert eng.set_tuning(dd_async=async_on)["dd_async"] == async_on
    r = eng.full_bead_forces(c["RRt"], c["RRc"], t=0)
    niter = [eng.energies(b)["niter"] for b in range(p["nbeads"])]
    eng.close()
    return r, niter


@pytest.mark.parametrize("nw,P,extra", [(128, 4, {}), (202, 2, {}), (100, 3, {}),
                                        (128, 2, dict(polar_eps=0.0, polar_maxiter=7)),
                                        (128, 2, dict(polar_eps=0.0, polar_maxiter=8))])
def test_async_equals_synchronous(pkg, engine_lib, nw, P, extra):
    c, p = case(pkg, nw, P, **extra)
    a, na = forces(pkg, c, p, 1)
    s, ns = forces(pkg, c, p, 0)
    assert na == ns
    if "polar_maxiter" in extra:
        assert na == [extra["polar_maxiter"]] * P
    for k in ("dRRt", "Upott", "dip_momIt", "dip_momEt", "virialt"):
        assert rel(a[k], s[k]) < 1e-9, k


def test_async_beads_converge_apart_and_match_oracle(pkg, orc, engine_lib):
    """Beads perturbed apart (their last FP32 dipoles sit in either buffer when they converge at
    iterations of different parity; the fixed counts of the odd and even polar_maxiter cases
    above cover both parities); the result stays within the mixed engine's budget of the oracle
    and equals the synchronous order."""
    c, p = case(pkg, 128, 4)
    R = c["RRt"].copy()
    R[1] += np.random.default_rng(5).normal(scale=0.08, size=R[1].shape)
    R[3] += np.random.default_rng(6).normal(scale=0.15, size=R[3].shape)
    Rc = R.mean(axis=0)
    out = []
    for v in (1, 0):
        eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
        eng.set_tuning(dd_async=v)
        r = eng.full_bead_forces(R, Rc, t=0)
        out.append((r, [eng.energies(b)["niter"] for b in range(4)]))
        eng.close()
    (a, na), (s, ns) = out
    assert na == ns
    assert rel(a["dRRt"], s["dRRt"]) < 1e-9
    ref = orc.full_bead_forces(p, R, Rc, t=0)
    g, gr = a["dRRt"], ref["dRRt"]
    assert np.sqrt(((g - gr) ** 2).mean()) / np.sqrt((gr ** 2).mean()) < 1e-5


def test_async_graph_steps_equal_synchronous(pkg, engine_lib):
    import torch

    runs = []
    for v in (1, 0):
        c, p = case(pkg, 128, 4)
        P, na = p["nbeads"], p["natoms"]
        W = pkg.waterbox
        eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
        eng.set_tuning(dd_async=v)
        eng.nm_init(P, W.KB_AMU * T * P / W.HBAR, DELT)
        eng.langevin_init(DELT / 2, 0, 0.1, P * T)
        eng.set_graph(True)
        mp = eng.md_params(DELT, c["massO"], c["massH"], langevin=1, seed=3)
        dev = torch.device("cuda", 0)
        R = torch.from_numpy(c["RRt"].copy()).to(dev)
        Pm = torch.from_numpy(c["PPt"].copy()).to(dev)
        G = torch.zeros_like(R)
        Rc = torch.zeros((na, 3), dtype=torch.float64, device=dev)
        out = torch.zeros(4, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        for t in range(1, 6):
            eng.md_step_device(mp, R.data_ptr(), Pm.data_ptr(), G.data_ptr(), Rc.data_ptr(), t, out.data_ptr())
        torch.cuda.synchronize()
        assert eng.tuning()["dd_async"] == v
        runs.append((R.cpu().numpy(), G.cpu().numpy(), out.cpu().numpy(), eng.energies(0)["niter"]))
        eng.close()
    (Ra, Ga, oa, na), (Rs, Gs, os_, ns) = runs
    assert na == ns
    assert rel(Ra, Rs) < 1e-12 and rel(Ga, Gs) < 1e-8
    assert np.abs(oa - os_).max() <= 1e-8 * np.abs(os_).max()


@pytest.mark.parametrize("graph", [False, True])
def test_programmatic_join_equals_full_join(pkg, engine_lib, graph):
    """The field pass launched on a programmatic event of the real-space field (dd_jpev: it may
    start as that grid drains and waits for it in griddepcontrol.wait before reading its field)
    gives the same steps as the full join."""
    import torch

    runs = []
    for v in (1, 0):
        c, p = case(pkg, 128, 4)
        P, na = p["nbeads"], p["natoms"]
        W = pkg.waterbox
        eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
        assert eng.set_tuning(dd_jpev=v)["dd_jpev"] == v
        eng.nm_init(P, W.KB_AMU * T * P / W.HBAR, DELT)
        eng.langevin_init(DELT / 2, 0, 0.1, P * T)
        eng.set_graph(graph)
        mp = eng.md_params(DELT, c["massO"], c["massH"], langevin=1, seed=3)
        dev = torch.device("cuda", 0)
        R = torch.from_numpy(c["RRt"].copy()).to(dev)
        Pm = torch.from_numpy(c["PPt"].copy()).to(dev)
        G = torch.zeros_like(R)
        Rc = torch.zeros((na, 3), dtype=torch.float64, device=dev)
        out = torch.zeros(4, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        for t in range(1, 6):
            eng.md_step_device(mp, R.data_ptr(), Pm.data_ptr(), G.data_ptr(), Rc.data_ptr(), t, out.data_ptr())
        torch.cuda.synchronize()
        runs.append((R.cpu().numpy(), G.cpu().numpy(), out.cpu().numpy(), eng.energies(0)["niter"]))
        eng.close()
    (Ra, Ga, oa, na_), (Rs, Gs, os_, ns) = runs
    assert na_ == ns
    assert rel(Ra, Rs) < 1e-12 and rel(Ga, Gs) < 1e-8
    assert np.abs(oa - os_).max() <= 1e-8 * np.abs(os_).max()
