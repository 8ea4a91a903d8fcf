"""GPU parity of the whole PIMD_VV step (MD.f90:35-110): Langevin_NM, half kicks, EvolveRing,
centroid PBCs and the force call, eager and as one captured CUDA graph, against the CPU FP64
oracle's MD step. Host-supplied normals make the thermostat comparable draw for draw.

Tolerances: FP64 positions 1e-12 and momenta 1e-9 relative (normwise) after 6 steps; graph
versus eager 1e-12 relative (the FP64 atomics of the real-space sums may round differently
from run to run, nothing else differs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def md_setup(pkg, nw=32, P=4, **kw):
    W = pkg.waterbox
    c = W.make_config("ttm3f_512x32", nw=nw, P=P)
    L = c["params"]["box"][0]
    rc = min(9.0, L / 2 - 0.01)
    p = dict(c["params"], rc=rc, rc1=0.8 * rc, alpha=3.5 / rc, nmax=8, polar_maxiter=60, polar_eps=1e-8,
             guess_initdip=1)
    p.update(kw)
    return c, p


def make_engine(pkg, c, p, precision=0, graph=False):
    W = pkg.waterbox
    P = p["nbeads"]
    eng = pkg.ForceEngine(p, precision=precision)
    delt, T = 0.25e-3, 300.0
    eng.nm_init(P, W.KB_AMU * T * P / W.HBAR, delt)
    eng.langevin_init(delt / 2, 0, 0.1, P * T)
    eng.set_graph(graph)
    mp = eng.md_params(delt, c["massO"], c["massH"], langevin=1, seed=99)
    return eng, mp


def test_md_steps_match_oracle(pkg, orc, engine_lib):
    """Six TTM3-F steps (the 4-step dipole predictor engages at t = 5, 6) against the oracle."""
    c, p = md_setup(pkg)
    P, na = p["nbeads"], p["natoms"]
    eng, mp = make_engine(pkg, c, p)
    o = orc.Oracle(p)
    md = dict(delt=0.25e-3, massO=c["massO"], massH=c["massH"], temp=300.0, langevin=1)
    R1, P1, g1 = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    R2, P2, g2 = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    rng = np.random.default_rng(5)
    for t in range(1, 7):
        x1, x2 = rng.standard_normal((na, P, 3)), rng.standard_normal((na, P, 3))
        out, RRc = eng.md_step(mp, R1, P1, g1, t, xi1=x1, xi2=x2)
        r = orc.pimd_vv_step(o, md, R2, P2, g2, x1, x2, t=t)
    assert rel(R1, R2) < 1e-12
    assert rel(P1, P2) < 1e-9
    assert rel(g1, g2) < 1e-9
    assert abs(out[0] - r["Upot"]) < 1e-9 * abs(r["Upot"])
    assert abs(out[3] - r["uk"]) < 1e-9 * abs(r["uk"])
    assert rel(RRc, r["RRc"]) < 1e-12


@pytest.mark.parametrize("precision", [0, 1])
def test_md_steps_64_beads(pkg, orc, engine_lib, precision):
    """Two steps at 64 beads (the integrator kernels' shared memory above 48 KB) against the
    oracle: FP64 to the tolerances above; mixed to its force error (momenta 1e-5, positions
    1e-8 relative: ~1e-5 relative force error moves an H atom by ~1e-8 A per step)."""
    c, p = md_setup(pkg, nw=8, P=64)
    P, na = p["nbeads"], p["natoms"]
    eng, mp = make_engine(pkg, c, p, precision=precision)
    o = orc.Oracle(p)
    md = dict(delt=0.25e-3, massO=c["massO"], massH=c["massH"], temp=300.0, langevin=1)
    R1, P1, g1 = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    R2, P2, g2 = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    rng = np.random.default_rng(64)
    for t in range(1, 3):
        x1, x2 = rng.standard_normal((na, P, 3)), rng.standard_normal((na, P, 3))
        out, RRc = eng.md_step(mp, R1, P1, g1, t, xi1=x1, xi2=x2)
        orc.pimd_vv_step(o, md, R2, P2, g2, x1, x2, t=t)
    tolR, tolP = (1e-12, 1e-9) if precision == 0 else (1e-8, 1e-5)
    assert rel(R1, R2) < tolR
    assert rel(P1, P2) < tolP
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_step_matches_eager(pkg, engine_lib, precision):
    """Eight steps as a replayed CUDA graph (device Langevin draws, predictor, dipole loop as a
    conditional node) equal eight eager steps from the same state; the graph is captured once."""
    c, p = md_setup(pkg, nw=64, P=4)
    res = []
    for graph in (False, True):
        eng, mp = make_engine(pkg, c, p, precision=precision, graph=graph)
        R, Pm, g = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
        niters = []
        for t in range(1, 9):
            out, _ = eng.md_step(mp, R, Pm, g, t)
            niters.append([eng.energies(k)["niter"] for k in range(p["nbeads"])])
        if graph:
            caps, launches = eng.graph_info()
            assert caps == 1 and launches == 8
        res.append((R, Pm, g, out, niters))
        eng.close()
    (Re, Pe, ge_, oe, ne), (Rg, Pg, gg, og, ng) = res
    assert ne == ng  # the conditional loop stops at the host loop's iteration, bead by bead
    assert rel(Rg, Re) < 1e-12
    assert rel(Pg, Pe) < 1e-10
    assert rel(gg, ge_) < 1e-9
    assert abs(og[0] - oe[0]) < 1e-9 * abs(oe[0])


def test_graph_recaptures_on_new_buffers(pkg, engine_lib):
    """A change of device buffers re-captures the graph instead of replaying stale pointers."""
    torch = pytest.importorskip("torch")
    c, p = md_setup(pkg, nw=32, P=2)
    eng, mp = make_engine(pkg, c, p, graph=True)
    dev = torch.device("cuda", 0)
    outs = []
    for trial in range(2):
        R = torch.from_numpy(c["RRt"]).to(dev)
        Pm = torch.from_numpy(c["PPt"]).to(dev)
        g = torch.zeros_like(R)
        Rc = torch.zeros((p["natoms"], 3), dtype=torch.float64, device=dev)
        o4 = torch.zeros(4, dtype=torch.float64, device=dev)
        for t in (1, 2):
            eng.md_step_device(mp, R.data_ptr(), Pm.data_ptr(), g.data_ptr(), Rc.data_ptr(), t, o4.data_ptr())
        torch.cuda.synchronize()
        outs.append(R.cpu().numpy())
    assert eng.graph_info()[0] == 2
    assert rel(outs[0], outs[1]) < 1e-12
