"""GPU parity of the MD step's Nose-Hoover thermostats and estimators against the CPU FP64 oracle:
the global chain-2 thermostat (Nose_Hoover.f90:33-112 on the module variable uk, MD.f90:43-46 and
101-104), the bead chains on the normal modes (main_stuff.f90:145-171, centroid included), and
write_out's per-step estimators (InputOutput.f90:566-571, estimators.f90:30-96) computed on the
device (pimd_md_step_ex / pimd_md_step_ex_device).

Tolerances (FP64 engine, 6 steps): positions 1e-12, momenta 1e-9 relative (normwise), chain
velocities and uk 1e-9, step outputs and estimators 1e-9 relative each (the device's exp may
differ from the host's by an ulp, and the FP64 atomics of the force sums by summation order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DELT, T = 0.25e-3, 300.0


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def setup(pkg, nw=32, P=4, setNMfreq=0.0, precision=0, **kw):
    W = pkg.waterbox
    c = W.make_config("ttm3f_512x32", nw=nw, P=P)
    L = c["params"]["box"][0]
    rc = min(9.0, L / 2 - 0.01)
    p = dict(c["params"], rc=rc, rc1=0.8 * rc, alpha=3.5 / rc, nmax=8, polar_maxiter=60, polar_eps=1e-8,
             guess_initdip=1)
    p.update(kw)
    eng = pkg.ForceEngine(p, precision=precision)
    eng.nm_init(P, W.KB_AMU * T * P / W.HBAR, DELT, setNMfreq)
    eng.langevin_init(DELT / 2, 0, 0.1, P * T)
    return c, p, eng


CASES = {
    # bead thermostat, global chain, centroid chain, Langevin, setNMfreq
    "bead_nh_global_centroid": (2, 1, 1, 0, 0.0),
    "bead_nh_only": (2, 0, 0, 0, 0.0),
    "global_with_pile": (0, 1, 0, 1, 0.0),
    "global_cmd_frequencies": (2, 1, 0, 0, 1500.0),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_thermostatted_steps_match_oracle(pkg, orc, engine_lib, case):
    bead, glob, cen, lang, nmfreq = CASES[case]
    c, p, eng = setup(pkg, setNMfreq=nmfreq)
    P, na = p["nbeads"], p["natoms"]
    tau = 0.05
    eng.set_thermostat(bead_thermostat=bead, global_thermostat=glob, tau=tau, temp=T, centroid_thermostat=cen,
                       tau_centroid=0.02)
    # the initial uk as the reference's initialize_velocities leaves it: the centroid KE
    Pc = c["PPt"].mean(axis=0)
    m = np.where(np.arange(na) % 3 == 0, c["massO"], c["massH"])
    uk0 = 0.5 * float((Pc ** 2 / m[:, None]).sum())
    eng.set_thermostat_state(np.ones(2), uk0)
    mp = eng.md_params(DELT, c["massO"], c["massH"], langevin=lang, seed=7)
    o = orc.Oracle(p)
    st = orc.thermostat_state(P, na, uk0)
    md = dict(delt=DELT, massO=c["massO"], massH=c["massH"], temp=T, langevin=lang, setNMfreq=nmfreq,
              centroid_thermostat=cen, tau_centroid=0.02)
    R1, P1, g1 = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    R2, P2, g2 = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    rng = np.random.default_rng(11)
    for t in range(1, 7):
        x1 = x2 = None
        if lang:
            x1, x2 = rng.standard_normal((na, P, 3)), rng.standard_normal((na, P, 3))
        got = eng.md_step_ex(mp, R1, P1, g1, t, xi1=x1, xi2=x2)
        ref = orc.pimd_vv_step_ex(o, md, R2, P2, g2, st, t=t, xi1=x1, xi2=x2, bead_thermostat=bead if bead else lang,
                                  global_thermostat=glob, tau=tau)
        for k in orc.MD_OUT_NAMES:
            assert abs(got[k] - ref[k]) <= 1e-9 * max(abs(ref[k]), 1e-12), (t, k, got[k], ref[k])
    assert rel(R1, R2) < 1e-12
    assert rel(P1, P2) < 1e-9
    assert rel(got["RRc"], ref["RRc"]) < 1e-12
    s = eng.thermostat_state(beads=bead == 2)
    assert rel(s["vxi_global"], st["vxi_global"]) < 1e-9
    assert abs(s["uk"] - st["uk"]) < 1e-9 * abs(st["uk"])
    if bead == 2:
        assert rel(s["vxi_beads"], st["vxi_beads"]) < 1e-9
    if glob:
        assert got["s_global"] != 1.0
    eng.close()


def test_graph_step_with_chains_equals_eager(pkg, orc, engine_lib):
    """The thermostatted step with device-side estimators as one CUDA graph equals the eager step."""
    import torch

    runs = []
    for graph in (False, True):
        c, p, eng = setup(pkg)
        eng.set_thermostat(bead_thermostat=2, global_thermostat=1, tau=0.05, temp=T, centroid_thermostat=1,
                           tau_centroid=0.02)
        eng.set_thermostat_state(np.ones(2), 12.0)
        eng.set_graph(graph)
        mp = eng.md_params(DELT, c["massO"], c["massH"], langevin=0, seed=7)
        dev = torch.device("cuda", 0)
        R = torch.from_numpy(c["RRt"].copy()).to(dev)
        Pm = torch.from_numpy(c["PPt"].copy()).to(dev)
        G = torch.zeros_like(R)
        Rc = torch.zeros(R.shape[1:], dtype=torch.float64, device=dev)
        out = torch.zeros(12, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        outs = []
        for t in range(1, 6):
            eng.md_step_ex_device(mp, R.data_ptr(), Pm.data_ptr(), G.data_ptr(), Rc.data_ptr(), t, out.data_ptr())
            torch.cuda.synchronize()  # the engine's own stream, not torch's current one
            outs.append(out.cpu().numpy().copy())
        torch.cuda.synchronize()
        runs.append((R.cpu().numpy(), Pm.cpu().numpy(), np.array(outs), eng.thermostat_state(beads=True)))
        if graph:
            assert eng.graph_info()[0] == 1 and eng.graph_info()[1] == 5
        eng.close()
    (Ra, Pa, oa, sa), (Rb, Pb, ob, sb) = runs
    assert rel(Rb, Ra) < 1e-12 and rel(Pb, Pa) < 1e-10
    assert np.abs(ob - oa).max() <= 1e-10 * np.abs(oa).max()
    assert rel(sb["vxi_beads"], sa["vxi_beads"]) < 1e-10 and rel(sb["vxi_global"], sa["vxi_global"]) < 1e-10


def test_mixed_engine_with_chains(pkg, orc, engine_lib):
    """Mixed precision with both chains: within its force error of the FP64 engine after 6 steps
    (positions 1e-8, momenta and chain velocities 1e-5 relative)."""
    res = []
    for prec in (0, 1):
        c, p, eng = setup(pkg, precision=prec)
        eng.set_thermostat(bead_thermostat=2, global_thermostat=1, tau=0.05, temp=T)
        eng.set_thermostat_state(np.ones(2), 12.0)
        mp = eng.md_params(DELT, c["massO"], c["massH"], langevin=0, seed=7)
        R, Pm, g = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
        for t in range(1, 7):
            out = eng.md_step_ex(mp, R, Pm, g, t)
        res.append((R, Pm, out, eng.thermostat_state(beads=True)))
        eng.close()
    (R0, P0, o0, s0), (R1, P1, o1, s1) = res
    assert rel(R1, R0) < 1e-8
    assert rel(P1, P0) < 1e-5
    assert rel(s1["vxi_beads"], s0["vxi_beads"]) < 1e-5
    assert abs(o1["E_virial"] - o0["E_virial"]) < 1e-5 * abs(o0["E_virial"])


def test_thermostat_arguments(pkg, engine_lib):
    c, p, eng = setup(pkg, P=4)
    with pytest.raises(pkg.PimdError):
        eng.set_thermostat(bead_thermostat=1)
    with pytest.raises(pkg.PimdError):
        eng.set_thermostat(global_thermostat=1, tau=0.0)
    eng.set_thermostat(bead_thermostat=2)
    mp = eng.md_params(DELT, c["massO"], c["massH"], langevin=1, seed=7)
    R, Pm, g = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    with pytest.raises(pkg.PimdError):  # Langevin_NM and the bead chains exclude each other
        eng.md_step_ex(mp, R, Pm, g, 1)
    eng.close()
