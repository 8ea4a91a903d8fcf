"""GPU parity of the q-SPC/Fw and SPC/F force call (pot_spc.f90) through the C ABI against
the CPU FP64 oracle. Tolerance 1e-10 relative (normwise) in FP64; neighbour lists bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def spc_case(pkg, model=4, P=8, nw=None):
    """q-SPC/Fw, 32 molecules, L = 9.865 A, Rc = 4.9 A, alpha = 3/Rc, |n| <= 7, P = 8 beads."""
    c = pkg.waterbox.make_config("qspcfw_32x8", P=P, nw=nw)
    p = dict(c["params"], pot_model=model)
    return c, p


@pytest.mark.parametrize("model", [4, 5])
def test_spc_full_bead_forces(pkg, orc, engine_lib, model):
    c, p = spc_case(pkg, model)
    eng = pkg.ForceEngine(p)
    got = eng.full_bead_forces(c["RRt"], c["RRc"], t=1)
    ref = orc.full_bead_forces(p, c["RRt"], c["RRc"], t=1)
    assert rel(got["dRRt"], ref["dRRt"]) < RTOL
    assert rel(got["Upott"], ref["Upott"]) < RTOL
    assert rel(got["virialt"], ref["virialt"]) < 1e3 * RTOL
    assert rel(got["dip_momIt"], ref["dip_momIt"]) < RTOL
    assert rel(got["chg"], ref["chg"]) < RTOL
    assert np.all(got["virialct"] == 0.0)  # pot_spc does not define virialc
    o = orc.Oracle(p)
    for k in (0, p["nbeads"] - 1):
        r = o.pot_spc(c["RRt"][k])
        e = eng.energies(k)
        scale = abs(r["Umon"]) + abs(r["Uvdw"]) + abs(r["Uelec"])
        for key in ("Umon", "Uvdw", "Uelec"):
            assert abs(e[key] - r[key]) < RTOL * scale, key
        assert e["Uind"] == 0.0
        assert rel(eng.virial(k), r["virt"]) < 1e-8
        assert np.array_equal(eng.neighbors(k), o.neighbors(c["RRt"][k]))


def test_pot_spc_dropin(pkg, orc, engine_lib):
    """The per-bead drop-in with the reference's pot_spc argument list."""
    c, p = spc_case(pkg, 4, P=1)
    eng = pkg.ForceEngine(p)
    got = eng.pot_spc(c["RRt"][0])
    ref = orc.Oracle(p).pot_spc(c["RRt"][0])
    assert abs(got["En"] - ref["En"]) < RTOL * (abs(ref["Umon"]) + abs(ref["Uvdw"]) + abs(ref["Uelec"]))
    assert rel(got["dRR"], ref["dRR"]) < RTOL
    assert rel(got["virt"], ref["virt"]) < 1e-8
    assert rel(got["dip_momI"], ref["dip_momI"]) < RTOL
    assert rel(got["chg"], ref["chg"]) < RTOL


def test_spc_larger_box(pkg, orc, engine_lib):
    """256 molecules (L = 19.72 A) with the 4.9 A cutoff: many neighbour-list rows per bead."""
    c, p = spc_case(pkg, 4, P=2, nw=256)
    eng = pkg.ForceEngine(p)
    got = eng.full_bead_forces(c["RRt"], c["RRc"])
    ref = orc.full_bead_forces(p, c["RRt"], c["RRc"])
    assert rel(got["dRRt"], ref["dRRt"]) < RTOL
    assert rel(got["Upott"], ref["Upott"]) < RTOL


def test_spc_mixed_precision_rejected(pkg, engine_lib):
    c, p = spc_case(pkg, 4, P=1)
    with pytest.raises(pkg.engine.PimdError):
        pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)


def test_spc_md_steps_match_oracle(pkg, orc, engine_lib):
    """Five PIMD_VV steps of q-SPC/Fw 32 x 8 (PILE thermostat with host-supplied normals) on the
    device against the oracle's MD step."""
    c, p = spc_case(pkg, 4)
    W = pkg.waterbox
    P, na = p["nbeads"], p["natoms"]
    eng = pkg.ForceEngine(p)
    delt, T = 0.25e-3, 300.0
    omegan = W.KB_AMU * T * P / W.HBAR
    eng.nm_init(P, omegan, delt)
    eng.langevin_init(delt / 2, 0, 0.1, P * T)
    mp = eng.md_params(delt, c["massO"], c["massH"], langevin=1)
    o = orc.Oracle(p)
    md = dict(delt=delt, massO=c["massO"], massH=c["massH"], temp=T, langevin=1)
    R1, P1 = c["RRt"].copy(), c["PPt"].copy()
    R2, P2 = c["RRt"].copy(), c["PPt"].copy()
    g1, g2 = np.zeros_like(R1), np.zeros_like(R2)
    rng = np.random.default_rng(11)
    for t in range(1, 6):
        x1, x2 = rng.standard_normal((na, P, 3)), rng.standard_normal((na, P, 3))
        out, _ = eng.md_step(mp, R1, P1, g1, t, xi1=x1, xi2=x2)
        r = orc.pimd_vv_step(o, md, R2, P2, g2, x1, x2, t=t)
    assert rel(R1, R2) < 1e-12
    assert rel(P1, P2) < 1e-9
    assert abs(out[0] - r["Upot"]) < 1e-9 * abs(r["Upot"])
