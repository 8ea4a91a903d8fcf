"""GPU parity of ring-polymer contraction with multiple time steps (contracted_MD, MD.f90:276-449)
and monomer PIMD (monomer_PIMD, MD.f90:117-265) through the C ABI, against the CPU FP64 oracle's
restatement of the same steps: the NASA monomer PES on every bead, the intermolecular potential
on the centroid only (one-bead context with contraction set for contracted_MD), the inner MTS
steps with the normal modes made for delt / intra_timesteps, the thermostats and estimators.

Tolerances (FP64 engine, 4 steps): positions 1e-12, momenta and gradients 1e-9 relative
(normwise), step outputs and estimators 1e-9 relative each, monomer dipoles 1e-10."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DELT, T = 0.25e-3, 300.0


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def run(pkg, orc, mode, intra, P=4, langevin=1, chains=False, steps=4, nw=32):
    W = pkg.waterbox
    c = W.make_config("ttm3f_512x32", nw=nw, P=P)
    L = c["params"]["box"][0]
    rc = min(9.0, L / 2 - 0.01)
    p = dict(c["params"], rc=rc, rc1=0.8 * rc, alpha=3.5 / rc, nmax=8, polar_maxiter=60, polar_eps=1e-8,
             guess_initdip=1)
    eng = pkg.ForceEngine(p)
    eng.nm_init(P, W.KB_AMU * T * P / W.HBAR, DELT / intra if mode == 0 else DELT)
    eng.langevin_init(DELT / 2, 0, 0.1, P * T)
    eng.contracted_init(mode, intra)
    bead = 0
    if chains:
        bead = 2
        eng.set_thermostat(bead_thermostat=2, global_thermostat=1, tau=0.05, temp=T, centroid_thermostat=1,
                           tau_centroid=0.02)
        eng.set_thermostat_state(np.ones(2), 14.0)
    mp = eng.md_params(DELT, c["massO"], c["massH"], langevin=langevin, seed=5)
    oc = orc.Oracle(dict(p, nbeads=1, contraction=1 if mode == 0 else 0))
    st = orc.thermostat_state(P, p["natoms"], 14.0)
    md = dict(delt=DELT, massO=c["massO"], massH=c["massH"], temp=T, langevin=langevin, centroid_thermostat=1 if chains else 0,
              tau_centroid=0.02)
    na = p["natoms"]
    R1, P1, g1, f1 = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"]), np.zeros_like(c["RRt"])
    R2, P2, g2, f2 = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"]), np.zeros_like(c["RRt"])
    rng = np.random.default_rng(3)
    for t in range(1, steps + 1):
        x1 = x2 = None
        if langevin:
            x1, x2 = rng.standard_normal((na, P, 3)), rng.standard_normal((na, P, 3))
        got = eng.contracted_step(mp, R1, P1, g1, f1 if mode == 0 else None, t, xi1=x1, xi2=x2, dipoles=True)
        ref = orc.contracted_step(oc, md, mode, intra, R2, P2, g2, f2, st, t=t, xi1=x1, xi2=x2,
                                  bead_thermostat=bead if chains else langevin, global_thermostat=1 if chains else 0,
                                  tau=0.05, dipoles=True)
        for k in orc.MD_OUT_NAMES:
            assert abs(got[k] - ref[k]) <= 1e-9 * max(abs(ref[k]), 1e-12), (t, k, got[k], ref[k])
    assert rel(R1, R2) < 1e-12
    assert rel(P1, P2) < 1e-9
    assert rel(g1, g2) < 1e-9
    if mode == 0:
        assert rel(f1, f2) < 1e-9
    assert rel(got["RRc"], ref["RRc"]) < 1e-12
    assert rel(got["dip_momIt"], ref["dip_momIt"]) < 1e-10
    assert rel(got["dip_momEt"], ref["dip_momEt"]) < 1e-10
    # every bead feels the same slow gradient (contracted) or it plus its own monomer gradient
    if mode == 0:
        assert np.array_equal(g1[0], g1[-1])
    eng.close()


@pytest.mark.parametrize("intra", [1, 5])
def test_contracted_mts_matches_oracle(pkg, orc, engine_lib, intra):
    run(pkg, orc, 0, intra)


def test_monomer_pimd_matches_oracle(pkg, orc, engine_lib):
    run(pkg, orc, 1, 1)


def test_contracted_with_chains_matches_oracle(pkg, orc, engine_lib):
    run(pkg, orc, 0, 3, langevin=0, chains=True, steps=3)


def test_contracted_one_bead(pkg, orc, engine_lib):
    """P = 1: the inner steps are free flights (MD.f90:334-340)."""
    run(pkg, orc, 0, 4, P=1, langevin=0, steps=3)
