"""GPU parity on the reference's own configuration files (tests/golden/reference_frames.npz,
made from input_coords/ and input_files/ by tests/golden/make_frames.py): equilibrated frames
with close O-O contacts and many Thole pairs inside 5 A, where the lattice boxes of the other
tests sample both branches of Q(2/3, x) less densely.

Every case runs the engine through the C ABI and the oracle on the same coordinates.
Tolerances: FP64 engine 1e-10 relative (normwise, max |diff| / max |oracle|) on gradients,
energies and dipoles, 1e-8 on virials, equal induced-dipole iteration counts and bit-exact
neighbour lists; mixed engine force RMS error <= 1e-4 relative (the stated target), energy
within 1e-5 of sum |U_i| and dipoles converged to the 1e-8 threshold."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10
FRAMES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_frames.npz")


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def rms_rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.sqrt(((a - b) ** 2).mean()) / np.sqrt((b ** 2).mean())


def frame(name, P, sigma=0.02, seed=5):
    """Beads = the reference frame plus seeded Gaussian displacements (sigma in A)."""
    d = np.load(FRAMES)
    RRc, box = d[name + "_RRc"], d[name + "_box"]
    rng = np.random.default_rng(seed)
    RRt = RRc[None] + (rng.normal(scale=sigma, size=(P,) + RRc.shape) if P > 1 else 0.0)
    return box, RRt, RRt.mean(axis=0)


def params(model, box, natoms, P, rc, alpha, nmax, **kw):
    p = dict(pot_model=model, natoms=natoms, nbeads=P, box=tuple(box), rc=rc, rc1=0.8 * rc, eps_ewald=1e-6,
             alpha=alpha, nmax=nmax, polar_maxiter=100, polar_sor=0.7, polar_eps=1e-8, guess_initdip=0)
    p.update(kw)
    return p


def usum(r):
    return abs(r["Umon"]) + abs(r["Uvdw"]) + abs(r["Uelec"]) + abs(r["Uind"])


def check_fp64(eng, o, got, RRt, RRc):
    for k in range(RRt.shape[0]):
        r = o.pot_ttm(RRt[k], RRc, bead=k)
        assert rel(got["dRRt"][k], r["dRR"]) < RTOL
        assert abs(got["Upott"][k] - r["En"]) < RTOL * usum(r)
        assert rel(got["dip_momIt"][k], r["dip_momI"]) < RTOL
        assert rel(eng.virial(k), r["virt"]) < 1e-8
        e = eng.energies(k)
        assert e["niter"] == r["niter"]
        assert np.array_equal(eng.neighbors(k), o.neighbors(RRt[k]))


def check_mixed(eng, o, got, RRt, RRc, p, tol=1e-4):
    for k in range(RRt.shape[0]):
        r = o.pot_ttm(RRt[k], RRc, bead=k)
        assert rms_rel(got["dRRt"][k], r["dRR"]) < tol
        assert abs(got["Upott"][k] - r["En"]) < 1e-5 * usum(r)
        assert rms_rel(got["dip_momIt"][k], r["dip_momI"]) < 1e-4
        e = eng.energies(k)
        assert e["niter"] < p["polar_maxiter"] and e["deltadip"] < p["polar_eps"]
        assert np.array_equal(eng.neighbors(k), o.neighbors(RRt[k]))


@pytest.mark.parametrize("precision", [0, 1])
def test_input_512_ttm3f(pkg, orc, engine_lib, precision):
    """input_coords/input_512.xyz (512 H2O, L = 24.832313 A), TTM3-F, Rc 9 A, |n| <= 12,
    2 beads, dipoles converged to 1e-8."""
    box, RRt, RRc = frame("input_512", 2)
    p = params(3, box, RRt.shape[1], 2, 9.0, pkg.waterbox.ewald_alpha_eps(9.0), 12)
    eng = pkg.ForceEngine(p, precision=precision)
    got = eng.full_bead_forces(RRt, RRc, t=1)
    o = orc.Oracle(p)
    if precision == 0:
        check_fp64(eng, o, got, RRt, RRc)
    else:
        assert eng.tuning()["sf_tc"] == 1 and eng.tuning()["ff_tc"] == 1
        check_mixed(eng, o, got, RRt, RRc, p)
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_4nm_cell_list(pkg, orc, engine_lib, precision):
    """input_files/4nm.xyz (2228 H2O, L = 40.5855 A): the cell-list neighbour build (N > 1024)
    on an equilibrated frame, one bead, |n| <= 6."""
    box, RRt, RRc = frame("4nm", 1)
    p = params(3, box, RRt.shape[1], 1, 9.0, 0.39, 6)
    eng = pkg.ForceEngine(p, precision=precision)
    got = eng.full_bead_forces(RRt, RRc, t=1)
    o = orc.Oracle(p)
    if precision == 0:
        check_fp64(eng, o, got, RRt, RRc)
    else:
        check_mixed(eng, o, got, RRt, RRc, p)
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_ttm21f_config_128(pkg, orc, engine_lib, precision):
    """The precision form's system: TTM2.1-F, 128 H2O in the reference's input_128 frame
    (L = 15.658825 A), Rc 7.8 A, |n| <= 9, dipoles to 1e-8, 2 beads."""
    box, RRt, RRc = frame("input_128", 2)
    p = params(2, box, RRt.shape[1], 2, 7.8, pkg.waterbox.ewald_alpha_eps(7.8), 9)
    eng = pkg.ForceEngine(p, precision=precision)
    got = eng.full_bead_forces(RRt, RRc, t=1)
    o = orc.Oracle(p)
    if precision == 0:
        check_fp64(eng, o, got, RRt, RRc)
    else:
        check_mixed(eng, o, got, RRt, RRc, p)
    eng.close()


def test_qspcfw_input_32(pkg, orc, engine_lib):
    """q-SPC/Fw on input_coords/input_32.xyz (L = 9.85467 A, molecules split across the box
    faces), Rc 4.9 A, alpha = 3/Rc, |n| <= 7, 2 beads (pot_spc's /box minimum images)."""
    box, RRt, RRc = frame("input_32", 2)
    p = params(4, box, RRt.shape[1], 2, 4.9, 3.0 / 4.9, 7)
    eng = pkg.ForceEngine(p)
    got = eng.full_bead_forces(RRt, RRc, t=1)
    ref = orc.full_bead_forces(p, RRt, RRc, t=1)
    assert rel(got["dRRt"], ref["dRRt"]) < RTOL
    assert rel(got["Upott"], ref["Upott"]) < RTOL
    assert rel(got["dip_momIt"], ref["dip_momIt"]) < RTOL
    assert rel(got["virialt"], ref["virialt"]) < 1e-8
    eng.close()


@pytest.mark.parametrize("path,nmax", [("fp32_pipe", 24), ("tensor_core", 24), ("tensor_core", 16)])
def test_ewald_large_k_shell(pkg, orc, engine_lib, path, nmax):
    """The mixed engine's Ewald passes at |n| <= 24 (the large-system k range: 28 888 k-vectors
    there, 29 000 here), TTM3-F on the input_128 frame, one bead, Rc 7.8 A with alpha from the
    eps = 1e-6 rule, as the large system uses: forced onto the FP32-pipe structure-factor and
    field kernels (sf_tc = ff_tc = 0), and on the tensor-core kernels, which take |kz| > 20 in
    a second band of run groups and run the field passes in several passes with the weights
    read from global memory. (With a much larger alpha, 0.9 / A, the FP32 reciprocal field's
    rounding floor, ~1.7e-8 D, lies above the 1e-8 threshold and the iterations run to
    polar_maxiter; the forces stay inside the budget.) |n| <= 16 has more runs than two field
    passes hold but no second band."""
    box, RRt, RRc = frame("input_128", 1)
    p = params(3, box, RRt.shape[1], 1, 7.8, pkg.waterbox.ewald_alpha_eps(7.8), nmax)
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    t = eng.tuning()
    if path == "fp32_pipe":
        t = eng.set_tuning(sf_tc=0, ff_tc=0)
        assert t["sf_tc"] == 0 and t["ff_tc"] == 0 and t["qd_tc"] == 0
    else:
        assert t["sf_tc"] == 1 and t["ff_tc"] == 1 and t["qd_tc"] == 1
    got = eng.full_bead_forces(RRt, RRc, t=1)
    o = orc.Oracle(p)
    assert eng.ewald_info()[1] == o.ewald_info()[1]
    check_mixed(eng, o, got, RRt, RRc, p)
    eng.close()
