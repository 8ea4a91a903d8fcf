"""GPU parity: the CUDA engine, called through the C ABI, against the CPU FP64 oracle on the
same seeded inputs. Tolerance for FP64 mode: 1e-10 relative (normwise: max |diff| over the
array divided by max |oracle value|); neighbour lists bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def small_case(pkg, model=3, nw=32, P=3, seed=None, **kw):
    W = pkg.waterbox
    name = "ttm3f_512x32" if model == 3 else "ttm21f_128x32"
    c = W.make_config(name, nw=nw, P=P, seed=seed)
    L = c["params"]["box"][0]
    rc = min(9.0, L / 2 - 0.01)
    p = dict(c["params"], rc=rc, rc1=0.8 * rc, alpha=3.5 / rc, nmax=8, polar_maxiter=30, polar_eps=0.0)
    p.update(kw)
    return c, p


def compare_beads(got, ref, tol=RTOL):
    assert rel(got["dRRt"], ref["dRRt"]) < tol
    assert rel(got["Upott"], ref["Upott"]) < tol
    assert rel(got["dip_momIt"], ref["dip_momIt"]) < tol
    assert rel(got["dip_momEt"], ref["dip_momEt"]) < tol
    assert rel(got["virialct"], ref["virialct"]) < 1e3 * tol
    assert rel(got["virialt"], ref["virialt"]) < 1e3 * tol
    assert rel(got["chg"], ref["chg"]) < tol


@pytest.mark.parametrize("model", [3, 2])
def test_full_bead_forces_small(pkg, orc, engine_lib, model):
    c, p = small_case(pkg, model)
    eng = pkg.ForceEngine(p)
    got = eng.full_bead_forces(c["RRt"], c["RRc"], t=1)
    ref = orc.full_bead_forces(p, c["RRt"], c["RRc"], t=1)
    compare_beads(got, ref)
    o = orc.Oracle(p)
    for k in range(p["nbeads"]):
        r = o.pot_ttm(c["RRt"][k], c["RRc"], bead=k)
        e = eng.energies(k)
        for key in ("Umon", "Uvdw", "Uelec", "Uind"):
            assert abs(e[key] - r[key]) < RTOL * (abs(r["Umon"]) + abs(r["Uvdw"]) + abs(r["Uelec"]) + abs(r["Uind"]))
        assert rel(eng.virial(k), r["virt"]) < 1e-8
        assert e["niter"] == p["polar_maxiter"]


def test_neighbour_list_bit_exact(pkg, orc, engine_lib):
    c, p = small_case(pkg, 3, nw=128, P=2)
    eng = pkg.ForceEngine(p)
    eng.full_bead_forces(c["RRt"], c["RRc"])
    o = orc.Oracle(p)
    for k in range(2):
        assert np.array_equal(eng.neighbors(k), o.neighbors(c["RRt"][k]))


def test_dipole_convergence_same_iterations(pkg, orc, engine_lib):
    """With a convergence threshold the engine stops at the same iteration as the oracle."""
    c, p = small_case(pkg, 3, nw=64, P=2, polar_eps=1e-8, polar_maxiter=100)
    eng = pkg.ForceEngine(p)
    got = eng.full_bead_forces(c["RRt"], c["RRc"])
    o = orc.Oracle(p)
    for k in range(2):
        r = o.pot_ttm(c["RRt"][k], c["RRc"], bead=k)
        assert eng.energies(k)["niter"] == r["niter"]
        assert rel(got["dRRt"][k], r["dRR"]) < RTOL


def test_pot_ttm_dropin(pkg, orc, engine_lib):
    """The per-bead drop-in with the reference's pot_ttm argument list."""
    c, p = small_case(pkg, 3, nw=32, P=1)
    eng = pkg.ForceEngine(p)
    got = eng.pot_ttm(c["RRt"][0], c["RRc"], t=1)
    ref = orc.Oracle(p).pot_ttm(c["RRt"][0], c["RRc"])
    assert abs(got["En"] - ref["En"]) < RTOL * (abs(ref["Umon"]) + abs(ref["Uvdw"]) + abs(ref["Uelec"]) + abs(ref["Uind"]))
    assert rel(got["dRR"], ref["dRR"]) < RTOL
    assert rel(got["virt"], ref["virt"]) < 1e-8
    assert abs(got["virialc"] - ref["virialc"]) < 1e-8 * np.abs(ref["virt"]).max()
    assert rel(got["dip_momI"], ref["dip_momI"]) < RTOL
    assert rel(got["chg"], ref["chg"]) < RTOL


def test_predictor_history_per_bead(pkg, orc, engine_lib):
    """guess_initdip: the 4-step predictor from each bead's own history (steps 1..6)."""
    c, p = small_case(pkg, 3, nw=32, P=2, guess_initdip=1, polar_maxiter=6)
    eng = pkg.ForceEngine(p)
    o = orc.Oracle(p)
    rng = np.random.default_rng(3)
    for t in range(1, 7):
        RRt = c["RRt"] + rng.normal(scale=0.002, size=c["RRt"].shape)
        got = eng.full_bead_forces(RRt, c["RRc"], t=t)
        for k in range(2):
            r = o.pot_ttm(RRt[k], c["RRc"], t=t, bead=k)
            assert rel(got["dRRt"][k], r["dRR"]) < RTOL


def test_headline_size_two_beads(pkg, orc, engine_lib):
    """TTM3-F 512 H2O, L = 24.86 A, Rc = 9 A, |n| <= 12: beads 0 and 31 of 32."""
    c = pkg.waterbox.make_config("ttm3f_512x32")
    p = dict(c["params"], polar_maxiter=12, polar_eps=0.0)
    eng = pkg.ForceEngine(p)
    assert eng.ewald_info()[1] == orc.Oracle(p).ewald_info()[1]
    got = eng.full_bead_forces(c["RRt"], c["RRc"])
    o = orc.Oracle(p)
    for k in (0, 31):
        r = o.pot_ttm(c["RRt"][k], c["RRc"], bead=k)
        assert rel(got["dRRt"][k], r["dRR"]) < RTOL
        assert abs(got["Upott"][k] - r["En"]) < RTOL * (abs(r["Umon"]) + abs(r["Uvdw"]) + abs(r["Uelec"]) + abs(r["Uind"]))


def test_normal_modes_bit_exact(pkg, orc, engine_lib):
    """InitNormalModes arrays and EvolveRing are bit-identical to the oracle."""
    c, p = small_case(pkg, 3, nw=8, P=8)
    eng = pkg.ForceEngine(p)
    for P in (8, 5, 64):  # 64 beads: the kernels take more than 48 KB of shared memory
        a = eng.nm_init(P, 1500.0, 2.5e-4)
        b = orc.nm_init(P, 1500.0, 2.5e-4)
        for key in ("A11", "A12", "A21", "A22", "omegalist", "msf", "C"):
            assert np.array_equal(a[key], b[key]), key
        rng = np.random.default_rng(P)
        RR, PP = rng.normal(size=(P, 3)), rng.normal(size=(P, 3))
        g = eng.evolve_ring(RR, PP, 1.008)
        r = orc.evolve_ring(b, RR, PP, 1.008)
        assert np.array_equal(g[0], r[0]) and np.array_equal(g[1], r[1])


# ---------------------------------------------------------------------------------------
# Mixed precision (FP32 pair/phase arithmetic, FP64 accumulation): error budget against the
# FP64 oracle. Force RMS error must stay below 1e-4 relative (the stated target); energy,
# dipoles and virial are held to the tolerances written below.
def rms_rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.sqrt(((a - b) ** 2).mean()) / np.sqrt((b ** 2).mean())


@pytest.mark.parametrize("model", [3, 2])
def test_mixed_error_budget_small(pkg, orc, engine_lib, model):
    c, p = small_case(pkg, model, nw=64, P=3, polar_maxiter=40)
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    got = eng.full_bead_forces(c["RRt"], c["RRc"], t=1)
    ref = orc.full_bead_forces(p, c["RRt"], c["RRc"], t=1)
    assert rms_rel(got["dRRt"], ref["dRRt"]) < 1e-5
    assert rel(got["dRRt"], ref["dRRt"]) < 1e-4
    o = orc.Oracle(p)
    for k in range(p["nbeads"]):
        r = o.pot_ttm(c["RRt"][k], c["RRc"], bead=k)
        scale = abs(r["Umon"]) + abs(r["Uvdw"]) + abs(r["Uelec"]) + abs(r["Uind"])
        assert abs(got["Upott"][k] - r["En"]) < 1e-6 * scale
    assert rms_rel(got["dip_momEt"], ref["dip_momEt"]) < 1e-5
    assert np.abs(got["virialt"] - ref["virialt"]).max() < 1e-5 * np.abs(ref["virialt"]).max() + 1e-3
    assert np.array_equal(eng.neighbors(0), o.neighbors(c["RRt"][0]))


@pytest.mark.parametrize("model", [3, 2])
def test_tensor_core_structure_factor_active(pkg, orc, engine_lib, model):
    """The mixed engine's dipole structure factor runs on the tcgen05 kernel (a silent fallback
    to the FP32-pipe kernel fails here) and stays inside the mixed error budget."""
    c, p = small_case(pkg, model, nw=64, P=4, polar_maxiter=40)
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    got = eng.full_bead_forces(c["RRt"], c["RRc"], t=1)
    tun = eng.tuning()
    assert tun["sf_tc"] == 1 and tun["ff_tc"] == 1 and tun["qd_tc"] == 1
    ref = orc.full_bead_forces(p, c["RRt"], c["RRc"], t=1)
    assert rms_rel(got["dRRt"], ref["dRRt"]) < 1e-5
    assert rms_rel(got["dip_momIt"], ref["dip_momIt"]) < 1e-5
    assert np.abs(got["virialt"] - ref["virialt"]).max() < 1e-5 * np.abs(ref["virialt"]).max() + 1e-3
    assert tun["x_cache"] == 1
    # building X in every iteration (no cache) is the same arithmetic: equal up to the FP64
    # atomic order of the block sums
    eng.set_tuning(x_cache=0)
    nocache = eng.full_bead_forces(c["RRt"], c["RRc"], t=1)
    assert eng.tuning()["x_cache"] == 0
    assert rms_rel(nocache["dRRt"], got["dRRt"]) < 1e-9
    # the field passes (dipole, charge, force) on the FP32 pipe instead agree within the budget
    eng.set_tuning(ff_tc=0)
    alt = eng.full_bead_forces(c["RRt"], c["RRc"], t=1)
    assert eng.tuning()["qd_tc"] == 0
    assert rms_rel(alt["dRRt"], got["dRRt"]) < 1e-5
    eng.close()


def test_mixed_headline_and_convergence(pkg, orc, engine_lib):
    """TTM3-F 512 H2O x 32 beads: force RMS error <= 1e-4 relative, and the induced dipoles
    converge to the 1e-8 threshold (deterministic FP32 field, FP64 residual)."""
    c = pkg.waterbox.make_config("ttm3f_512x32")
    p = dict(c["params"], polar_maxiter=100, polar_eps=1e-8)
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    got = eng.full_bead_forces(c["RRt"], c["RRc"])
    o = orc.Oracle(p)
    for k in (0, 17):
        r = o.pot_ttm(c["RRt"][k], c["RRc"], bead=k)
        assert rms_rel(got["dRRt"][k], r["dRR"]) < 1e-4
        e = eng.energies(k)
        assert e["niter"] < p["polar_maxiter"] and e["deltadip"] < p["polar_eps"]
        assert abs(e["niter"] - r["niter"]) <= 2


@pytest.mark.parametrize("precision", [0, 1])
def test_cell_list_neighbours_large_box(pkg, orc, engine_lib, precision):
    """1800 molecules (L = 37.8 A, 4 cells of >= 9 A per edge): the cell-list build gives the
    reference's list bit for bit, and the forces follow (FP64 1e-10; mixed 1e-4 relative)."""
    c = pkg.waterbox.make_config("ttm3f_512x32", nw=1800, P=1)
    p = dict(c["params"], rc=9.0, rc1=7.2, alpha=0.39, nmax=6, polar_maxiter=8, polar_eps=0.0)
    eng = pkg.ForceEngine(p, precision=precision)
    got = eng.full_bead_forces(c["RRt"], c["RRc"])
    o = orc.Oracle(p)
    assert np.array_equal(eng.neighbors(0), o.neighbors(c["RRt"][0]))
    r = o.pot_ttm(c["RRt"][0], c["RRc"])
    tol = RTOL if precision == 0 else 1e-4
    assert rel(got["dRRt"][0], r["dRR"]) < tol


@pytest.mark.parametrize("nmol", [1, 2])
def test_one_and_two_molecules(pkg, orc, engine_lib, nmol):
    """The smallest systems (FP64): one molecule (no intermolecular pair: the monomer PES, its
    intramolecular terms and its own periodic images through the Ewald sums) and two, cut from a
    32-molecule box (L = 9.86 A, Rc 4.92 A), 2 beads, against the oracle."""
    c, p = small_case(pkg, 3, nw=32, P=2)
    RRt = np.ascontiguousarray(c["RRt"][:, :3 * nmol, :])
    RRc = np.ascontiguousarray(c["RRc"][:3 * nmol])
    p = dict(p, natoms=3 * nmol)
    eng = pkg.ForceEngine(p)
    got = eng.full_bead_forces(RRt, RRc, t=1)
    ref = orc.full_bead_forces(p, RRt, RRc, t=1)
    compare_beads(got, ref)
    if nmol == 2:
        assert np.array_equal(eng.neighbors(0), orc.Oracle(p).neighbors(RRt[0]))
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_neighbour_overflow_reported(pkg, engine_lib, precision):
    """100 molecules packed at liquid density into one corner of a 40 A box: far more pairs than
    the list capacity sized from the box's mean density (1024 here). The call reports the
    overflow (the lists keep their first entries; every kernel stays within the stored length),
    and the next call on spread-out molecules runs normally."""
    c = pkg.waterbox.make_config("ttm3f_512x32", nw=100, P=1, seed=3)
    L0, L = c["params"]["box"][0], 40.0
    p = dict(c["params"], box=(L, L, L), rc=9.0, rc1=7.2, alpha=0.39, nmax=6, polar_maxiter=6,
             polar_eps=0.0)
    eng = pkg.ForceEngine(p, precision=precision)
    with pytest.raises(pkg.engine.PimdError, match="neighbour list capacity"):
        eng.full_bead_forces(c["RRt"], c["RRc"])
    # the same molecules with their O sites spread over the whole box
    R = c["RRt"].copy()
    O = R[:, 0::3, :].copy()
    for a in range(3):
        R[:, a::3, :] += (L / L0 - 1.0) * O
    got = eng.full_bead_forces(R, R.mean(axis=0))
    assert np.isfinite(got["dRRt"]).all() and np.isfinite(got["Upott"]).all()
    eng.close()


@pytest.mark.parametrize("nw,precision", [(1024, 0), (1024, 1), (1100, 0), (1100, 1)])
def test_neighbour_path_edges(pkg, orc, engine_lib, nw, precision):
    """The edges of the neighbour-list paths: 1024 molecules, the most the one-cluster build
    takes (hit masks of 128 KB in a CTA), and 1100 (L = 32.0 A: three cells of >= 9 A per edge,
    too few for the cell lists), which takes the count / scan / fill build. Lists bit for bit equal
    to the reference's, forces FP64 1e-10, mixed 1e-4 relative."""
    c = pkg.waterbox.make_config("ttm3f_512x32", nw=nw, P=1, seed=7 + nw)
    L = c["params"]["box"][0]
    p = dict(c["params"], rc=9.0, rc1=7.2, alpha=0.39, nmax=6, polar_maxiter=8, polar_eps=0.0)
    if nw > 1024:
        assert L / 9.001 < 4  # fewer than four cells per edge: not the cell-list build
    eng = pkg.ForceEngine(p, precision=precision)
    got = eng.full_bead_forces(c["RRt"], c["RRc"])
    o = orc.Oracle(p)
    assert np.array_equal(eng.neighbors(0), o.neighbors(c["RRt"][0]))
    r = o.pot_ttm(c["RRt"][0], c["RRc"])
    tol = RTOL if precision == 0 else 1e-4
    assert rel(got["dRRt"][0], r["dRR"]) < tol
    eng.close()


@pytest.mark.parametrize("setNMfreq", [0.0, 1500.0])
def test_normal_mode_helpers_bit_exact(pkg, orc, engine_lib, setNMfreq):
    """real2NM / NM2real and gen_rand_ring / gen_rand_ring_momenta (NormalModes.f90:224-341)
    through the C ABI, with the normal draws supplied: bit-identical to the oracle; with the
    context's own draws: the mode deviations of the free-ring distribution."""
    c, p = small_case(pkg, 3, nw=8, P=8)
    eng = pkg.ForceEngine(p)
    W = pkg.waterbox
    for P in (8, 5):
        omegan = W.KB_AMU * 300.0 * P / W.HBAR
        eng.nm_init(P, omegan, 2.5e-4, setNMfreq)
        nm = orc.nm_init(P, omegan, 2.5e-4, setNMfreq)
        rng = np.random.default_rng(P)
        A = rng.normal(size=(P, 3))
        assert np.array_equal(eng.real2nm(A), orc.real2nm(nm, A))
        assert np.array_equal(eng.nm2real(A), orc.nm2real(nm, A))
        xi = rng.standard_normal((P, 3))
        for m in (15.9994, 1.008):
            assert np.array_equal(eng.gen_rand_ring(m, 300.0, P, xi), orc.gen_rand_ring(nm, m, 300.0, xi))
            assert np.array_equal(eng.gen_rand_ring_momenta(m, 300.0 * P, P, xi),
                                  orc.gen_rand_ring_momenta(nm, m, 300.0 * P, xi))
        # the context's generator: normal-mode deviations sqrt(kB T P / (m msf omega_k^2)) and
        # sqrt(kB m msf T P) within 10 % over 4000 rings
        m = 1.008
        R = np.array([eng.real2nm(eng.gen_rand_ring(m, 300.0, P)) for _ in range(4000)])
        Pm = np.array([eng.real2nm(eng.gen_rand_ring_momenta(m, 300.0 * P, P)) for _ in range(4000)])
        sdr = np.sqrt(W.KB_AMU * 300.0 * P / (m * nm["msf"][1:] * nm["omegalist"][1:] ** 2))
        assert np.allclose(R[:, 1:].std(axis=(0, 2)), sdr, rtol=0.1)
        assert np.abs(R[:, 0]).max() < 1e-12
        assert np.allclose(Pm.std(axis=(0, 2)), np.sqrt(W.KB_AMU * m * nm["msf"] * 300.0 * P), rtol=0.1)
    eng.close()


def test_invalid_input_rejected(pkg, engine_lib):
    """Invalid input is refused with PIMD_ERR_ARG before any device work: a cutoff beyond half the
    box (the reference's check, InputOutput.f90:277-281), an atom count that is not a multiple of
    three, no beads, an unknown model or precision; and a knob out of range."""
    c, p = small_case(pkg, 3, nw=32, P=2)
    L = p["box"][0]
    bad = [dict(rc=0.5 * L + 0.1), dict(natoms=p["natoms"] - 1), dict(nbeads=0), dict(pot_model=7)]
    for d in bad:
        with pytest.raises(pkg.engine.PimdError):
            pkg.ForceEngine(dict(p, **d))
    with pytest.raises(pkg.engine.PimdError):
        pkg.ForceEngine(p, precision=5)
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    with pytest.raises(pkg.engine.PimdError):
        eng.set_tuning(loop_unroll=0)
    got = eng.full_bead_forces(c["RRt"], c["RRc"])  # still usable
    assert np.isfinite(got["dRRt"]).all()
    eng.close()
