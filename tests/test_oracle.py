"""Known-answer and self-consistency tests that pin the CPU oracle (no GPU needed).

The reference ships no tests or golden outputs and cannot be compiled here (Fortran), so
the oracle is pinned by physics: the Partridge-Schwenke monomer minimum, forces as the
gradient of the energy, the virial as the strain derivative, Ewald alpha-independence,
translational/rotational invariance, orthogonality of the normal-mode matrix and exactness
of the free ring-polymer propagation.
"""
import math

import numpy as np
import pytest


def small_box(pkg, nw=64, seed=99, P=2):
    W = pkg.waterbox
    L = (nw * 29.96) ** (1 / 3)
    RRc = W.centroid_box(nw, L, 0.9572, 104.52, seed)
    RRt, PPt = W.ring_polymer(RRc, P, 300.0, 15.9994, 1.008, seed)
    return L, RRt, PPt, RRt.mean(axis=0)


def ttm_params(nw, L, model=3, **kw):
    rc = L / 2 - 0.01
    p = dict(pot_model=model, natoms=3 * nw, box=(L, L, L), rc=rc, rc1=rc, alpha=3.6 / rc, nmax=12,
             polar_eps=1e-14, polar_maxiter=400)
    p.update(kw)
    return p


def monomer(r1, r2, th):
    return np.array([[0, 0, 0], [r1 * math.sin(th / 2), 0, r1 * math.cos(th / 2)],
                     [-r2 * math.sin(th / 2), 0, r2 * math.cos(th / 2)]])


def test_nasa_pes_minimum(orc):
    """nasa_mod.f90 Partridge-Schwenke PES: minimum at r_e = 0.9578 A, theta_e = 104.51 deg with
    energy ~0 after the reference's +0.44739574026257 cm-1 shift (nasa.f90:89)."""
    from scipy.optimize import minimize

    o = orc.Oracle(dict(pot_model=3, natoms=3, box=(40, 40, 40), rc=9, rc1=9, alpha=0.3, nmax=2, polar_maxiter=3))
    f = lambda x: o.pot_ttm(monomer(*x), monomer(*x))["Umon"]  # noqa: E731
    res = minimize(f, [0.9586, 0.9586, math.radians(104.35)], method="Nelder-Mead",
                   options=dict(xatol=1e-10, fatol=1e-15, maxiter=4000))
    r1, r2, th = res.x
    assert abs(r1 - 0.95784) < 2e-4 and abs(r2 - 0.95784) < 2e-4
    assert abs(math.degrees(th) - 104.508) < 0.02
    assert abs(res.fun) < 1e-3  # kcal/mol


def test_dms_dipole_at_equilibrium(orc):
    """The Partridge-Schwenke dipole-moment surface gives ~1.85 D at equilibrium (TTM2.1-F
    uses it unmodified: dms_param1..3 = 0)."""
    o = orc.Oracle(dict(pot_model=2, natoms=3, box=(60, 60, 60), rc=9, rc1=9, alpha=0.25, nmax=2, polar_maxiter=1))
    R = monomer(0.95784, 0.95784, math.radians(104.508))
    r = o.pot_ttm(R, R)
    q = r["chg"]  # e * CHARGECON, atoms O H H
    mu = (q[:, None] * R).sum(0) / 18.22234397655801 * 4.8033324 / 1.0  # e*A -> Debye
    assert abs(np.linalg.norm(mu) - 1.855) < 0.01


@pytest.mark.parametrize("model", [3, 4])
def test_forces_are_energy_gradient(pkg, orc, model):
    """dRR equals the central finite difference of En (TTM3-F with rc1 = Rc so the
    force-only vdW switch is off; q-SPC/Fw). Tolerance covers the A&S erfc/Thole Q(2/3,x)
    approximations (relative 1e-7..1e-6)."""
    nw = 64
    L, RRt, _, RRc = small_box(pkg, nw)
    if model == 3:
        p = ttm_params(nw, L)
    else:
        RRc = pkg.waterbox.centroid_box(nw, L, 1.0, 112.0, 5)
        RRt = RRc[None]
        p = dict(pot_model=4, natoms=3 * nw, box=(L, L, L), rc=L / 2 - 0.01, alpha=3.6 / (L / 2), nmax=12)
    o = orc.Oracle(p)
    RR = RRt[0].copy()
    r0 = o.potential(RR, RRc)
    h = 1e-5
    worst = 0.0
    for a in [0, 1, 2, 5, 40, 77, 100, 150]:
        for d in range(3):
            Rp, Rm = RR.copy(), RR.copy()
            Rp[a, d] += h
            Rm[a, d] -= h
            fd = (o.potential(Rp, RRc)["En"] - o.potential(Rm, RRc)["En"]) / (2 * h)
            worst = max(worst, abs(fd - r0["dRR"][a, d]))
    assert worst < 2e-5 * np.abs(r0["dRR"]).max()


def test_virial_is_strain_derivative(pkg, orc):
    """trace(virt) = dE/dlambda for a uniform scaling of coordinates, box, cutoff and 1/alpha;
    the long-range correction enters the virial at fixed cutoff (pot_ttm.f90:588-591), so the
    scaled-cutoff derivative exceeds it by -3 Uvdw_lrc."""
    nw = 64
    L, RRt, _, RRc = small_box(pkg, nw)
    p = ttm_params(nw, L)
    RR = RRt[0]
    r0 = orc.Oracle(p).pot_ttm(RR, RRc)

    def scaled(lam):
        q = dict(p)
        q.update(box=tuple(lam * np.array(p["box"])), alpha=p["alpha"] / lam, rc=p["rc"] * lam, rc1=p["rc"] * lam)
        return orc.Oracle(q).pot_ttm(RR * lam, RRc * lam)["En"]

    h = 1e-5
    fd = (scaled(1 + h) - scaled(1 - h)) / (2 * h)
    rc = p["rc"]
    ulrc = 2 * math.pi * nw * nw / L ** 3 * (-0.72298855e03 / (3 * rc ** 3))
    assert abs(fd - (np.trace(r0["virt"]) - 3 * ulrc)) < 5e-4 * abs(fd)


def test_ewald_alpha_independence(pkg, orc):
    """A converged Ewald sum does not depend on the splitting parameter."""
    nw = 64
    L, RRt, _, RRc = small_box(pkg, nw)
    p = ttm_params(nw, L)
    e1 = orc.Oracle(p).pot_ttm(RRt[0], RRc)["En"]
    q = dict(p, alpha=3.9 / p["rc"], nmax=14)
    e2 = orc.Oracle(q).pot_ttm(RRt[0], RRc)["En"]
    assert abs(e1 - e2) < 1e-4 * abs(e1)


def test_invariances(pkg, orc):
    """Sum of the gradient vanishes; the energy is invariant under a rigid rotation of an
    isolated cluster and under a translation by a lattice vector."""
    nw = 32
    L, RRt, _, RRc = small_box(pkg, nw, P=1)
    p = ttm_params(nw, L, polar_eps=1e-12)
    o = orc.Oracle(p)
    r = o.pot_ttm(RRt[0], RRc)
    assert np.abs(r["dRR"].sum(0)).max() < 1e-6 * np.abs(r["dRR"]).max()
    shifted = RRt[0] + np.array([L, -L, 2 * L])
    r2 = o.pot_ttm(shifted, RRc + np.array([L, -L, 2 * L]))
    assert abs(r2["En"] - r["En"]) < 1e-9 * abs(r["En"])
    # rotation: three molecules far apart inside a big box
    X = np.concatenate([monomer(0.96, 0.95, 1.8) + np.array(o_) for o_ in ([0, 0, 0], [2.9, 0.1, 0.2], [0.3, 2.8, -0.4])])
    big = dict(pot_model=3, natoms=9, box=(60, 60, 60), rc=20, rc1=20, alpha=0.18, nmax=10, polar_eps=1e-13,
               polar_maxiter=300)
    ob = orc.Oracle(big)
    th = 0.7
    Rz = np.array([[math.cos(th), -math.sin(th), 0], [math.sin(th), math.cos(th), 0], [0, 0, 1]])
    e0 = ob.pot_ttm(X, X)["En"]
    e1 = ob.pot_ttm(X @ Rz.T, X @ Rz.T)["En"]
    assert abs(e1 - e0) < 5e-5 * max(1.0, abs(e0))


def test_neighbour_cutoff_edge_cases(orc):
    """find_neigh uses a strict R^2 < Rc^2 under the anint minimum image."""
    L = 20.0
    X = np.concatenate([monomer(0.96, 0.96, 1.82) + np.array([x, 0, 0]) for x in (0.0, 9.0, -9.0 + L / 2)])
    p = dict(pot_model=3, natoms=9, box=(L, L, L), rc=9.0, rc1=8.0, alpha=0.35, nmax=6, polar_maxiter=30)
    r = orc.Oracle(p).pot_ttm(X, X)
    assert np.isfinite(r["En"])


def test_normal_mode_matrix_orthogonal(orc):
    for P in (1, 2, 7, 8, 32):
        nm = orc.nm_init(P, omegan=1234.0, delta=2.5e-4)
        C = nm["C"]
        assert np.abs(C @ C.T - np.eye(P)).max() < 1e-13


def test_free_ring_propagation_is_exact(orc):
    """EvolveRing rotates each normal mode in phase space: the free ring-polymer energy
    sum p^2/2m + m wn^2/2 sum |x_j - x_{j+1}|^2 is conserved to round-off."""
    P, m, T = 16, 1.008, 300.0
    omegan = 0.831447148 * T * P / 6.35077993041
    nm = orc.nm_init(P, omegan, 2.5e-4)
    rng = np.random.default_rng(1)
    RR, PP = rng.normal(size=(P, 3)) * 0.1, rng.normal(size=(P, 3)) * 3.0

    def energy(R, Q):
        spring = 0.5 * m * omegan ** 2 * ((R - np.roll(R, -1, axis=0)) ** 2).sum()
        return (Q ** 2).sum() / (2 * m) + spring

    e0 = energy(RR, PP)
    for _ in range(200):
        RR, PP = orc.evolve_ring(nm, RR, PP, m)
    assert abs(energy(RR, PP) - e0) < 1e-10 * e0


def test_langevin_coefficients(orc):
    """Init_Langevin_NM: c1 = exp(-dt/2 * 2 w_k), c2 = sqrt(1-c1^2) sqrt(kB T_P)."""
    P = 8
    nm = orc.nm_init(P, 800.0, 2.5e-4)
    c1, c2 = orc.langevin_init(nm, 1.25e-4, 0, 0.1, 300.0 * P)
    assert c1[0] == 1.0 and c2[0] == 0.0
    j = 3
    e = math.exp(-1.25e-4 * 2 * nm["omegalist"][j])
    assert abs(c1[j] - e) < 1e-15
    assert abs(c2[j] - math.sqrt(1 - e * e) * math.sqrt(0.831447148 * 300.0 * P)) < 1e-12


def test_full_bead_forces_threads_match_serial(pkg, orc):
    """The threaded bead loop (the CPU baseline) equals per-bead serial calls."""
    c = pkg.waterbox.make_config("ttm3f_512x32", nw=32, P=3)
    p = dict(c["params"], rc=4.9, rc1=3.9, alpha=0.7, nmax=6, polar_maxiter=12)
    r = orc.full_bead_forces(p, c["RRt"], c["RRc"], nthreads=3)
    o = orc.Oracle(p)
    for k in range(3):
        s = o.pot_ttm(c["RRt"][k], c["RRc"], bead=k)
        assert s["En"] == r["Upott"][k]
        assert np.array_equal(s["dRR"], r["dRRt"][k])


def test_nose_hoover_half_step_is_time_reversible(orc):
    """Nose_Hoover.f90:33-112 is a symmetric Trotter splitting: the half step with -delt2 undoes
    the half step with +delt2 (chain velocities and uk back to their start), and s = e^(-vxi1 dt/2)."""
    vxi = np.array([0.37, -0.21])
    s, uk = orc.nose_hoover(250.0, vxi, 0.04, 1.25e-4, 960, 9600.0)
    assert 0 < s < 2 and abs(uk - 250.0 * s * s) < 1e-12 * uk
    s2, uk2 = orc.nose_hoover(uk, vxi, 0.04, -1.25e-4, 960, 9600.0)
    assert np.allclose(vxi, [0.37, -0.21], rtol=0, atol=1e-14)
    assert abs(uk2 - 250.0) < 1e-11 and abs(s * s2 - 1.0) < 1e-14


def test_ring_k0_and_simple_estimator_on_free_rings(orc):
    """K0 (estimators.f90:57-73) equals its normal-mode form sum m (omega_k / omega_n)^2 x_k^2, and on
    free ring polymers drawn from the free-ring distribution at T (NormalModes.f90:224-250) the
    simple (primitive) energy estimator averages 4.5 kb T per molecule, the classical kinetic
    energy of three atoms."""
    P, nat, T = 8, 30, 300.0
    mO, mH = 15.9994, 1.008
    omegan = 0.831447148 * T * P / 6.35077993041
    nm = orc.nm_init(P, omegan, 2.5e-4)
    C, om = nm["C"], nm["omegalist"]
    m = np.where(np.arange(nat) % 3 == 0, mO, mH)
    rng = np.random.default_rng(17)
    kbT = 0.0019872041 * T
    uk = T * nat * P * P / 0.80181484527  # sys_temp = T exactly
    Es = []
    for it in range(2000):
        x = np.zeros((P, nat, 3))
        for k in range(1, P):
            x[k] = rng.standard_normal((nat, 3)) * np.sqrt(omegan * 6.35077993041 / (m[:, None] * om[k] ** 2))
        R = np.einsum("kj,kac->jac", C, x)  # NM2real: r_j = sum_k C(k, j) x_k
        K0 = orc.ring_k0(mO, mH, R)
        if it == 0:
            k0nm = sum((m[:, None] * (om[k] / omegan) ** 2 * x[k] ** 2).sum() for k in range(P))
            assert abs(K0 - k0nm) < 1e-10 * K0
        e = orc.estimators(nat, P, 1000.0, omegan, 0.0, 0.0, 0.0, uk, K0)
        assert abs(e["sys_temp"] - T) < 1e-9
        Es.append(e["E_simple"])
    assert abs(np.mean(Es) / (4.5 * kbT) - 1.0) < 0.03


def test_four1_is_the_discrete_fourier_transform(orc):
    """four1.f: isign = -1 is the DFT exp(-2 pi i jk/n), isign = +1 the unnormalised inverse
    (checked against numpy.fft in single precision)."""
    rng = np.random.default_rng(9)
    for n in (8, 64, 1024):
        z = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
        assert np.abs(orc.four1(z, -1) - np.fft.fft(z)).max() < 2e-5 * np.sqrt(n) * np.abs(z).max()
        assert np.abs(orc.four1(z, 1) - np.fft.ifft(z) * n).max() < 2e-5 * np.sqrt(n) * np.abs(z).max()


def test_msd_of_a_uniform_drift(orc):
    """calc_diff_RMSD / write_out_diffusion on a uniform drift v per frame: aMS(k) = |v|^2 (20 (k-1))^2
    (the first sample is taken at the first frame), so the fitted slope is that of the samples."""
    nat, box = 12, np.array([30.0, 30.0, 30.0])
    m = orc.MSD(nat, 200, box)
    R = np.random.default_rng(3).uniform(-5, 5, size=(nat, 3))
    v = np.array([0.01, -0.02, 0.005])
    for k in range(200):
        m.step(R + k * v)
    r = m.report(0.25e-3)
    k = np.arange(len(r["aMS"]))
    assert np.allclose(r["aMS"], (v ** 2).sum() * (20.0 * k) ** 2, rtol=1e-9, atol=1e-15)
