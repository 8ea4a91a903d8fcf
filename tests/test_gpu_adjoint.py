"""GPU tests of the differentiation form (TTM3-F, FP64): the adjoint backward against central
finite differences of the forward's own energies, in positions and in every parameter theta,
and against the analytic forces when the dipoles are converged.

The finite differences use a fixed number of dipole iterations (polar_eps = 0), so the energy
is a smooth function of positions and parameters. Tolerances (normwise, relative to the largest
gradient component): positions 2e-5 (h = 1e-5 A; the A&S erfc and the NR Q(2/3,x) of the
reference make the analytic derivative consistent with the energy only to ~1e-7 relative per
term); parameters 1e-4 relative (h = 1e-4 relative: smaller steps drown in the ~1e-12 rounding
noise of the energy's FP64 atomic sums)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def case(pkg, nw=32, P=2, K=6, eps=0.0, seed=31, nmax=7):
    c = pkg.waterbox.make_config("ttm3f_512x32", nw=nw, P=P, seed=seed)
    L = c["params"]["box"][0]
    rc = min(9.0, L / 2 - 0.01)
    p = dict(c["params"], rc=rc, rc1=0.8 * rc, alpha=3.2 / rc, nmax=nmax, polar_maxiter=K, polar_eps=eps,
             guess_initdip=0)
    return c, p


def energy(eng, RRt, RRc, ebar):
    U = eng.pot_forward(RRt, RRc)
    return float(np.dot(ebar, U))


def test_adjoint_position_gradient_matches_fd(pkg, engine_lib):
    c, p = case(pkg)
    eng = pkg.ForceEngine(p)
    ebar = np.array([1.0, 0.5])
    RRt, RRc = c["RRt"].copy(), c["RRc"]
    energy(eng, RRt, RRc, ebar)
    g, _ = eng.pot_backward(ebar)
    scale = np.abs(g).max()
    h = 1e-5
    rng = np.random.default_rng(2)
    worst = 0.0
    for _ in range(12):
        b, a, k = int(rng.integers(2)), int(rng.integers(p["natoms"])), int(rng.integers(3))
        Rp, Rm = RRt.copy(), RRt.copy()
        Rp[b, a, k] += h
        Rm[b, a, k] -= h
        fd = (energy(eng, Rp, RRc, ebar) - energy(eng, Rm, RRc, ebar)) / (2 * h)
        worst = max(worst, abs(fd - g[b, a, k]) / scale)
    assert worst < 2e-5, worst


def test_adjoint_theta_gradient_matches_fd(pkg, engine_lib):
    c, p = case(pkg, P=1)
    eng = pkg.ForceEngine(p)
    ebar = np.array([1.0])
    RRt, RRc = c["RRt"], c["RRc"]
    energy(eng, RRt, RRc, ebar)
    _, dth = eng.pot_backward(ebar)
    th0 = eng.get_theta()
    names = pkg.engine.THETA_NAMES
    bad = []
    for i, name in enumerate(names):
        h = 1e-4 * max(abs(th0[i]), 1e-3)
        tp, tm = th0.copy(), th0.copy()
        tp[i] += h
        tm[i] -= h
        eng.set_theta(tp)
        ep = energy(eng, RRt, RRc, ebar)
        eng.set_theta(tm)
        em = energy(eng, RRt, RRc, ebar)
        eng.set_theta(th0)
        fd = (ep - em) / (2 * h)
        if abs(fd - dth[i]) > 1e-4 * max(abs(fd), 1e-6 * abs(ep)):
            bad.append((name, fd, dth[i]))
    assert not bad, bad


def test_adjoint_equals_analytic_forces_when_converged(pkg, orc, engine_lib):
    """With converged dipoles (1e-12) and no force-only vdW switch (rc1 = rc) the exact
    derivative of the energy equals the reference's analytic gradient (Hellmann-Feynman) to the
    ~1e-7 consistency of its A&S erfc / NR Q(2/3,x)."""
    c, p = case(pkg, P=2, K=200, eps=1e-12)
    p["rc1"] = p["rc"]
    eng = pkg.ForceEngine(p)
    ebar = np.ones(2)
    eng.pot_forward(c["RRt"], c["RRc"])
    g, _ = eng.pot_backward(ebar)
    ref = orc.full_bead_forces(p, c["RRt"], c["RRc"])["dRRt"]
    assert np.abs(g - ref).max() < 1e-5 * np.abs(ref).max()


def test_backward_requires_forward(pkg, engine_lib):
    c, p = case(pkg, P=1)
    eng = pkg.ForceEngine(p)
    with pytest.raises(pkg.engine.PimdError):
        eng.pot_backward(np.ones(1))


def rms_rel(a, b):
    return float(np.sqrt(((a - b) ** 2).mean() / (b ** 2).mean()))


@pytest.mark.parametrize("eps,nmax", [(0.0, 7), (1e-4, 7), (0.0, 16)])
def test_mixed_backward_matches_fp64(pkg, engine_lib, eps, nmax):
    """The mixed engine's forward + backward (FP32 pair, table and reciprocal products, FP64 sums)
    against the FP64 engine's on the same coordinates and parameters: the position gradient
    within the mixed force budget (1e-4 RMS relative) and every dE/dtheta within 1e-4 of the
    largest. eps = 0 runs a fixed 6 iterations; eps = 1e-4 stops at a loose tolerance, where
    the backward differentiates the truncated iteration (both engines stop at the same count);
    |n| <= 16 takes more field-pass columns. The mixed sweep runs the forward's tensor-core
    structure factor, field pass and dipole-force pass (asserted)."""
    c, p = case(pkg, nw=64, P=2, K=6 if eps == 0.0 else 40, eps=eps, nmax=nmax)
    ebar = np.array([1.0, 0.5])
    res = []
    for prec in (pkg.engine.PIMD_FP64, pkg.engine.PIMD_MIXED):
        eng = pkg.ForceEngine(p, precision=prec)
        if prec == pkg.engine.PIMD_MIXED:  # the sweep's reciprocal passes run on the tensor cores
            t = eng.tuning()
            assert t["sf_tc"] == 1 and t["ff_tc"] == 1 and t["qd_tc"] == 1
        U = eng.pot_forward(c["RRt"], c["RRc"])
        n = [eng.energies(k)["niter"] for k in range(2)]
        g, dth = eng.pot_backward(ebar)
        res.append((U, n, g, dth))
        eng.close()
    (U64, n64, g64, th64), (Um, nm, gm, thm) = res
    assert n64 == nm
    assert np.abs(Um - U64).max() < 1e-5 * np.abs(U64).max()
    assert rms_rel(gm, g64) < 1e-4
    assert np.abs(thm - th64).max() < 1e-4 * np.abs(th64).max()


def test_mixed_backward_fp32_pipe_sweep(pkg, engine_lib):
    """The mixed sweep without the tensor-core passes (sf_tc = ff_tc = 0: the register-tiled
    structure factor and field pass, and the site-parallel reciprocal bilinear kernel) against the
    FP64 backward, same tolerances."""
    c, p = case(pkg, nw=64, P=2, K=6, eps=0.0)
    ebar = np.array([1.0, 0.5])
    eng = pkg.ForceEngine(p)
    eng.pot_forward(c["RRt"], c["RRc"])
    g64, th64 = eng.pot_backward(ebar)
    eng.close()
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    t = eng.set_tuning(sf_tc=0, ff_tc=0)
    assert t["sf_tc"] == 0 and t["ff_tc"] == 0
    eng.pot_forward(c["RRt"], c["RRc"])
    gm, thm = eng.pot_backward(ebar)
    eng.close()
    assert rms_rel(gm, g64) < 1e-4
    assert np.abs(thm - th64).max() < 1e-4 * np.abs(th64).max()


def test_mixed_backward_equals_mixed_forces_when_converged(pkg, engine_lib):
    """At converged dipoles (1e-10) and rc1 = rc the mixed backward's position gradient equals the
    mixed engine's own analytic forces within the mixed budget."""
    c, p = case(pkg, nw=64, P=2, K=100, eps=1e-10)
    p["rc1"] = p["rc"]
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    eng.pot_forward(c["RRt"], c["RRc"])
    g, _ = eng.pot_backward(np.ones(2))
    ref = eng.full_bead_forces(c["RRt"], c["RRc"])["dRRt"]
    assert rms_rel(g, ref) < 1e-4
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_backward_repeats(pkg, engine_lib, precision):
    """Two backward calls after one forward give the same gradients (the sweep leaves the tape and
    the forward's buffers it reads intact)."""
    c, p = case(pkg, nw=64, P=2, K=6, eps=0.0)
    eng = pkg.ForceEngine(p, precision=precision)
    eng.pot_forward(c["RRt"], c["RRc"])
    g1, t1 = eng.pot_backward(np.array([1.0, 0.5]))
    g2, t2 = eng.pot_backward(np.array([1.0, 0.5]))
    eng.close()
    assert np.array_equal(g1, g2) or np.abs(g1 - g2).max() < 1e-12 * np.abs(g1).max()
    assert np.abs(t1 - t2).max() < 1e-12 * np.abs(t1).max()
