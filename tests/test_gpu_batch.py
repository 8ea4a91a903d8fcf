"""GPU tests of the replica batch (independent ring polymers of uneven sizes in one CUDA graph
per step) and of the launch-shape autotuner, through the C ABI.

Batch: each replica's trajectory must equal the same replica stepped alone in its own context
(same seed, temperature, cutoff min(9 A, L/2), Ewald by the eps = 1e-6 rule). FP64 engine;
tolerance 1e-9 relative after 6 steps (the FP64 atomics of the real-space sums may round
differently when beads of several replicas share a launch). Autotuner: results before and
after tuning agree to the mixed engine's FP32 summation-order level (1e-6 relative)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DELT, SEED = 0.25e-3, 777


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def common_params(**kw):
    p = dict(pot_model=3, rc=9.0, rc1=7.2, alpha=0.0, eps_ewald=1e-6, polar_maxiter=60, polar_eps=1e-8,
             polar_sor=0.7, guess_initdip=1)
    p.update(kw)
    return p


def replica_state(pkg, nw, P, T, seed):
    c = pkg.waterbox.make_config("ttm3f_512x32", nw=nw, P=P, T=T, seed=seed)
    return c


def test_batch_matches_single_contexts(pkg, engine_lib):
    W = pkg.waterbox
    specs = [(32, 4, 300.0), (32, 2, 250.0), (64, 4, 350.0)]
    reps, states = [], []
    for i, (nw, P, T) in enumerate(specs):
        c = replica_state(pkg, nw, P, T, 100 + i)
        L = c["params"]["box"][0]
        reps.append(dict(natoms=3 * nw, nbeads=P, box=(L, L, L), temp=T))
        states.append(c)
    common = common_params()
    bt = pkg.engine.ReplicaBatch(common, reps, DELT, 15.9994, 1.008, langevin=1, seed=SEED)
    ng, gof = bt.groups()
    assert ng == 2 and gof == [0, 0, 1]
    for i, c in enumerate(states):
        bt.set_state(i, c["RRt"], c["PPt"])
    bt.forces()
    bt.step(6)
    bt.sync()
    for i, (c, r) in enumerate(zip(states, reps)):
        P, T, L = r["nbeads"], r["temp"], r["box"][0]
        rc = min(9.0, L / 2)
        p = dict(common, natoms=r["natoms"], nbeads=P, box=r["box"], rc=rc, rc1=rc * 0.8)
        eng = pkg.ForceEngine(p)
        eng.nm_init(P, W.KB_AMU * T * P / W.HBAR, DELT)
        eng.langevin_init(DELT / 2, 0, 0.1, P * T)
        mp = eng.md_params(DELT, 15.9994, 1.008, langevin=1, seed=SEED + i)
        R, Pm = c["RRt"].copy(), c["PPt"].copy()
        g = eng.full_bead_forces(R, R.mean(axis=0), t=0)["dRRt"]
        for t in range(1, 7):
            out, _ = eng.md_step(mp, R, Pm, g, t)
        Rb, Pb, Gb, ob = bt.get_state(i)
        assert rel(Rb, R) < 1e-9, i
        assert rel(Pb, Pm) < 1e-9, i
        assert rel(Gb, g) < 1e-8, i
        assert abs(ob[0] - out[0]) < 1e-8 * abs(out[0]), i
        eng.close()
    bt.close()


def rms_rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.sqrt(((a - b) ** 2).mean()) / np.sqrt((b ** 2).mean())


def test_batch_uneven_mixed_matches_single_contexts(pkg, engine_lib):
    """Mixed-precision batch with four box sizes and three bead counts, autotuned, 6 steps: each
    replica against the same replica stepped alone in its own mixed-precision context (same
    seed, temperature and cutoff). The two differ only by FP32 summation order (the batch's
    tuned launch shapes, beads of several replicas per launch): gradient RMS error <= 1e-5
    relative, positions and momenta 1e-6, energy 1e-6."""
    W = pkg.waterbox
    specs = [(32, 8, 260.0), (64, 16, 300.0), (128, 32, 340.0), (256, 8, 280.0), (64, 8, 320.0)]
    reps, states = [], []
    for i, (nw, P, T) in enumerate(specs):
        c = replica_state(pkg, nw, P, T, 200 + i)
        L = c["params"]["box"][0]
        reps.append(dict(natoms=3 * nw, nbeads=P, box=(L, L, L), temp=T))
        states.append(c)
    common = common_params()
    bt = pkg.engine.ReplicaBatch(common, reps, DELT, 15.9994, 1.008, seed=SEED, precision=pkg.engine.PIMD_MIXED)
    ng, gof = bt.groups()
    assert ng == 4 and gof[1] == gof[4]
    for i, c in enumerate(states):
        bt.set_state(i, c["RRt"], c["PPt"])
    bt.autotune()
    bt.forces()
    bt.step(6)
    bt.sync()
    for i, (c, r) in enumerate(zip(states, reps)):
        P, T, L = r["nbeads"], r["temp"], r["box"][0]
        rc = min(9.0, L / 2)
        p = dict(common, natoms=r["natoms"], nbeads=P, box=r["box"], rc=rc, rc1=rc * 0.8)
        eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
        eng.nm_init(P, W.KB_AMU * T * P / W.HBAR, DELT)
        eng.langevin_init(DELT / 2, 0, 0.1, P * T)
        mp = eng.md_params(DELT, 15.9994, 1.008, langevin=1, seed=SEED + i)
        R, Pm = c["RRt"].copy(), c["PPt"].copy()
        g = eng.full_bead_forces(R, R.mean(axis=0), t=0)["dRRt"]
        for t in range(1, 7):
            out, _ = eng.md_step(mp, R, Pm, g, t)
        Rb, Pb, Gb, ob = bt.get_state(i)
        assert np.isfinite(Rb).all() and np.isfinite(Gb).all() and np.isfinite(ob).all()
        assert rms_rel(Gb, g) < 1e-5, i
        assert rel(Rb, R) < 1e-6, i
        assert rel(Pb, Pm) < 1e-6, i
        assert abs(ob[0] - out[0]) < 1e-6 * abs(out[0]), i
        eng.close()
    bt.close()


def test_autotune_keeps_results(pkg, engine_lib):
    c = pkg.waterbox.make_config("ttm3f_512x32", nw=128, P=4)
    rc = min(9.0, c["params"]["box"][0] / 2)
    p = dict(c["params"], rc=rc, rc1=0.8 * rc, polar_maxiter=40, polar_eps=1e-8)
    eng = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    a = eng.full_bead_forces(c["RRt"], c["RRc"], t=0)
    tuned = eng.autotune()
    assert set(tuned) == {"sf_tiled", "sf_groups", "ff_regs", "max_slices", "nbr_block", "wave_shapes", "sf_tc", "ff_tc",
                          "dd_overlap", "x_cache", "pdl", "loop_unroll", "ewald_overlap", "dd_otf", "qd_tc", "l2_keep",
                          "dd_async", "dd_pev", "dd_jpev", "nbr_overlap"}
    assert 1 <= tuned["max_slices"] <= 16
    b = eng.full_bead_forces(c["RRt"], c["RRc"], t=0)
    assert rel(b["dRRt"], a["dRRt"]) < 1e-6
    assert rel(b["Upott"], a["Upott"]) < 1e-6
    # pinned shapes: the passes on a second stream or in line, the field pass as a programmatic
    # dependent or a plain launch, are the same arithmetic in the same order (equal up to the
    # FP64 atomic order of the block sums)
    runs = []
    for ov in (0, 1):
        assert eng.set_tuning(dd_overlap=ov, pdl=ov, ewald_overlap=ov)["ewald_overlap"] == ov
        runs.append(eng.full_bead_forces(c["RRt"], c["RRc"], t=0))
    assert rel(runs[0]["dRRt"], runs[1]["dRRt"]) < 1e-7
    # real-space dipole tensors cached per list entry or formed in each iteration: the same
    # FP32 terms contracted in another order
    otf = []
    for v in (0, 1):
        assert eng.set_tuning(dd_otf=v)["dd_otf"] == v
        otf.append(eng.full_bead_forces(c["RRt"], c["RRc"], t=0))
    assert rel(otf[0]["dRRt"], otf[1]["dRRt"]) < 1e-6
    with pytest.raises(ValueError):
        eng.set_tuning(no_such_knob=1)
    eng.close()
