"""Exact restart (pimd_checkpoint_write / pimd_checkpoint_read) through the C ABI: a run of 8 MD
steps with the dipole predictor and both Nose-Hoover chains, interrupted after step 4 and continued
from the file in a fresh context, equals the uninterrupted run (FP64 engine: gradients and positions
1e-12 relative, the order of the FP64 atomics of the force sums being the only difference); a
restart from the same coordinates without the file's predictor history and chain state does not.
Files from another system are refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DELT, T = 0.25e-3, 300.0


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def context(pkg, nw=32, P=4):
    W = pkg.waterbox
    c = W.make_config("ttm3f_512x32", nw=nw, P=P)
    L = c["params"]["box"][0]
    rc = min(9.0, L / 2 - 0.01)
    p = dict(c["params"], rc=rc, rc1=0.8 * rc, alpha=3.5 / rc, nmax=8, polar_maxiter=60, polar_eps=1e-6,
             guess_initdip=1)
    eng = pkg.ForceEngine(p)
    eng.nm_init(P, W.KB_AMU * T * P / W.HBAR, DELT)
    eng.langevin_init(DELT / 2, 0, 0.1, P * T)
    eng.set_thermostat(bead_thermostat=2, global_thermostat=1, tau=0.05, temp=T, centroid_thermostat=1,
                       tau_centroid=0.02)
    eng.set_thermostat_state(np.ones(2), 15.0)
    mp = eng.md_params(DELT, c["massO"], c["massH"], langevin=0, seed=31)
    return c, eng, mp


def test_restart_reproduces_the_uninterrupted_run(pkg, engine_lib, tmp_path):
    c, eng, mp = context(pkg)
    R, Pm, g = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    path = tmp_path / "run.ckpt"
    for t in range(1, 9):
        eng.md_step_ex(mp, R, Pm, g, t)
        if t == 4:
            eng.checkpoint_write(path, R, Pm, g, t, 31)
            R4, P4, g4 = R.copy(), Pm.copy(), g.copy()
    eng.close()
    # a fresh context continued from the file
    c2, eng2, mp2 = context(pkg)
    Rb, Pb, gb, t0, seed = eng2.checkpoint_read(path)
    assert t0 == 4 and seed == 31
    assert np.array_equal(Rb, R4) and np.array_equal(Pb, P4) and np.array_equal(gb, g4)
    for t in range(t0 + 1, 9):
        eng2.md_step_ex(mp2, Rb, Pb, gb, t)
    assert rel(gb, g) < 1e-12 and rel(Rb, R) < 1e-12 and rel(Pb, Pm) < 1e-11
    eng2.close()
    # the same coordinates without the file's history and chain state: another trajectory
    c3, eng3, mp3 = context(pkg)
    Rc, Pc, gc = R4.copy(), P4.copy(), g4.copy()
    for t in range(5, 9):
        eng3.md_step_ex(mp3, Rc, Pc, gc, t)
    assert rel(gc, g) > 1e-9
    eng3.close()


def test_restart_refuses_another_system(pkg, engine_lib, tmp_path):
    c, eng, mp = context(pkg, nw=32, P=4)
    path = tmp_path / "a.ckpt"
    R, Pm, g = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    eng.checkpoint_write(path, R, Pm, g, 0, 1)
    eng.close()
    c2, eng2, _ = context(pkg, nw=32, P=2)
    with pytest.raises(pkg.PimdError):
        eng2.checkpoint_read(path)
    eng2.close()
