"""GPU parity of the run analyses against the oracle's restatement of the reference's routines:
calc_geometry / write_out_geometry / write_out_histogram (geometry_calculator.f90), calc_diff_RMSD
/ write_out_diffusion (diffusion_calculator.f90), calc_infrared_spectrum and calc_DOS
(spectral_properties.f90 with math.f90 and four1.f; cuFFT on the device).

Tolerances: histogram counts and O-H maxima exact; geometry sums and reports 1e-12 relative (FP64
atomics change the summation order); MSD samples and fit 1e-10; spectra normwise 2e-4 (single
precision transforms of another algorithm), frequencies 1e-12."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FRAMES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_frames.npz")


def setup(pkg, P=4):
    d = np.load(FRAMES)
    RRc, box = d["input_128_RRc"], d["input_128_box"]
    p = dict(pot_model=3, natoms=len(RRc), nbeads=P, box=tuple(box), rc=7.8, rc1=6.24, alpha=0.45, nmax=6,
             polar_maxiter=20, polar_sor=0.7, polar_eps=1e-8)
    return RRc, box, pkg.ForceEngine(p)


def test_geometry_matches_oracle(pkg, orc, engine_lib):
    import torch

    P = 4
    RRc0, box, eng = setup(pkg, P)
    dev = torch.device("cuda", 0)
    g = orc.Geometry(len(RRc0), P, box)
    eng.geometry_reset()
    rng = np.random.default_rng(1)
    for f in range(5):
        RRt = RRc0[None] + rng.normal(scale=0.05, size=(P,) + RRc0.shape)
        RRt[:, 7] += 0.6  # one stretched O-H bond (above the 1.5 A warning mark in some beads)
        RRc = RRt.mean(axis=0)
        a, b = torch.from_numpy(RRc).to(dev), torch.from_numpy(RRt).to(dev)
        eng.geometry_accumulate_device(a.data_ptr(), b.data_ptr())
        torch.cuda.synchronize()
        g.accumulate(RRc, RRt)
    r = eng.geometry_report()
    acc, ref = r["accumulator"], g.acc
    assert np.array_equal(acc[16:], ref[16:])  # both histograms, counts
    assert np.array_equal(acc[12:16], ref[12:16])  # maxima, num_total, warnings
    assert acc[15] > 0 and acc[16:].sum() > 0
    assert np.allclose(acc[:12], ref[:12], rtol=1e-12, atol=0)
    assert np.allclose(r["report"], g.report(), rtol=1e-12, atol=1e-12)
    nt = ref[14]
    assert np.allclose(r["hist_centroid"][:, 1], ref[16:96] / (2 * nt), rtol=0, atol=0)
    eng.close()


def test_msd_matches_oracle(pkg, orc, engine_lib):
    import torch

    RRc0, box, eng = setup(pkg, 2)
    dev = torch.device("cuda", 0)
    steps = 400  # 20 samples: the fit takes the last 9
    m = orc.MSD(len(RRc0), steps, box)
    eng.msd_init(steps)
    rng = np.random.default_rng(2)
    R = RRc0.copy()
    for k in range(steps):
        R = R + rng.normal(scale=0.05, size=R.shape)
        a = torch.from_numpy(R).to(dev)
        eng.msd_accumulate_device(a.data_ptr())
        torch.cuda.synchronize()
        m.step(R)
    got, ref = eng.msd_report(0.25e-3), m.report(0.25e-3)
    assert np.allclose(got["aMS"], ref["aMS"], rtol=1e-10, atol=1e-14)
    for k in ("D", "errD", "slope", "intercept"):
        assert abs(got[k] - ref[k]) <= 1e-10 * abs(ref[k]), k
    eng.close()


def test_spectra_match_oracle(pkg, orc, engine_lib):
    import torch

    P = 2
    RRc0, box, eng = setup(pkg, P)
    nw, na = len(RRc0) // 3, len(RRc0)
    dev = torch.device("cuda", 0)
    T, dt = 300, 0.5e-3
    eng.spectra_init(T, 1.008)
    rng = np.random.default_rng(3)
    ts = np.arange(T) * dt
    dips, hvels = [], []
    CH, DE = 18.22234397655801030455, 4.8033324
    for k in range(T):
        # dipoles with two vibrations (3700 and 1600 cm^-1) and noise; momenta likewise
        w = 2 * np.pi * 3.0e10 * 1e-12 * np.array([3700.0, 1600.0])
        dip = (rng.normal(scale=0.2, size=(P, nw, 3)) + np.cos(w[0] * ts[k]) + 0.5 * np.sin(w[1] * ts[k])) * CH
        PPt = rng.normal(scale=1.0, size=(P, na, 3)) + 3 * np.cos(w[0] * ts[k])
        a, b = torch.from_numpy(dip).to(dev), torch.from_numpy(PPt).to(dev)
        eng.spectra_record_device(a.data_ptr(), b.data_ptr())
        torch.cuda.synchronize()
        dm = (dip * DE / CH).sum(axis=0) / P  # per molecule, bead-averaged (Debye)
        dips.append(dm.sum(axis=0).astype(np.float32))
        Pc = PPt.sum(axis=0) / P
        hv = np.zeros((2 * nw, 3))
        hv[1::2] = Pc[1::3] * (1.0 / 1.008)
        hv[0::2] = Pc[0::3] * (1.0 / 1.008)
        hvels.append(hv.astype(np.float32))
    dips = np.array(dips)
    hvel = np.transpose(np.array(hvels), (1, 0, 2))
    f, ir = eng.ir_spectrum(dt, 300.0)
    fr, irr = orc.ir_spectrum(dips, box, dt, 300.0)
    assert len(f) == len(fr) and np.allclose(f, fr, rtol=1e-12)
    assert np.abs(ir - irr).max() <= 2e-4 * np.abs(irr).max()
    f, d = eng.dos(dt)
    fr, dr = orc.dos(hvel, dt)
    assert len(f) == len(fr) and np.allclose(f, fr, rtol=1e-12)
    assert np.abs(d - dr).max() <= 2e-4 * np.abs(dr).max()
    eng.close()
