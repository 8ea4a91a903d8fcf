#!/usr/bin/env python3
"""Differentiation-form study (TTM3-F 512 H2O x 32 beads, L = 24.86 A, Rc = 9 A, |n| <= 12):
the FP64 adjoint backward (pimd_pot_backward) against central finite differences of the
forward energies, and the reference's analytic forces against the same finite differences, on
seeded frames with the model parameters theta perturbed uniformly by +-5 % from the published
values; then a sweep of the induced-dipole tolerance.

For each frame: E = sum_k w_k Upot_k with seeded bead weights w; the adjoint gives dE/dx and
dE/dtheta. Finite differences: h = 1e-5 A on `--ncomp` random coordinates, 1e-4 relative on
every theta (smaller steps drown in the rounding noise of FP64 atomic sums). Tolerance sweep:
the adjoint and the analytic (Hellmann-Feynman) gradient against finite differences at each
tolerance (with rc1 = Rc, so the force-only vdW switch of pot_ttm.f90:171 does not separate
them); the finite differences use the same tolerance (the stopping iteration does not move for
steps this small, which the script checks).

Mixed engine: on every frame the same forward + backward on a mixed-precision context (FP32
operators, FP64 sums), compared with the FP64 gradients (RMS relative for positions, largest
relative to the largest for theta), with the wall times of both engines' forward and backward.

  python pimd-f90_gb300/adjoint_study.py --frames 20
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=20)
    ap.add_argument("--ncomp", type=int, default=6)
    ap.add_argument("--eps", type=float, default=1e-8)
    ap.add_argument("--sweep", default="1e-4,1e-6,1e-8,1e-10")
    args = ap.parse_args()
    pkg = ge.load_package()
    pkg.build_lib.build()
    E = pkg.engine
    rng = np.random.default_rng(20261203 + 3)
    base = pkg.waterbox.make_config("ttm3f_512x32")
    p0 = dict(base["params"], polar_eps=args.eps, polar_maxiter=200, guess_initdip=0)
    P = p0["nbeads"]
    eng = E.ForceEngine(p0)
    engm = E.ForceEngine(p0, precision=E.PIMD_MIXED)
    th_pub = eng.get_theta()
    t0 = time.time()
    frames = []
    times = dict(fp64_forward=[], fp64_backward=[], mixed_forward=[], mixed_backward=[])
    for f in range(args.frames):
        c = pkg.waterbox.make_config("ttm3f_512x32", seed=20261203 + 3 + 101 * (f + 1))
        th = th_pub * (1.0 + rng.uniform(-0.05, 0.05, size=th_pub.shape))
        eng.set_theta(th)
        w = rng.uniform(0.5, 1.5, size=P)
        R, Rc = c["RRt"], c["RRc"]

        def energy(RR, theta=None):
            if theta is not None:
                eng.set_theta(theta)
            U = eng.pot_forward(RR, Rc)
            if theta is not None:
                eng.set_theta(th)
            return float(np.dot(w, U))

        ta = time.perf_counter()
        e0 = energy(R)
        tb = time.perf_counter()
        g, dth = eng.pot_backward(w)
        tc = time.perf_counter()
        engm.set_theta(th)
        engm.pot_forward(R, Rc)
        td = time.perf_counter()
        gm, dthm = engm.pot_backward(w)
        te = time.perf_counter()
        for k, v in zip(times, (tb - ta, tc - tb, td - tc, te - td)):
            times[k].append(1e3 * v)
        mixed_g = float(np.sqrt(((gm - g) ** 2).mean() / (g ** 2).mean()))
        mixed_th = float(np.abs(dthm - dth).max() / np.abs(dth).max())
        gs = np.abs(g).max()
        errx = 0.0
        for _ in range(args.ncomp):
            b, a, k = int(rng.integers(P)), int(rng.integers(p0["natoms"])), int(rng.integers(3))
            Rp, Rm = R.copy(), R.copy()
            Rp[b, a, k] += 1e-5
            Rm[b, a, k] -= 1e-5
            fd = (energy(Rp) - energy(Rm)) / 2e-5
            errx = max(errx, abs(fd - g[b, a, k]) / gs)
        errt = []
        for i in range(len(th)):
            h = 1e-4 * abs(th[i])
            tp, tm = th.copy(), th.copy()
            tp[i] += h
            tm[i] -= h
            fd = (energy(R, tp) - energy(R, tm)) / (2 * h)
            errt.append(abs(fd - dth[i]) / max(abs(fd), 1e-9 * abs(e0)))
        frames.append(dict(frame=f, grad_fd_err=errx, theta_fd_err_max=max(errt),
                           theta_fd_err={n: e for n, e in zip(E.THETA_NAMES, errt)},
                           mixed_grad_rms_rel=mixed_g, mixed_theta_rel=mixed_th))
    eng.set_theta(th_pub)
    # tolerance sweep on the first frame
    sweep = []
    c = pkg.waterbox.make_config("ttm3f_512x32", seed=20261203 + 3 + 101)
    R, Rc = c["RRt"], c["RRc"]
    w = np.ones(P)
    for tol in [float(x) for x in args.sweep.split(",")]:
        # rc1 = rc: no force-only vdW switch, so analytic and exact gradients differ by the
        # dipole convergence alone
        e2 = E.ForceEngine(dict(p0, polar_eps=tol, rc1=p0["rc"]))
        U = e2.pot_forward(R, Rc)
        niter = [e2.energies(k)["niter"] for k in range(P)]
        g, _ = e2.pot_backward(w)
        hf = e2.full_bead_forces(R, Rc)["dRRt"]
        gs = np.abs(g).max()
        ea, eh, moved = 0.0, 0.0, False
        for _ in range(args.ncomp):
            b, a, k = int(rng.integers(P)), int(rng.integers(p0["natoms"])), int(rng.integers(3))
            vals = []
            for s in (1, -1):
                Rs = R.copy()
                Rs[b, a, k] += s * 1e-5
                vals.append(float(np.dot(w, e2.pot_forward(Rs, Rc))))
                moved |= e2.energies(b)["niter"] != niter[b]
            fd = (vals[0] - vals[1]) / 2e-5
            ea = max(ea, abs(fd - g[b, a, k]) / gs)
            eh = max(eh, abs(fd - hf[b, a, k]) / gs)
        sweep.append(dict(polar_eps=tol, mean_iterations=float(np.mean(niter)), adjoint_vs_fd=ea,
                          analytic_vs_fd=eh, stopping_iteration_moved=moved))
        e2.close()
    out = dict(workload="TTM3-F 512 H2O x 32 beads, FP64 (finite differences) and mixed, theta +-5 %", frames=len(frames),
               grad_fd_err_max=max(f["grad_fd_err"] for f in frames),
               theta_fd_err_max=max(f["theta_fd_err_max"] for f in frames),
               mixed_vs_fp64=dict(grad_rms_rel_max=max(f["mixed_grad_rms_rel"] for f in frames),
                                  theta_rel_max=max(f["mixed_theta_rel"] for f in frames),
                                  ms_median={k: round(float(np.median(v[1:] if len(v) > 1 else v)), 2)
                                             for k, v in times.items()}),
               per_frame=frames, tolerance_sweep=sweep, wall_s=round(time.time() - t0, 1))
    print(json.dumps(out))


if __name__ == "__main__":
    main()
