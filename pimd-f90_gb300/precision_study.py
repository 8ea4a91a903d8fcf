#!/usr/bin/env python3
"""Precision-form study: the mixed engine (FP32 pair and Ewald-phase arithmetic, FP64
accumulation) against the FP64 engine on the same trajectories.

Two measurements, printed as one JSON line:

1. Frame-by-frame error. An FP64 PILE trajectory is run; every `--every` steps the mixed engine
   evaluates the same frame and its energy, gradient (force) RMS, induced dipoles and virial are
   compared with the FP64 engine's on that frame.
2. NVE drift. From the end of that thermalised trajectory both engines run NVE (no thermostat)
   for `--nve-steps` steps from the same phase-space point. The conserved ring-polymer energy
     H = [sum p^2/2m + sum_j 1/2 m w_P^2 |x_j - x_j+1|^2] / MASSCON + sum_j V(x_j)
   (kcal/mol; the reference's PIMD_VV integrates exactly this Hamiltonian, MD.f90:35-110 with
   the free-ring propagator of NormalModes.f90:34-63) is sampled and its linear drift per ps and
   per molecule is fitted for each engine.

  python pimd-f90_gb300/precision_study.py --config ttm21f_128x32 --steps 2000 --every 20
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

MASSCON = 418.4
KB_AMU = 0.831447148
HBAR = 6.35077993041


def ring_energy(RRt, PPt, masses, omegan):
    """Kinetic + spring energy of the ring polymer (amu A^2/ps^2)."""
    ke = 0.5 * (PPt ** 2 / masses[None, :, None]).sum()
    d = RRt - np.roll(RRt, -1, axis=0)
    spring = 0.5 * omegan ** 2 * (masses[None, :, None] * d ** 2).sum()
    return ke + spring


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="ttm21f_128x32")
    ap.add_argument("--steps", type=int, default=2000, help="thermostatted FP64 steps with frame comparisons")
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--nve-steps", type=int, default=2000)
    ap.add_argument("--nve-every", type=int, default=10)
    ap.add_argument("--dt-fs", type=float, default=0.25)
    ap.add_argument("--temp", type=float, default=300.0)
    ap.add_argument("--polar-eps", type=float, default=1e-8)
    args = ap.parse_args()
    pkg = ge.load_package()
    pkg.build_lib.build()
    W = pkg.waterbox
    c = W.make_config(args.config)
    p = dict(c["params"], polar_eps=args.polar_eps, polar_maxiter=200, guess_initdip=1)
    P, na = p["nbeads"], p["natoms"]
    masses = np.where(np.arange(na) % 3 == 0, c["massO"], c["massH"])
    delt = args.dt_fs / 1000.0
    omegan = KB_AMU * args.temp * P / HBAR

    def engine(prec, langevin):
        e = pkg.ForceEngine(p, precision=prec)
        e.nm_init(P, omegan, delt)
        e.langevin_init(delt / 2, 0, 0.1, P * args.temp)
        e.set_graph(True)
        return e, e.md_params(delt, c["massO"], c["massH"], langevin=langevin, seed=4242)

    e64, mp64 = engine(pkg.engine.PIMD_FP64, 1)
    emx = pkg.ForceEngine(p, precision=pkg.engine.PIMD_MIXED)
    R, Pm, g = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    errs = dict(energy_abs=[], energy_rel=[], force_rms_rel=[], force_max_rel=[], dipole_rms_rel=[], virial_rel=[])
    t0 = time.time()
    for t in range(1, args.steps + 1):
        _, RRc = e64.md_step(mp64, R, Pm, g, t)
        if t % args.every == 0:
            a = e64.full_bead_forces(R, RRc, t=t)
            b = emx.full_bead_forces(R, RRc, t=t)
            du = b["Upott"] - a["Upott"]
            errs["energy_abs"].append(float(np.abs(du).max()))
            errs["energy_rel"].append(float(np.abs(du).max() / np.abs(a["Upott"]).max()))
            errs["force_rms_rel"].append(float(np.sqrt(((b["dRRt"] - a["dRRt"]) ** 2).mean() / (a["dRRt"] ** 2).mean())))
            errs["force_max_rel"].append(float(np.abs(b["dRRt"] - a["dRRt"]).max() / np.abs(a["dRRt"]).max()))
            errs["dipole_rms_rel"].append(float(np.sqrt(((b["dip_momIt"] - a["dip_momIt"]) ** 2).mean() /
                                                        (a["dip_momIt"] ** 2).mean())))
            errs["virial_rel"].append(float(np.abs(b["virialt"] - a["virialt"]).max() / np.abs(a["virialt"]).max()))
    t_frames = time.time() - t0
    emx.close()
    # NVE from the thermalised point, both engines
    drift = {}
    for name, prec in (("fp64", pkg.engine.PIMD_FP64), ("mixed", pkg.engine.PIMD_MIXED)):
        e, mp = engine(prec, 0)
        R2, P2, g2 = R.copy(), Pm.copy(), g.copy()
        ts, H = [], []
        for k in range(1, args.nve_steps + 1):
            out, _ = e.md_step(mp, R2, P2, g2, args.steps + k)
            if k % args.nve_every == 0:
                ts.append(k * delt)
                H.append(ring_energy(R2, P2, masses, omegan) / MASSCON + out[0])
        ts, H = np.array(ts), np.array(H)
        slope = np.polyfit(ts, H, 1)[0]
        drift[name] = dict(drift_kcal_per_mol_ps_per_molecule=float(slope / (na // 3)),
                           H_rms_fluct=float(np.std(H - np.polyval(np.polyfit(ts, H, 1), ts))),
                           H0=float(H[0]), samples=len(H))
        e.close()
    e64.close()
    d64, dmx = drift["fp64"]["drift_kcal_per_mol_ps_per_molecule"], drift["mixed"]["drift_kcal_per_mol_ps_per_molecule"]
    summary = {k: dict(max=float(np.max(v)), mean=float(np.mean(v))) for k, v in errs.items()}
    print(json.dumps(dict(config=args.config, model=p["pot_model"], nw=na // 3, beads=P, dt_fs=args.dt_fs,
                          polar_eps=args.polar_eps, frames=len(errs["energy_abs"]), steps=args.steps,
                          frame_errors=summary, nve=drift, nve_steps=args.nve_steps,
                          drift_ratio_mixed_over_fp64=dmx / d64 if d64 else None, wall_s=round(t_frames, 1))))


if __name__ == "__main__":
    main()
