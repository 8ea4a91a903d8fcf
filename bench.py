#!/usr/bin/env python3
"""Benchmark: full PIMD velocity-Verlet MD steps per second for TTM3-F water, 512 H2O x 32
beads (L = 24.86 A, Rc = 9 A, Ewald |n| <= 12, T = 300 K, dt = 0.25 fs, PILE thermostat),
on synthetic jittered-lattice boxes (seeded; the reference ships no benchmark dataset).

One step = Langevin_NM, half kick, EvolveRing for every atom, centroid + PBCs, the force
call for all 32 beads (monomer PES, real-space charge/dipole sums, Ewald reciprocal sums,
induced-dipole solve to 1e-8 with the 4-step predictor), half kick, Langevin_NM
(MD.f90:35-110).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm times the CUDA engine through its C ABI with the MD state resident in HBM (value)
and again through the host-array entry point with host<->device copies every step (e2e).
The reference arm times the reference algorithm (CPU FP64 restatement, threads over beads
like the reference's MPI ranks) on this machine's host cores. Multi-GPU runs are
independent replicas, one per rank (the path has no cross-replica exchange).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

METRIC = "TTM3-F 512 H2O×32 beads: MD steps/s mixed vs FP64 GPU at ≤1e-4 rel force err"
CONFIG = "ttm3f_512x32"
DT_FS = 0.25
TEMP = 300.0
POLAR = dict(polar_eps=1e-8, polar_maxiter=100, guess_initdip=1, polar_sor=0.7)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=CONFIG)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch", action="store_true",
                    help="the batching form instead of the headline: 64 TTM3-F replicas of uneven sizes in one graph")
    ap.add_argument("--batch-replicas", type=int, default=64)
    ap.add_argument("--config-large", action="store_true",
                    help="TTM3-F 4096 H2O x 32 beads (|n| <= 24) steps/s for FP64, mixed and mixed+graph")
    ap.add_argument("--profile-force", choices=["fp64", "mixed"],
                    help="run two force calls of the workload and exit (the case profiled with ncu)")
    ap.add_argument("--profile-md", choices=["fp64", "mixed"],
                    help="run three eager MD steps of the workload and exit (integrator kernels under ncu)")
    ap.add_argument("--profile-backward", choices=["fp64", "mixed"],
                    help="run two forward + backward pairs of the differentiation form on the workload and exit")
    return ap.parse_args()


def profile_force(pkg, which):
    c, p = workload(pkg, CONFIG)
    prec = pkg.engine.PIMD_MIXED if which == "mixed" else pkg.engine.PIMD_FP64
    eng = pkg.ForceEngine(p, precision=prec)
    for t in (1, 2):
        r = eng.full_bead_forces(c["RRt"], c["RRc"], t=t)
    print(json.dumps(dict(profile_force=which, Upot=float(r["Upot"]), niter=eng.energies(0)["niter"])))
    eng.close()


def profile_md(pkg, which):
    c, p = workload(pkg, CONFIG)
    prec = pkg.engine.PIMD_MIXED if which == "mixed" else pkg.engine.PIMD_FP64
    eng = pkg.ForceEngine(p, precision=prec)
    P = p["nbeads"]
    delt = DT_FS / 1000.0
    eng.nm_init(P, pkg.waterbox.KB_AMU * TEMP * P / pkg.waterbox.HBAR, delt)
    eng.langevin_init(delt / 2, 0, 0.1, P * TEMP)
    mp = eng.md_params(delt, c["massO"], c["massH"], langevin=1, seed=replica_seed(0))
    RRt, PPt, dRRt = c["RRt"].copy(), c["PPt"].copy(), np.zeros_like(c["RRt"])
    for t in (1, 2, 3):
        out, _ = eng.md_step(mp, RRt, PPt, dRRt, t)
    print(json.dumps(dict(profile_md=which, Upot=float(out[0]), uk=float(out[3]))))
    eng.close()


def profile_backward(pkg, which):
    c, p = workload(pkg, CONFIG)
    prec = pkg.engine.PIMD_MIXED if which == "mixed" else pkg.engine.PIMD_FP64
    eng = pkg.ForceEngine(p, precision=prec)
    ebar = np.ones(p["nbeads"])
    for _ in range(2):
        t0 = time.perf_counter()
        U = eng.pot_forward(c["RRt"], c["RRc"])
        t1 = time.perf_counter()
        g, dth = eng.pot_backward(ebar)
        t2 = time.perf_counter()
    print(json.dumps(dict(profile_backward=which, Upot=float(U.sum()), forward_ms=round(1e3 * (t1 - t0), 2),
                          backward_ms=round(1e3 * (t2 - t1), 2), grad_max=float(np.abs(g).max()))))
    eng.close()


def batch_workload(pkg, nrep, seed=20261203 + 4):
    """64 replicas: N from {32, 64, 128, 256}, P from {8, 16, 32}, T uniform in [250, 350] K, each at
    0.997 g/cm^3 (L = (N 29.96 A^3)^(1/3)) with cutoff min(9 A, L/2), seeded."""
    rng = np.random.default_rng(seed)
    reps, states = [], []
    for i in range(nrep):
        nw = int(rng.choice([32, 64, 128, 256]))
        P = int(rng.choice([8, 16, 32]))
        T = float(rng.uniform(250.0, 350.0))
        c = pkg.waterbox.make_config("ttm3f_512x32", nw=nw, P=P, T=T, seed=seed + 1000 + i)
        L = c["params"]["box"][0]
        reps.append(dict(natoms=3 * nw, nbeads=P, box=(L, L, L), temp=T))
        states.append(c)
    return reps, states


def run_batch(args, pkg):
    import torch

    reps, states = batch_workload(pkg, args.batch_replicas)
    common = dict(pot_model=3, rc=9.0, rc1=7.2, alpha=0.0, eps_ewald=1e-6, **POLAR)
    out = {}
    for name, prec, steps in (("mixed", pkg.engine.PIMD_MIXED, args.steps), ("fp64", pkg.engine.PIMD_FP64,
                                                                          max(3, min(args.steps, 20)))):
        bt = pkg.engine.ReplicaBatch(common, reps, DT_FS / 1000.0, 15.9994, 1.008, langevin=1, seed=20261203,
                                     precision=prec)
        for i, c in enumerate(states):
            bt.set_state(i, c["RRt"], c["PPt"])
        t0 = time.perf_counter()
        bt.autotune()
        tune_s = time.perf_counter() - t0
        bt.forces()
        bt.step(args.warmup)
        bt.sync()
        with ClockSampler(0) as clk:
            t0 = time.perf_counter()
            bt.step(steps)
            bt.sync()
            dt = time.perf_counter() - t0
        ng, gof = bt.groups()
        energies = [bt.get_state(i)[3][0] for i in range(len(reps))]
        out[name] = dict(batch_steps_per_s=steps / dt, steps=steps, ms_per_step=1000 * dt / steps, groups=ng,
                         autotune_s=round(tune_s, 2), clocks=clk.summary(),
                         finite=bool(np.all(np.isfinite(energies))))
        bt.close()
    beads = sum(r["nbeads"] for r in reps)
    mol_beads = sum(r["nbeads"] * r["natoms"] // 3 for r in reps)
    line = dict(metric="batch of %d uneven TTM3-F replicas: batch MD steps/s (all replicas advance one step)" % len(reps),
                value=out["mixed"]["batch_steps_per_s"], unit="batch steps/s", n_gpus=1, higher_is_better=True,
                dtype="f32 pair/phase arithmetic, f64 accumulation", data="synthetic (seeded replicas)",
                config=dict(workload="64 replicas, N in {32,64,128,256}, P in {8,16,32}, T in [250,350] K, "
                                     "rc = min(9, L/2), Ewald eps 1e-6", replicas=len(reps), total_beads=beads,
                            molecule_beads=mol_beads, timing="host wall clock around stream-ordered graph launches"),
                mixed=out["mixed"], fp64=out["fp64"], mixed_over_fp64=out["mixed"]["batch_steps_per_s"] /
                out["fp64"]["batch_steps_per_s"])
    print(json.dumps(line))


def run_large(args, pkg):
    """TTM3-F 4096 H2O x 32 beads, L = 49.72 A, Rc = 9 A, |n| <= 24: steps/s per precision form."""
    res = {}
    for name, prec, graph, steps in (("mixed", pkg.engine.PIMD_MIXED, False, args.steps),
                                     ("mixed_graph", pkg.engine.PIMD_MIXED, True, args.steps),
                                     ("fp64", pkg.engine.PIMD_FP64, False, max(2, min(args.steps, 4)))):
        r = run_gpu_arm(args, pkg, 0, 1, 0, prec, steps, graph=graph)
        res[name] = dict(steps_per_s=steps / (r["dev_ms"] / 1000.0), ms_per_step=r["dev_ms"] / steps, steps=steps,
                         dipole_iterations_mean=float(np.mean(r["niters"])), clocks=r["clocks"])
    print(json.dumps(dict(metric="TTM3-F 4096 H2O x 32 beads: MD steps/s", unit="steps/s",
                          value=res["mixed_graph"]["steps_per_s"], config=dict(workload="ttm3f_4096x32"), **res)))


def workload(pkg, name):
    c = pkg.waterbox.make_config(name)
    p = dict(c["params"])
    p.update(POLAR)
    return c, p


# DRAM bytes (read + write) of one mixed ewald_std_dd call at the headline workload, from one
# ncu capture of its two kernels (k_sfac_tc 34.8 MB -- the tables plus the cached X operand,
# 31.5 MB, loaded evict-first -- and k_field_tc 7.4 MB, cold cache)
DD_TRAFFIC_BYTES = 42.3e6


def tensor_flops_dd(nmax, ndip, P):
    """Tensor-core flops one mixed ewald_std_dd call executes (3 products of the FP16 hi + lo
    split, padding included): structure factor M = 128 x N = 2 runs (rounded to 16) x K = the
    dipole sites; field pass M = the sites (128 per tile) x N = 4 runs x K = 2 (nmax + 1)."""
    nrun = 0
    for kx in range(0, nmax + 1):
        for ky in range(-nmax, nmax + 1):
            if (kx == 0 and ky < 0) or kx * kx + ky * ky > nmax * nmax:
                continue
            if kx == 0 and ky == 0 and nmax < 1:
                continue
            nrun += 1
    r16 = lambda x: (x + 15) // 16 * 16
    ksites = r16(ndip)
    sfac = 6.0 * 128 * r16(2 * nrun) * ksites
    field = 6.0 * ((ksites + 127) // 128 * 128) * r16(4 * nrun) * r16(2 * (nmax + 1))
    return P * (sfac + field)


def flops_ewald_dd(nk, ndip, P):
    """Algorithmic flops of one ewald_std_dd call for P beads (ewald.f90:56-119): 22 per
    (k-vector, dipole site), the per-unit count of the reference's loop body."""
    return 22.0 * nk * ndip * P


def reduce_max(value, device, world):
    """The job's time is the slowest rank's: max over ranks (no-op for one rank)."""
    if world <= 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank):
    """Each rank is an independent replica: its own Langevin stream."""
    return 20261203 + rank


# ---------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for ln in fh:
                parts = [x.strip() for x in ln.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------------------
def force_error(pkg, local):
    """Mixed vs FP64 engine on the initial frame: RMS and max relative gradient error."""
    c, p = workload(pkg, CONFIG)
    out = {}
    for prec in (pkg.engine.PIMD_FP64, pkg.engine.PIMD_MIXED):
        eng = pkg.ForceEngine(p, precision=prec, device=local)
        out[prec] = eng.full_bead_forces(c["RRt"], c["RRc"], t=1)
        eng.close()
    a, b = out[pkg.engine.PIMD_MIXED]["dRRt"], out[pkg.engine.PIMD_FP64]["dRRt"]
    rms = float(np.sqrt(((a - b) ** 2).mean() / (b ** 2).mean()))
    mx = float(np.abs(a - b).max() / np.abs(b).max())
    ue = out[pkg.engine.PIMD_MIXED]["Upott"] - out[pkg.engine.PIMD_FP64]["Upott"]
    return dict(force_rel_rms=rms, force_rel_max=mx, energy_abs_max=float(np.abs(ue).max()))


def run_gpu_arm(args, pkg, rank, world, local, precision, steps, graph=False):
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    c, p = workload(pkg, args.config)
    P, na, nw = p["nbeads"], p["natoms"], p["natoms"] // 3
    # one non-default stream carries the engine's kernels, the L2 flush and the timing events
    stream = torch.cuda.Stream(dev)
    eng = pkg.ForceEngine(p, precision=precision, device=local)
    eng.set_stream(stream.cuda_stream)
    eng.set_graph(graph)
    alpha, nk, _ = eng.ewald_info()
    delt = DT_FS / 1000.0
    omegan = pkg.waterbox.KB_AMU * TEMP * P / pkg.waterbox.HBAR
    eng.nm_init(P, omegan, delt)
    eng.langevin_init(delt / 2, 0, 0.1, P * TEMP)
    mp = eng.md_params(delt, c["massO"], c["massH"], langevin=1, seed=replica_seed(rank))
    # device-resident MD state
    RRt = torch.from_numpy(c["RRt"]).to(dev)
    PPt = torch.from_numpy(c["PPt"]).to(dev)
    dRRt = torch.zeros_like(RRt)
    RRc = torch.zeros((na, 3), dtype=torch.float64, device=dev)
    out4 = torch.zeros(4, dtype=torch.float64, device=dev)
    RRc.copy_(RRt.mean(0))
    torch.cuda.synchronize(dev)
    pkg.engine.load().pimd_full_bead_forces_device(eng.h, RRt.data_ptr(), RRc.data_ptr(), None, dRRt.data_ptr(),
                                                   None, None, None, None, None, 1)
    with torch.cuda.stream(stream):
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2
    t = 1
    for _ in range(args.warmup):
        eng.md_step_device(mp, RRt.data_ptr(), PPt.data_ptr(), dRRt.data_ptr(), RRc.data_ptr(), t, out4.data_ptr())
        t += 1
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    eng.timers_reset(True)
    L = pkg.engine.load()
    launches0 = L.pimd_launch_count(eng.h)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    niters = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize(dev)
        wall0 = time.perf_counter()
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
            ev[k][0].record(stream)
            eng.md_step_device(mp, RRt.data_ptr(), PPt.data_ptr(), dRRt.data_ptr(), RRc.data_ptr(), t, out4.data_ptr())
            ev[k][1].record(stream)
            if k % 10 == 0 or k == steps - 1:
                niters.append(eng.energies(0)["niter"])  # synchronises the stream
            t += 1
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - wall0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    launches = L.pimd_launch_count(eng.h) - launches0
    graph_launches = eng.graph_info()[1]
    timers = eng.timers()
    eng.timers_reset(False)
    dev_ms = reduce_max(sum(step_ms), dev, world)
    out = out4.cpu().numpy()
    # e2e: the host-array C-ABI step, copies in and out every step, from pinned host memory
    def pinned(x):
        h = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
        h.copy_(x)
        return h.numpy()

    hR, hP, hG = pinned(RRt), pinned(PPt), pinned(dRRt)
    e2e_steps = max(3, steps // 2)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        eng.md_step(mp, hR, hP, hG, t)
        t += 1
    e2e_s = time.perf_counter() - t0
    res = dict(dev_ms=dev_ms, step_ms=step_ms, wall=wall, timers=timers, niters=niters, clocks=clk.summary(),
               launches=launches, graph_launches=graph_launches,
               out=out.tolist(), nk=nk, alpha=alpha, P=P, nw=nw, e2e_s=e2e_s, e2e_steps=e2e_steps,
               h2d=3 * hR.nbytes, d2h=3 * hR.nbytes + 4 * 8 + hR.shape[1] * 24, tuning=eng.tuning())
    eng.close()
    return res


def cpu_baseline(pkg, orc, steps, warm=1):
    """Reference algorithm (CPU FP64 restatement) on all host cores: bead pool threads. The first
    `warm` of `steps` MD steps are untimed."""
    c, p = workload(pkg, CONFIG)
    ncores = os.cpu_count() or 1
    pool = orc.Pool(p, nthreads=ncores)
    o = orc.Oracle(p)
    md = dict(delt=DT_FS / 1000.0, massO=c["massO"], massH=c["massH"], temp=TEMP, langevin=1)
    RRt, PPt = c["RRt"].copy(), c["PPt"].copy()
    dRRt = np.zeros_like(RRt)
    rng = np.random.default_rng(1)
    P, na = RRt.shape[0], RRt.shape[1]
    ts = []
    for k in range(steps):
        xi1, xi2 = rng.standard_normal((na, P, 3)), rng.standard_normal((na, P, 3))
        t0 = time.perf_counter()
        orc.pimd_vv_step(o, md, RRt, PPt, dRRt, xi1, xi2, t=k + 1, pool=pool)
        ts.append(time.perf_counter() - t0)
    # the first step has no predictor history and a zero gradient for the first kick
    timed = ts[warm:] if len(ts) > warm else ts[-1:]
    return dict(value=len(timed) / sum(timed), cores=ncores, step_s=ts)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pkg = ge.load_package()
    if args.profile_force:
        pkg.build_lib.build()
        profile_force(pkg, args.profile_force)
        return 0
    if args.profile_md:
        pkg.build_lib.build()
        profile_md(pkg, args.profile_md)
        return 0
    if args.profile_backward:
        pkg.build_lib.build()
        profile_backward(pkg, args.profile_backward)
        return 0
    if args.impl == "reference":
        if rank != 0:
            return 0
        orc = ge.load_oracle()
        orc.build()
        # a bounded sample: at most 20 timed MD steps (~15 s on 16 cores) after W (at most 5)
        # untimed ones
        warm = min(max(1, args.warmup), 5)
        steps = min(max(1, args.steps), 20) + warm
        r = cpu_baseline(pkg, orc, steps, warm)
        line = dict(metric=METRIC, value=r["value"], unit="steps/s", n_gpus=args.gpus, steps=steps - warm,
                    warmup=warm, ms_per_step=1000.0 / r["value"], higher_is_better=True, scaling="weak",
                    vs_baseline=None, dtype="f64", data="synthetic", impl="reference",
                    config=dict(workload=CONFIG + " (TTM3-F, 512 H2O x 32 beads, L=24.86 A, Rc=9 A, |n|<=12)",
                                polar_eps=POLAR["polar_eps"], dt_fs=DT_FS),
                    cpu_baseline=dict(value=r["value"], unit="steps/s", cores=r["cores"], kind="port",
                                      sample="%d MD steps of 512 H2O x 32 beads after %d untimed" % (steps - warm, warm)),
                    e2e=dict(value=r["value"], unit="steps/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
        print(json.dumps(line))
        return 0

    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", rank=rank, world_size=world)
        if local == 0:  # one build per node; the other ranks load what it wrote
            pkg.build_lib.build()
        dist.barrier()
    else:
        pkg.build_lib.build()
    if args.batch:
        run_batch(args, pkg)
        return 0
    if args.config_large:
        args.config = "ttm3f_4096x32"
        run_large(args, pkg)
        return 0
    # the FP64 engine is the comparison arm: at most 40 timed steps (~2.5 s)
    steps64 = min(args.steps, 40)
    res64 = run_gpu_arm(args, pkg, rank, world, local, pkg.engine.PIMD_FP64, steps64)
    # mixed precision, eager launches with per-phase timers (the roofline and phase breakdown)
    rese = run_gpu_arm(args, pkg, rank, world, local, pkg.engine.PIMD_MIXED, args.steps)
    # headline: mixed precision with the whole MD step replayed as one CUDA graph
    res = run_gpu_arm(args, pkg, rank, world, local, pkg.engine.PIMD_MIXED, args.steps, graph=True)
    if rank != 0:
        return 0
    ferr = force_error(pkg, local)
    steps_total = args.steps * world
    value = steps_total / (res["dev_ms"] / 1000.0)
    ms_per_step = res["dev_ms"] / args.steps
    eager_value = steps_total / (rese["dev_ms"] / 1000.0)
    timers = rese["timers"]
    # dominant phase and the ewald_std_dd roofline (dd_smu + dd_update implement ewald_std_dd)
    phases = sorted(timers.items(), key=lambda kv: -kv[1][0])
    dd_ms = timers.get("dd_smu", (0, 0))[0] + timers.get("dd_update", (0, 0))[0]
    dd_calls = timers.get("dd_update", (0, 1))[1]
    L = pkg.engine.load()
    import ctypes

    pk = ctypes.c_double()
    L.pimd_peak_flops(local, 0, ctypes.byref(pk))
    peak32 = pk.value
    L.pimd_peak_flops(local, 1, ctypes.byref(pk))
    peak64 = pk.value
    ach = flops_ewald_dd(rese["nk"], rese["nw"], rese["P"]) * dd_calls / (dd_ms / 1000.0) / 1e12 if dd_ms else None
    tach = tensor_flops_dd(12, rese["nw"], rese["P"]) * dd_calls / (dd_ms / 1000.0) / 1e12 if dd_ms else None
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak_tc = peaks.get("bf16_tflops", 1900.0)
    t64 = res64["timers"]
    dd64_ms = t64.get("dd_smu", (0, 0))[0] + t64.get("dd_update", (0, 0))[0]
    ach64 = flops_ewald_dd(res64["nk"], res64["nw"], res64["P"]) * t64.get("dd_update", (0, 1))[1] / (dd64_ms / 1e3) / 1e12
    fp64_value = steps64 * world / (res64["dev_ms"] / 1000.0)
    cpu = None
    if not args.no_cpu_baseline:
        orc = ge.load_oracle()
        orc.build()
        r = cpu_baseline(pkg, orc, args.cpu_steps + 1)
        cpu = dict(value=r["value"], unit="steps/s", cores=r["cores"], kind="port",
                   sample="%d MD steps of 512 H2O x 32 beads on the host cores (first step excluded)" % args.cpu_steps)
    line = dict(
        metric=METRIC, value=value, unit="steps/s", n_gpus=world, steps=args.steps, warmup=args.warmup,
        ms_per_step=ms_per_step, higher_is_better=True, scaling="weak", vs_baseline=None,
        dtype="f32 pair/phase arithmetic, f64 accumulation, f64 integrator",
        data="synthetic (seeded jittered-lattice water boxes with free ring-polymer beads)",
        config=dict(workload=CONFIG + " (TTM3-F, 512 H2O x 32 beads, L=24.86 A, Rc=9 A, |n|<=12, %d k-vectors)" % res["nk"],
                    precision="mixed", polar_eps=POLAR["polar_eps"], predictor=True, dt_fs=DT_FS,
                    l2="256 MB buffer written between timed steps", parallelism="replicas" if world > 1 else "1 GPU",
                    execution="one CUDA graph per MD step (dipole loop as a conditional while node)",
                    tensor_core_structure_factor=bool(res["tuning"]["sf_tc"]),
                    tensor_core_field_pass=bool(res["tuning"]["ff_tc"]),
                    dipole_iterations_mean=float(np.mean(res["niters"])),
                    fp64_dipole_iterations_mean=float(np.mean(res64["niters"]))),
        fp64=dict(value=fp64_value, steps=steps64, ms_per_step=res64["dev_ms"] / steps64,
                  e2e=res64["e2e_steps"] / res64["e2e_s"],
                  phases_ms={k: round(v[0] / steps64, 4) for k, v in sorted(t64.items(), key=lambda kv: -kv[1][0])},
                  roofline=dict(kernel="ewald_std_dd", bound="fp64-pipe", achieved=ach64, peak=peak64,
                                unit="TFLOP/s", frac=ach64 / peak64)),
        mixed_eager=dict(value=eager_value, ms_per_step=rese["dev_ms"] / args.steps,
                         e2e=rese["e2e_steps"] / rese["e2e_s"], gpu_launches=rese["launches"]),
        mixed_over_fp64=value / fp64_value,
        accuracy=ferr,
        e2e=dict(value=res["e2e_steps"] / res["e2e_s"], unit="steps/s", h2d_bytes_per_step=res["h2d"],
                 d2h_bytes_per_step=res["d2h"]),
        roofline=dict(kernel="ewald_std_dd (k_sfac_tc + k_field_tc)", bound="tensor",
                      achieved=ach, peak=peak_tc, unit="TFLOP/s", frac=(ach / peak_tc) if ach else None,
                      traffic=DD_TRAFFIC_BYTES, traffic_unit="bytes per call",
                      achieved_meaning="algorithmic: 22 flops per (k-vector, dipole site) per call (ewald.f90:56-119)",
                      peak_source="MEASURED_PEAKS.json bf16_tflops (burst; FP16 inputs run at the bf16 rate)",
                      executed_tensor_tflops=tach, executed_tensor_frac=(tach / peak_tc) if tach else None,
                      fp32_equivalent_frac=(ach / peak32) if ach else None, fp32_peak=peak32),
        cpu_baseline=cpu,
        clocks=res["clocks"],
        gpu_launches=rese["launches"],
        graph_launches=res["graph_launches"],
        phases_ms={k: round(v[0] / args.steps, 4) for k, v in phases},
        phase_calls={k: v[1] for k, v in phases},
        dominant_phase=phases[0][0] if phases else None,
        energy=dict(Upot=res["out"][0], virial=res["out"][1], virialc=res["out"][2], uk=res["out"][3]),
    )
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
