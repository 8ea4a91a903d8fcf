/*
 * pimd_gb300.h -- C ABI of the GB300 force engine and ring-polymer propagator.
 *
 * Drop-in boundary for PIMD-F90's hot path. Every entry point takes plain pointers and
 * sizes, returns an int status (PIMD_OK on success) and never aborts the process; the
 * reference's Fortran `stop`s (math.f90:199,229,244,282) become error codes.
 *
 * Array layouts are the reference's Fortran column-major layouts, passed as double*:
 *   RR(3,Natoms), RRt(3,Natoms,Nbeads), dRR(3,Natoms), virt(3,3), dip_momI(3,Nwaters),
 * with atoms ordered O H H O H H ... Units: Angstrom, kcal/mol, amu, ps. dRR is the
 * gradient dE/dx (not the force), as in the reference.
 *
 * A context replaces the reference's module state (system_mod.f90:22-44, pot_mod.f90:47-83):
 * it owns all device memory, the Ewald tables and one induced-dipole predictor history per
 * bead. Calls on one context must not overlap; different contexts are independent.
 */
#ifndef PIMD_GB300_H
#define PIMD_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PIMD_OK = 0,
    PIMD_ERR_ARG = 1,               /* invalid argument / unsupported combination         */
    PIMD_ERR_CUDA = 2,              /* CUDA runtime error (see pimd_last_error)           */
    PIMD_ERR_NEIGHBOR_OVERFLOW = 3, /* more O-O pairs than the neighbour-list capacity     */
    PIMD_ERR_GAMMQ = 4,             /* Thole Q(2/3,x) iteration did not converge          */
    PIMD_ERR_NOMEM = 5,             /* device allocation failed                            */
    PIMD_ERR_STATE = 6              /* call order violated (e.g. no normal modes set up)   */
};

enum { PIMD_FP64 = 0, PIMD_MIXED = 1 };

/* Potential parameters: the input-file keys of input_file_reader.f90 that reach the
 * force call, plus two explicit Ewald settings. With alpha > 0 the Ewald splitting
 * parameter and the integer k shell |n|^2 <= nmax^2 are used as given; with alpha <= 0 the
 * reference rule of ewald.f90:312-319 is applied to eps_ewald. */
typedef struct {
    int pot_model;      /* 2 TTM2.1-F, 3 TTM3-F, 4 q-SPC/Fw, 5 SPC/F                       */
    int natoms;         /* 3 * Nwaters                                                     */
    int nbeads;         /* beads evaluated per batched call (>= 1)                         */
    double box[3];      /* orthorhombic box (A)                                            */
    double rc;          /* real-space cutoff (A), <= min(box)/2                            */
    double rc1;         /* start of the TTM3-F vdW force switch (A)                        */
    double eps_ewald;   /* ewald.f90 accuracy parameter (used when alpha <= 0)             */
    double alpha;       /* explicit Ewald alpha (1/A), or <= 0                             */
    int nmax;           /* explicit k shell, used when alpha > 0                           */
    int polar_maxiter;  /* induced-dipole iteration cap                                    */
    double polar_sor;   /* SOR mixing factor                                               */
    double polar_eps;   /* convergence threshold on DEBYE/CHARGECON/sqrt(Natoms)*|dmu|     */
    int guess_initdip;  /* 4-step dipole predictor from the previous MD steps              */
    int contraction;    /* skip the monomer PES (ring-polymer contraction runs)            */
    int precision;      /* PIMD_FP64 or PIMD_MIXED                                         */
    int device;         /* CUDA device ordinal                                             */
} pimd_params;

typedef struct pimd_ctx pimd_ctx;

/* init_pot (pot_ttm/potential.f90:43-199) + ewald_set(.true.) (pot_ttm/ewald.f90:293). */
int pimd_create(pimd_ctx **ctx, const pimd_params *p);
int pimd_destroy(pimd_ctx *ctx);
/* Run all work of the context on this cudaStream_t (NULL = the context's own stream). */
int pimd_set_stream(pimd_ctx *ctx, void *cuda_stream);
/* Text of the last error on this context. */
const char *pimd_last_error(pimd_ctx *ctx);
/* Ewald set-up results: alpha, number of half-space k-vectors, (hmax, kmax, lmax). */
int pimd_ewald_info(pimd_ctx *ctx, double *alpha, int *nk, int *hkl_max);

/* pot_ttm (pot_ttm/pot_ttm.f90:3): one bead, host arrays, same argument order. Uses the
 * predictor-history slot of bead 0. Blocks until the results are in host memory. */
int pimd_pot_ttm(pimd_ctx *ctx, const double *RR, const double *RRc, double *En, double *dRR,
                 double *virt, double *virialc, double *dip_momI, double *Edip_mom, double *chg,
                 int t);

/* pot_spc (pot_ttm/pot_spc.f90:1): one bead, host arrays. */
int pimd_pot_spc(pimd_ctx *ctx, const double *RR, double *En, double *dRR, double *virt,
                 double *dip_momI, double *chg);

/* The body of full_bead_forces (force_calc.f90:26-106) for all nbeads beads in one call,
 * host arrays: RRt(3,Natoms,P), RRc(3,Natoms) in; Upott(P), dRRt(3,Natoms,P), virialt(P),
 * virialct(P), dip_momIt(3,Nw,P), dip_momEt(3,Nw,P) and chg(Natoms) (bead P) out. Any
 * output pointer may be NULL. virialt(k) = trace of bead k's virial tensor. */
int pimd_full_bead_forces(pimd_ctx *ctx, const double *RRt, const double *RRc, double *Upott,
                          double *dRRt, double *virialt, double *virialct, double *dip_momIt,
                          double *dip_momEt, double *chg, int t);

/* Same with device pointers, stream-ordered on the context's stream (no host copies). */
int pimd_full_bead_forces_device(pimd_ctx *ctx, const double *RRt, const double *RRc,
                                 double *Upott, double *dRRt, double *virialt, double *virialct,
                                 double *dip_momIt, double *dip_momEt, double *chg, int t);

/* Energy components of bead `bead` after the last force call (the reference's globals
 * Umon, Uvdw, Uelec, Uind of system_mod.f90:30), the per-bead 3x3 virial tensor and the
 * induced-dipole iteration count / final stath*|dmu|. */
int pimd_get_energies(pimd_ctx *ctx, int bead, double U[4]);
int pimd_get_virial(pimd_ctx *ctx, int bead, double virt[9]);
int pimd_get_dipole_info(pimd_ctx *ctx, int bead, int *niter, double *deltadip);

/* The half neighbour list of bead `bead` from the last force call: O-O pairs (i, j), 0-based,
 * i < j, in find_neigh's order (find_neigh.f90:75-117). Writes min(npairs, cap) pairs to
 * ij[2*cap] and the total to *npairs. */
int pimd_get_neighbors(pimd_ctx *ctx, int bead, int *ij, int cap, int *npairs);

/* Named phase timers (the reference's dans_timer.f90 start_timer/stop_timer/
 * print_timing_report), kept as CUDA events on the context's stream. reset clears the
 * totals and switches recording on (enable != 0) or off. get returns the number of timers
 * and, for 0 <= i < that number, timer i's name, total milliseconds and call count. */
int pimd_timers_reset(pimd_ctx *ctx, int enable);
/* Number of CUDA kernels this context has launched so far. */
long long pimd_launch_count(pimd_ctx *ctx);
int pimd_timers_get(pimd_ctx *ctx, int i, char *name, int namelen, double *ms, long long *count);

/* Induced-dipole iteration control for batched calls: check convergence on the host every
 * `every` iterations (0 = run exactly polar_maxiter iterations with converged beads
 * skipped on the device, which needs no host synchronisation). Default 1. */
int pimd_set_dipole_check(pimd_ctx *ctx, int every);

/* ---------------------------------------------------------------------------------------
 * Ring-polymer normal modes (NormalModes.f90) and PILE thermostat (Langevin.f90).
 */
/* InitNormalModes (NormalModes.f90:68-218) for P beads; optional outputs (NULL to skip):
 * A11..A22, omegalist, MassScaleFactor (length P) and C(P,P) column-major. */
int pimd_nm_init(pimd_ctx *ctx, int nbeads, double omegan, double delta, double setNMfreq,
                 double *A11, double *A12, double *A21, double *A22, double *omegalist,
                 double *msf, double *C);
/* real2NM and NM2real (NormalModes.f90:308-341) for one atom with the context's C: A(3,P) in,
 * out(3,P) (host arrays, may not alias). */
int pimd_real2nm(pimd_ctx *ctx, const double *A, double *out, int nbeads);
int pimd_nm2real(pimd_ctx *ctx, const double *A, double *out, int nbeads);
/* gen_rand_ring and gen_rand_ring_momenta (NormalModes.f90:224-275) for one atom, host RR(3,P) /
 * PP(3,P) out, with the normal-mode frequencies and mass scale factors of pimd_nm_init. xi(3,P)
 * holds the standard normal draws (the reference's rand_norm with unit deviation); NULL draws them
 * from the context's own host generator (splitmix64, Box-Muller; the reference's Fortran
 * random_number stream is not reproduced). gen_rand_ring takes the physical temperature;
 * gen_rand_ring_momenta the temperature its caller passes (temp*Nbeads, main_stuff.f90:306). */
int pimd_gen_rand_ring(pimd_ctx *ctx, double *RR, double mass, double temp, int nbeads,
                       const double *xi);
int pimd_gen_rand_ring_momenta(pimd_ctx *ctx, double *PP, double mass, double temp, int nbeads,
                               const double *xi);
/* EvolveRing (NormalModes.f90:34-63) for one atom, host arrays RR(3,P), PP(3,P) inout. */
int pimd_evolve_ring(pimd_ctx *ctx, double *RR, double *PP, int nbeads, double mass);
/* EvolveRing for every atom of RRt(3,Natoms,P)/PPt (MD.f90:53-58); device pointers. */
int pimd_evolve_all_device(pimd_ctx *ctx, double *RRt, double *PPt, double massO, double massH);
/* Init_Langevin_NM (Langevin.f90:68-98) after pimd_nm_init; temp_P = P * T. */
int pimd_langevin_init(pimd_ctx *ctx, double delt2, int centroid_thermostat, double tau_centroid,
                       double temp_P);
/* Langevin_NM (Langevin.f90:30-64) on device PPt(3,Natoms,P). xi(3,P,Natoms) holds the
 * standard normal draws (device pointer); NULL draws them on the device from (seed, counter)
 * with a counter-based generator. */
int pimd_langevin_nm_device(pimd_ctx *ctx, double *PPt, const double *xi, double massO,
                            double massH, unsigned long long seed, unsigned long long counter);

/* One velocity-Verlet PIMD step (MD.f90:35-110, PIMD_VV without Nose-Hoover/barostat) on
 * device state RRt, PPt, dRRt (3,Natoms,P) and RRc (3,Natoms): Langevin, half kick,
 * EvolveRing, centroid, PBCs (main_stuff.f90:107-125), full_bead_forces, half kick,
 * Langevin. Writes the bead-summed Upot, virial, virialc/P and the kinetic energy uk
 * (main_stuff.f90:349-388) to device out4[4]. xi1/xi2 as in pimd_langevin_nm_device. */
typedef struct {
    double delt;                 /* ps */
    double massO, massH;         /* amu */
    int langevin;                /* PILE bead thermostat on/off */
    unsigned long long seed;     /* Langevin stream seed when xi == NULL */
} pimd_md_params;
int pimd_md_step_device(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt,
                        double *dRRt, double *RRc, const double *xi1, const double *xi2, int t,
                        double *out4);
/* The same step on host arrays (copied in and out every call): RRt, PPt, dRRt inout
 * (3,Natoms,P), RRc out (3,Natoms), out4 host [Upot, virial, virialc, uk]; xi1/xi2 host
 * standard normals (3,P,Natoms) or NULL for the device generator. */
int pimd_md_step(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt,
                 double *RRc, const double *xi1, const double *xi2, int t, double *out4);

/* Thermostats of the MD step beyond PILE (main_stuff.f90:132-188, MD.f90:41-46, 96-104), after
 * pimd_nm_init: bead_thermostat 2 runs one chain-2 Nose-Hoover thermostat (Nose_Hoover.f90:33-112,
 * L = 1, Nbeads*temp) per (atom, normal mode k >= 2, component) with tau = 1/omega_k, and on the
 * centroid mode too with centroid_thermostat (tau_centroid), before the first and after the second
 * half kick (pimd_md_params.langevin must then be 0); bead_thermostat 0 leaves the bead thermostat
 * to pimd_md_params.langevin. global_thermostat adds the global chain (THERMOSTAT: L = 3 Natoms
 * Nbeads, temp*Nbeads, tau) on the module variable uk at the start and the end of the step, each
 * followed by PPt = s PPt. Chain velocities start as the reference sets them (vxi_global = 1,
 * vxi_beads = 0, InputOutput.f90:395-404) and uk at 0: set the initial uk with
 * pimd_set_thermostat_state (the reference's initialize_velocities leaves calc_uk_centroid there).
 * The chains and the thermostats' kinetic energies run in the exact FP64 integrator kernels in
 * both engines. */
typedef struct {
    int bead_thermostat;     /* 0 (PILE / none, per pimd_md_params.langevin) or 2 (Nose-Hoover) */
    int global_thermostat;   /* != 0: the global chain                                         */
    double tau;              /* global chain time constant (ps)                                 */
    double temp;             /* K; the chains couple to Nbeads*temp                             */
    int centroid_thermostat; /* bead chains on the centroid mode as well                        */
    double tau_centroid;     /* ps                                                              */
} pimd_thermostat;
int pimd_set_thermostat(pimd_ctx *ctx, const pimd_thermostat *th);
/* Chain state for checkpoints (the reference's save_checkpoint / load_checkpoint records):
 * vxi_global[2], the module variable uk, and vxi_beads(2,Natoms,Nbeads,3) (NULL to skip; needs
 * bead_thermostat 2). Blocking. */
int pimd_get_thermostat_state(pimd_ctx *ctx, double *vxi_global, double *uk, double *vxi_beads);
int pimd_set_thermostat_state(pimd_ctx *ctx, const double *vxi_global, double uk,
                              const double *vxi_beads);
/* The MD step with the quantities write_out takes from it (InputOutput.f90:566-571,
 * estimators.f90:30-96), computed on the device: out[PIMD_MD_NOUT] = {Upot, virial, virialc, uk
 * (the module variable after the step), calc_uk after the force call, K0 = sum m (r_k -
 * r_(k-1))^2 (amu A^2), sys_temp (K), quantum-virial energy (kcal/mol per molecule) and pressure
 * (bar), simple-estimator energy and pressure, the global chain's last scale factor s}. Device
 * variant: out is a device pointer, stream-ordered (no host synchronisation); host variant: as
 * pimd_md_step with out on the host. Works with pimd_set_graph like pimd_md_step_device. */
enum { PIMD_MD_NOUT = 12 };
int pimd_md_step_ex_device(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt,
                           double *dRRt, double *RRc, const double *xi1, const double *xi2, int t,
                           double *out);
int pimd_md_step_ex(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt,
                    double *RRc, const double *xi1, const double *xi2, int t, double *out);

/* Ring-polymer contraction with multiple time steps (contracted_MD, MD.f90:276-449; mode 0) and
 * monomer PIMD (monomer_PIMD, MD.f90:117-265; mode 1), TTM models: the NASA monomer PES acts on
 * every bead, the intermolecular potential on the centroid alone (a one-bead context made by
 * pimd_contracted_init with the context's parameters; contraction set in mode 0, so its pot_ttm
 * skips the monomer PES, and unset in mode 1, which keeps it at the centroid as the reference
 * does). Mode 0 runs intra_timesteps inner steps of fast kicks and EvolveRing per step: make the
 * normal modes with pimd_nm_init(delta = delt / intra_timesteps) first (InputOutput.f90:382-386),
 * and for mode 1 with delta = delt. Thermostats as pimd_md_step (PILE, the bead and global
 * chains). */
int pimd_contracted_init(pimd_ctx *ctx, int mode, int intra_timesteps);
/* One step: RRt, PPt, dRRt (3,Natoms,P) inout, dRRfast (3,Natoms,P) inout in mode 0 (the
 * reference's saved fast gradient; zero before the first step; unused in mode 1), RRc out,
 * out[PIMD_MD_NOUT] as pimd_md_step_ex with Upot = sum of the beads' monomer energies + P times
 * the centroid's potential, virial = monomer virial + the centroid's, virialc = monomer centroid
 * virial / P + the centroid's; dip_momIt / dip_momEt (3,Nw,P) (may be NULL) as
 * calc_monomer_dip_moments (force_calc.f90:205-264) plus the centroid's induced dipoles. Device
 * variant: device pointers, stream-ordered; host variant: host arrays, blocking. */
int pimd_contracted_step_device(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt,
                                double *dRRt, double *dRRfast, double *RRc, const double *xi1,
                                const double *xi2, int t, double *out, double *dip_momIt,
                                double *dip_momEt);
int pimd_contracted_step(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt,
                         double *dRRt, double *dRRfast, double *RRc, const double *xi1,
                         const double *xi2, int t, double *out, double *dip_momIt, double *dip_momEt);

/* Exact restart (no counterpart in the reference, whose .img image keeps 6 decimals and no
 * predictor history): writes the MD state RRt, PPt, dRRt (3,Natoms,P) host arrays, the step
 * index t of the last completed step, the Langevin seed, and the context state the next steps read
 * -- each bead's dipole-predictor history and the Nose-Hoover chain state -- to a little-endian
 * binary file; reading it into a context made with the same pimd_params (and thermostats) and
 * continuing from step t + 1 reproduces the uninterrupted run. PIMD_ERR_ARG when the file's
 * system (atoms, beads, model) or thermostats differ from the context's. Blocking. */
int pimd_checkpoint_write(pimd_ctx *ctx, const char *path, const double *RRt, const double *PPt,
                          const double *dRRt, int t, unsigned long long seed);
int pimd_checkpoint_read(pimd_ctx *ctx, const char *path, double *RRt, double *PPt, double *dRRt,
                         int *t, unsigned long long *seed);

/* CUDA-graph execution of pimd_md_step_device / pimd_md_step (enable != 0). The whole step --
 * Langevin, kicks, EvolveRing, PBCs and the force call -- is captured on its first call and
 * replayed on later calls with the same buffers and parameters (a change of any pointer or
 * md parameter re-captures). The induced-dipole iterations run inside the graph as a
 * conditional while node: the device tests convergence after each iteration and stops at the
 * same iteration as the host loop, without returning to the host. The MD step index t is
 * written to the device before each launch, so the predictor and the Langevin stream follow t
 * exactly as in the eager path. Phase timers then report the step as one phase ("md_graph").
 * No counterpart in the reference (MD.f90:35-110 is a host loop). */
int pimd_set_graph(pimd_ctx *ctx, int enable);
/* Number of graph captures and graph launches made by this context so far. */
int pimd_graph_info(pimd_ctx *ctx, long long *captures, long long *launches);

/* ---------------------------------------------------------------------------------------
 * Differentiation form (TTM3-F, FP64 contexts). Model parameters theta, in this order, with the
 * published TTM3-F values (pot_mod.f90:16-24) and NASA PES scale factors (nasa_mod.f90) as
 * defaults: */
enum {
    PIMD_TH_POLAR_M = 0, /* polarisability of the M site (A^3)                          */
    PIMD_TH_A_DD,        /* Thole damping, dipole-dipole                                 */
    PIMD_TH_A_CC,        /* Thole damping, charge-charge and charge-dipole               */
    PIMD_TH_VDW_C,       /* O-O C6 (C/r^6)                                               */
    PIMD_TH_VDW_D,       /* O-O Born-Mayer prefactor (D exp(-E r))                       */
    PIMD_TH_VDW_E,       /* O-O Born-Mayer exponent                                      */
    PIMD_TH_DMS1,        /* TTM3-F charge corrections dms_param1..3 (nasa.f90:234-242)   */
    PIMD_TH_DMS2,
    PIMD_TH_DMS3,
    PIMD_TH_GAMMA_M,     /* M-site placement / charge redistribution gamma               */
    PIMD_TH_F5Z,         /* NASA PES scale factors f5z, fbasis, fcore, frest             */
    PIMD_TH_FBASIS,
    PIMD_TH_FCORE,
    PIMD_TH_FREST,
    PIMD_NTHETA
};
int pimd_get_theta(pimd_ctx *ctx, double *theta);
int pimd_set_theta(pimd_ctx *ctx, const double *theta);
/* Forward: the force call of pimd_full_bead_forces (host arrays) that also records every
 * induced-dipole iteration for the backward. TTM3-F contexts of either precision. Needs the
 * dipole predictor off at this step (guess_initdip = 0 or t <= 4). No counterpart in the
 * reference. */
int pimd_pot_forward(pimd_ctx *ctx, const double *RRt, const double *RRc, double *Upott, int t);
/* Backward: for E = sum_k Ebar[k] Upot_k of the last forward, the exact derivative of the
 * computed energies -- the induced dipoles as the forward computed them, after its own number of
 * Jacobi-SOR iterations per bead, differentiated through those iterations by the transposed
 * (adjoint) iteration, which reuses the symmetric dipole-field operator -- with respect to the
 * positions, dRRt(3,Natoms,P), and to theta, dtheta[PIMD_NTHETA]. Pair geometry is recomputed,
 * not stored. A mixed context runs the backward with the forward's FP32 operators (FP32 pair,
 * table and reciprocal products, FP64 sums): the gradients agree with an FP64 context's within
 * the mixed force budget (~1e-6 relative on water boxes). No counterpart in the reference. */
int pimd_pot_backward(pimd_ctx *ctx, const double *Ebar, double *dRRt, double *dtheta);

/* ---------------------------------------------------------------------------------------
 * Tile-shape autotuner. Times force calls of this context on its current positions (device
 * RRt(3,Natoms,P) and RRc(3,Natoms) if given, else the last ones it was called with) for
 * candidate launch shapes -- tensor-core vs. FP32-pipe dipole structure factors, site groups of
 * the structure-factor kernels, k-slices of the field passes, register-tiled vs. generic Ewald
 * kernels, one-launch vs. three-launch neighbour lists
 * -- by coordinate descent, and keeps the fastest. Results change only by FP32 summation order.
 * Call before MD starts (it overwrites the dipole predictor history) and before graph capture.
 * No counterpart in the reference. */
int pimd_autotune(pimd_ctx *ctx, const double *RRt, const double *RRc);
/* The chosen shapes: [tiled structure factors, site groups (0 = sized from the SM count),
 * register-row field kernels, max k-slices, one-launch neighbour lists] and, when n >= 6,
 * [wave-quantised split counts], when n >= 7 [tensor-core (tcgen05) dipole structure factor
 * in use], when n >= 8 [tensor-core dipole field pass in use], when n >= 9 [real-space dipole
 * field on a second stream beside the structure factor (mixed engine)], when n >= 10 [the
 * dipole iterations' structure factor reuses its position-only operand from the first
 * iteration], when n >= 11 [the iterations' field pass is a programmatic dependent launch of
 * the structure factor (its set-up overlaps that grid's end)], when n >= 12 [dipole iterations
 * per body of the CUDA graph's conditional loop, 1-4], when n >= 13 [the reciprocal charge and
 * force passes on a second stream beside the pair kernels (mixed engine)], when n >= 14
 * [real-space dipole tensors formed inside each iteration rather than cached per list entry
 * (mixed engine)], when n >= 15 [tensor-core force pass in use (follows the field-pass knob;
 * reported only)], when n >= 16 [the iterations' cached operands loaded evict-last in L2], when
 * n >= 17 [the real-space dipole field beside the field pass too, each unit of 128 dipole
 * sites updated by whichever of the two finishes it last (mixed engine, TTM3-F)], when n >= 18
 * [at the start of each graph-loop body the real-space dipole field waits until every CTA of
 * the structure factor is resident (a programmatic event), mixed engine], when n >= 19 [the
 * iterations' field pass may start as the real-space dipole field drains (a programmatic
 * event; it waits for that grid before reading its output), mixed engine], when n >= 20 [the
 * neighbour lists built from the input positions on the second stream beside the monomer
 * kernel, mixed engine]; n >= 5. */
int pimd_get_tuning(pimd_ctx *ctx, int *knobs, int n);
/* Sets the shapes in the order pimd_get_tuning reports them (n >= 5; entry 15, the tensor-core
 * force pass, is a report only), e.g. to reuse an earlier autotune result without timing
 * again. Tensor-core paths are used only where available whatever their knob says. Site groups
 * must lie in [0, 1024] and max k-slices in [1, 16], iterations per graph-loop body in [1, 4]
 * (else PIMD_ERR_ARG). A captured MD-step graph is captured again at the next step. No
 * counterpart in the reference. */
int pimd_set_tuning(pimd_ctx *ctx, const int *knobs, int n);

/* ---------------------------------------------------------------------------------------
 * Batches of independent ring polymers (replicas) of uneven sizes: each replica has its own
 * molecule count, bead count, box and temperature (the reference runs one per job). Replicas
 * sharing a box are stacked on the bead axis of one engine, so each force kernel covers all of
 * them in one launch; the whole PIMD_VV step of the batch (MD.f90:35-110, PILE thermostat with
 * the device generator, seed = md.seed + replica index) is one CUDA graph with one branch per
 * box. Cutoff per replica: min(common.rc, half its smallest box edge); rc1 scales with it;
 * Ewald by common.eps_ewald (common.alpha <= 0) or the explicit alpha/nmax. No counterpart in
 * the reference. */
typedef struct {
    int natoms;      /* 3 * Nwaters */
    int nbeads;      /* 1..64 */
    double box[3];   /* A */
    double temp;     /* K: normal-mode frequencies and thermostat */
} pimd_replica;
typedef struct pimd_batch pimd_batch;
int pimd_batch_create(pimd_batch **bt, const pimd_params *common, const pimd_replica *reps, int nrep,
                      const pimd_md_params *md);
int pimd_batch_destroy(pimd_batch *bt);
const char *pimd_batch_last_error(pimd_batch *bt);
/* number of box groups and the group of each replica (group_of_replica[nrep], may be NULL) */
int pimd_batch_info(pimd_batch *bt, int *ngroups, int *group_of_replica);
/* host arrays RRt, PPt (3,Natoms,P) of replica r; the centroid is computed from RRt */
int pimd_batch_set_state(pimd_batch *bt, int r, const double *RRt, const double *PPt);
/* host copies of replica r's state; out4 = [Upot, virial, virialc, uk] of its last step */
int pimd_batch_get_state(pimd_batch *bt, int r, double *RRt, double *PPt, double *dRRt, double *out4);
/* gradients of the current positions of every replica (call once before the first step) */
int pimd_batch_forces(pimd_batch *bt);
/* pimd_autotune for every box group (before the first pimd_batch_step) */
int pimd_batch_autotune(pimd_batch *bt);
/* nsteps steps of every replica; stream-ordered, returns without waiting */
int pimd_batch_step(pimd_batch *bt, int nsteps);
int pimd_batch_sync(pimd_batch *bt);

/* ---------------------------------------------------------------------------------------
 * Configuration and checkpoint files (InputOutput.f90), host only: no context, no device work.
 * Arrays as elsewhere: RRc(3,Natoms), RRt/PPt(3,Natoms,Nbeads) column-major, atoms O H H ...
 */
/* Header of a configuration file (read_and_initialize_all_nodes, InputOutput.f90:67-116).
 * ".img": '(2i10)' Natoms, Nbeads and '(f12.6,2x,f12.6,3(1x,f12.6))' time, box. ".xyz": box and
 * atom count as a box record then the count, the count then a box record, or the count and the
 * box on one record (*nbeads = 0, *time = 0). nbeads and time may be NULL. PIMD_ERR_ARG for a
 * missing file, another suffix, or a malformed header. */
int pimd_read_config_header(const char *path, int *natoms, int *nbeads, double *time, double *box);
/* The coordinate records of an ".xyz" file (read_coords_and_init, InputOutput.f90:422-446):
 * read_method 0 (all O, then the H pairs) or 1 (O H H ...); with read_method 1 the coordinates
 * are shifted by their mean, as the reference does. natoms must equal the header's. */
int pimd_read_xyz(const char *path, int read_method, int natoms, double *RRc);
/* save_XYZ (InputOutput.f90:948-981): one frame, '(i10)' Natoms, a blank record, then
 * '(a2,3(1x,f12.6))' per atom; append != 0 adds it to the end of the file. */
int pimd_write_xyz(const char *path, int append, int natoms, const double *RR);
/* save_checkpoint (InputOutput.f90:987-1024): the ".img" image of the ring polymers (velocities
 * PPt/mass written), then, if n_vxi_beads != 0, the bead Nose-Hoover chain velocities
 * vxi_beads(2,Natoms,Nbeads,3) (n_vxi_beads = 6 Natoms Nbeads), and, if n_vxi_global != 0, the
 * global chain velocities; time = t*delt + init_time. */
int pimd_save_image(const char *path, int natoms, int nbeads, double time, const double *box,
                    const double *RRt, const double *PPt, double massO, double massH,
                    const double *vxi_beads, int n_vxi_beads, const double *vxi_global,
                    int n_vxi_global);
/* load_checkpoint with its header (InputOutput.f90:86-96, 1030-1074): RRt, PPt (velocities times
 * the masses), the chain velocities when asked for, then the centroid RRc (may be NULL) and the
 * centroid-following PBC shift of main_stuff.f90:107-125. Natoms and Nbeads must match the
 * header's (else PIMD_ERR_ARG, as the reference's abort at InputOutput.f90:90-94). */
int pimd_load_image(const char *path, int natoms, int nbeads, double massO, double massH,
                    double *time, double *box, double *RRt, double *PPt, double *RRc,
                    double *vxi_beads, int n_vxi_beads, double *vxi_global, int n_vxi_global);

/* ---------------------------------------------------------------------------------------
 * Run analyses on the device (the reference's geometry_calculator.f90, diffusion_calculator.f90,
 * spectral_properties.f90 with math.f90:42-140). Accumulating calls take device arrays of the
 * context's system and are stream-ordered on its stream; reports are blocking.
 */
/* calc_geometry (geometry_calculator.f90:21-125) of one frame: centroid RRc(3,Natoms) and beads
 * RRt(3,Natoms,P). reset clears the accumulator (allocates it on the first call). */
int pimd_geometry_reset(pimd_ctx *ctx);
int pimd_geometry_accumulate_device(pimd_ctx *ctx, const double *RRc, const double *RRt);
/* write_out_geometry (:129-190): out[14] = average and RMS of the H-H distance, the O-H distance
 * and the H-O-H angle (A, degrees) over the centroids, the same over the beads, then the largest
 * centroid and bead O-H distances (the centroid one updated as the reference's lines 57-58 do).
 * hist_c / hist_b [80][2] (may be NULL): write_out_histogram's (bin end, count / (2 num_total
 * [Nbeads])); counts[176] (may be NULL): the raw accumulator, the reference's module variables
 * in the order sum_HH, sum_OH, sum_HOH, their squares, the bead sums, max_OH, bmax_OH,
 * num_total, warnings (O-H > 1.5 A), dOHhist(80), bdOHhist(80). */
int pimd_geometry_report(pimd_ctx *ctx, double *out, double *hist_c, double *hist_b, double *counts);
/* calc_diff_RMSD (diffusion_calculator.f90:14-58) of a run of num_timesteps frames: the mean
 * square displacement every 20 frames of atom 3i (1-based) of each molecule, as the reference
 * tracks it, from the centroids RRc(3,Natoms). */
int pimd_msd_init(pimd_ctx *ctx, int num_timesteps);
int pimd_msd_accumulate_device(pimd_ctx *ctx, const double *RRc);
/* write_out_diffusion (:60-118): aMS[ntimes] (may be NULL), *ntimes (may be NULL) and out4 =
 * {D, errD (10^-5 cm^2/s), slope, intercept} of the fit to the last half; timestep in ps. */
int pimd_msd_report(pimd_ctx *ctx, double timestep, double *aMS, int *ntimes, double *out4);
/* The spectra's time series (InputOutput.f90:680-688): per frame the total dipole in Debye from
 * dip_momIt(3,Nw,P) (write_out's dip_mom) and the centroid velocities of the atoms the reference
 * stores as "H" velocities (the first H and the O of each molecule, momenta over massH); either
 * pointer may be NULL. init sets the capacity (frames) and clears the series. */
int pimd_spectra_init(pimd_ctx *ctx, int max_steps, double massH);
int pimd_spectra_record_device(pimd_ctx *ctx, const double *dip_momIt, const double *PPt);
/* calc_infrared_spectrum (spectral_properties.f90:10-123) and calc_DOS (:128-187) of the series
 * recorded so far, with the transforms by cuFFT in single precision; timestep in ps, temp in K.
 * *npoints in: the reference's NumPointsOut (350 at the start of a run), out: the points written
 * to freq (cm^-1) and ir / dos. The IR series is zero-padded where the reference's work array is
 * left uninitialised. */
int pimd_ir_spectrum(pimd_ctx *ctx, double timestep, double temp, int *npoints, double *freq, double *ir);
int pimd_dos(pimd_ctx *ctx, double timestep, int *npoints, double *freq, double *dos);

/* O-O half neighbour list of one bead without any device allocation. No counterpart in the
 * reference; it serves callers that must not let a library allocate device memory (drivers
 * that own all GPU memory through their own pool, applications with a fixed per-GPU budget,
 * code recording CUDA graphs, where cudaMalloc is not a stream operation).
 * In (device): RR(3,Natoms) of one bead, atoms O H H ...; box[3] and rc on the host.
 * Out (device): ij[2*cap] int pairs (i, j), 0-based, i < j, in find_neigh's order, bit-identical
 * to pimd_get_neighbors; *npairs (device int) = total pairs found, which may exceed cap (then
 * only the first cap pairs are written). Stream-ordered on cuda_stream (NULL = default stream);
 * allocates nothing and does not synchronise.
 * Limit: Natoms/3 <= 16384 molecules; larger inputs, and a box edge that is not a finite
 * positive length, return PIMD_ERR_ARG with a message. cuda_stream must belong to the current
 * device (else PIMD_ERR_ARG). Cost: an all-pairs FP64 test run twice (count, then fill), one
 * thread per molecule: about 1.3e8 distance tests per pass at the 16384-molecule limit, far
 * slower than the context's neighbour step, which it is not meant to replace.
 * Its per-molecule counts and offsets live in one fixed 128 KB device array per GPU that is
 * shared by every call and fully rewritten by each call; calls that overlap on the GPU (two
 * streams, or two host threads) race on it. The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) and should come before any stream capture. */
int pimd_neighbors_noalloc(const double *RR, int natoms, const double *box, double rc, int *ij,
                           int cap, int *npairs, void *cuda_stream);

/* Measured CUDA-core FMA throughput of `device` in TFLOP/s (fp64 != 0: double, else float):
 * the roofline denominator for kernels bound by the FP64 / FP32 pipes. No counterpart in the
 * reference (which has no GPU path). */
int pimd_peak_flops(int device, int fp64, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* PIMD_GB300_H */
