/*
 * pimd_oracle.h -- CPU FP64 oracle for the PIMD-F90 force/propagation hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA engine is compared
 * against; it is never linked into, called by, or shipped with the engine. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 *
 * It restates, line by line and in IEEE double with no FMA contraction, the reference's
 *   pot_ttm/pot_ttm.f90, pot_ttm/ewald.f90, pot_ttm/smear.f90, pot_ttm/find_neigh.f90,
 *   pot_ttm/nasa.f90, pot_ttm/potential.f90 (init_pot), pot_ttm/pot_spc.f90,
 *   math.f90 (erfc, gammq2_3), NormalModes.f90, Langevin.f90, MD.f90 (PIMD_VV),
 *   main_stuff.f90 (PBCs, calc_uk), force_calc.f90 (full_bead_forces).
 *
 * Parity status: the reference is Fortran and no Fortran compiler exists in the build
 * container, so this restatement is NOT pinned by outputs of the reference itself
 * ("parity unpinned"). It is pinned by physics known-answer tests instead (tests/).
 *
 * Units as in the reference: Angstrom, kcal/mol, amu, ps. dRR is the gradient dE/dx.
 */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int pot_model;       /* 2 TTM2.1-F, 3 TTM3-F, 4 q-SPC/Fw, 5 SPC/F                  */
    int natoms;          /* 3 * Nwaters, atoms ordered O H H O H H ...                  */
    double box[3];       /* orthorhombic box lengths (A)                                */
    double rc;           /* real-space cutoff (A)                                       */
    double rc1;          /* start of the vdW force switch (A), TTM3-F only             */
    double eps_ewald;    /* reference Ewald rule: alpha = sqrt(-ln eps)/Rc (alpha<=0)   */
    double alpha;        /* explicit Ewald alpha (1/A) when > 0                          */
    int nmax;            /* explicit k shell |n|^2 <= nmax^2 when alpha > 0             */
    int polar_maxiter;   /* dipole iterations cap                                       */
    double polar_sor;    /* SOR mixing                                                  */
    double polar_eps;    /* convergence threshold on stath*|dmu|                        */
    int guess_initdip;   /* 4-step predictor from the dipole history                   */
    int contraction;     /* CONTRACTION: skip the monomer PES                           */
    int nbeads;          /* number of predictor-history slots (one per bead)            */
    int shared_history;  /* 1: all beads share slot 0 (reference on one MPI rank)       */
} orc_params;

void *orc_create(const orc_params *p);
void orc_destroy(void *h);
/* Ewald set-up outputs: alpha, nk, hmax/kmax/lmax */
void orc_ewald_info(void *h, double *alpha, int *nk, int *hkl_max);
void orc_kvectors(void *h, int *k_hkl /* 3*nk */, double *kvec /* 3*nk */, double *Ak /* nk */);

/* pot_ttm.f90:3 -- one bead. bead selects the predictor history slot. */
void orc_pot_ttm(void *h, int bead, const double *RR, const double *RRc, double *En, double *dRR,
                 double *virt, double *virialc, double *dip_momI, double *Edip_mom, double *chg,
                 int t);
/* pot_spc.f90:1 */
void orc_pot_spc(void *h, const double *RR, double *En, double *dRR, double *virt,
                 double *dip_momI, double *chg);
/* find_neigh.f90 for all molecules of RR(3,Natoms): writes (i, j) 0-based pairs in the
 * reference's order (i ascending, then j ascending) and returns the pair count */
int orc_neighbors(void *h, const double *RR, int *ij, int cap);
/* system_mod.f90:30 globals after the last call: Umon, Uvdw, Uelec, Uind; and iterations */
void orc_energies(void *h, double *U4, int *niter, double *last_deltadip);

/* force_calc.f90:26-106 over all beads with nthreads worker threads (one oracle state per
 * thread). Layouts as the reference: RRt(3,Natoms,P), dRRt(3,Natoms,P), dip(3,Nw,P). */
void orc_full_bead_forces(const orc_params *p, int nthreads, const double *RRt, const double *RRc,
                          double *Upott, double *dRRt, double *virialt, double *virialct,
                          double *dip_momIt, double *dip_momEt, double *chg, int t);

/* NormalModes.f90:68 InitNormalModes. Outputs arrays of length P and C(P,P) col-major. */
void orc_nm_init(int P, double omegan, double delta, double setNMfreq, double *A11, double *A12,
                 double *A21, double *A22, double *omegalist, double *msf, double *C);
/* NormalModes.f90:34 EvolveRing for one atom: RR(3,P), PP(3,P) inout */
void orc_evolve_ring(int P, const double *A11, const double *A12, const double *A21,
                     const double *A22, const double *msf, const double *C, double *RR,
                     double *PP, double mass);
/* Langevin.f90:68 Init_Langevin_NM */
void orc_langevin_init(int P, const double *omegalist, double delt2, int centroid_thermostat,
                       double tau_centroid, double temp_P, double *c1, double *c2);
/* Langevin.f90:30 Langevin_NM with the standard normals supplied: xi(3,P,Natoms) */
void orc_langevin_nm(int P, int natoms, const double *C, const double *msf, const double *c1,
                     const double *c2, double massO, double massH, double *PPt, const double *xi);
/* main_stuff.f90:349 calc_uk */
double orc_calc_uk(int P, int natoms, double massO, double massH, const double *PPt,
                   double setNMfreq, const double *C, const double *msf);

/* MD.f90:35-110 PIMD_VV for one replica: Langevin bead thermostat (when xi1/xi2 given),
 * half kick, EvolveRing, centroid, PBCs, full_bead_forces, half kick, thermostat.
 * State RRt, PPt, dRRt inout; outputs the summed potential, virial, centroid virial.   */
typedef struct {
    double delt;         /* ps */
    double massO, massH;
    double setNMfreq;
    int langevin;        /* apply Langevin_NM before the first and after the second kick */
    int centroid_thermostat;
    double tau_centroid;
    double temp;         /* K (physical); the thermostat uses temp*P                   */
} orc_md_params;

void orc_pimd_vv_step(void *h, const orc_md_params *mp, int P, double *RRt, double *PPt,
                      double *dRRt, double *RRc, const double *xi1, const double *xi2, int t,
                      double *Upot, double *virial, double *virialc, double *uk);

/* A pool of nthreads oracle states; bead k is always evaluated by thread k % nthreads, so
 * the per-bead predictor history persists across calls (the MPI-over-beads analogue of
 * force_calc.f90:26-106 on the host cores). */
void *orc_pool_create(const orc_params *p, int nthreads);
void orc_pool_destroy(void *pool);
void orc_pool_forces(void *pool, const double *RRt, const double *RRc, double *Upott, double *dRRt,
                     double *virialt, double *virialct, int t);
void orc_pimd_vv_step_pool(void *h, void *pool, const orc_md_params *mp, int P, double *RRt,
                           double *PPt, double *dRRt, double *RRc, const double *xi1,
                           const double *xi2, int t, double *Upot, double *virial,
                           double *virialc, double *uk);

/* NormalModes.f90:308-341 (real2NM, NM2real) and 224-275 (gen_rand_ring, gen_rand_ring_momenta
 * with the unit normal draws xi(3,P) supplied) for one atom. */
void orc_real2nm(int P, const double *C, const double *A, double *out);
void orc_nm2real(int P, const double *C, const double *A, double *out);
void orc_gen_rand_ring(int P, const double *C, const double *omegalist, const double *msf, double mass,
                       double temp, const double *xi, double *RR);
void orc_gen_rand_ring_momenta(int P, const double *C, const double *msf, double mass, double temp,
                               const double *xi, double *PP);
/* Nose_Hoover.f90:33-112 (one half step of a chain-2 thermostat), main_stuff.f90:145-171 (the
 * bead Nose-Hoover thermostat on the normal modes, vxi_beads(2,natoms,P,3)), estimators.f90:57-73
 * (ring K0) and estimators.f90:30-96 with InputOutput.f90:566 (sys_temp, virial-estimator energy
 * and pressure, simple-estimator energy and pressure into est5). */
void orc_nose_hoover(double *s, double *uk, double *vxi, double tau, double delt2, int L, double temp);
void orc_bead_nose_hoover(int P, int natoms, const double *C, const double *omegalist, const double *msf,
                          double massO, double massH, double *PPt, double *vxi_beads, int centroid_thermostat,
                          double tau_centroid, double delt2, double temp);
double orc_ring_k0(int P, int natoms, double massO, double massH, const double *RRt);
void orc_estimators(int natoms, int P, double volume, double omegan, double Upot, double virial,
                    double virialc, double uk, double K0raw, double *est5);
/* PIMD_VV with bead_thermostat 0 none / 1 Langevin_NM (xi1, xi2) / 2 Nose-Hoover on the normal
 * modes, and the global chain thermostat (tau) when global_thermostat != 0; uk_state is the
 * reference's uk across steps, vxi_global[2] and vxi_beads the chain velocities; out[12]. */
#define ORC_MD_NOUT 12
void orc_pimd_vv_step_ex(void *h, void *pool, const orc_md_params *mp, int bead_thermostat,
                         int global_thermostat, double tau, int P, double *RRt, double *PPt,
                         double *dRRt, double *RRc, const double *xi1, const double *xi2,
                         double *vxi_global, double *uk_state, double *vxi_beads, int t,
                         double *out);

/* contracted_MD (MD.f90:276-449, mode 0, intra_timesteps inner steps) and monomer_PIMD
 * (MD.f90:117-265, mode 1): h is a one-bead oracle of the centroid (contraction set in mode 0). */
void orc_contracted_step(void *h, const orc_md_params *mp, int mode, int intra_timesteps,
                         int bead_thermostat, int global_thermostat, double tau, int P, double *RRt,
                         double *PPt, double *dRRt, double *dRRfast, double *RRc, const double *xi1,
                         const double *xi2, double *vxi_global, double *uk_state, double *vxi_beads,
                         int t, double *out, double *dip_momIt, double *dip_momEt);

/* Analyses: geometry_calculator.f90 (accumulator of 176 doubles), diffusion_calculator.f90 (MSD
 * state [t, initialised, aMS(ntimes+1), netdisp(3 Nw), Oxy(3 Nw)]), four1.f, math.f90:42-140 and
 * spectral_properties.f90 (IR spectrum of dip(3, tread), DOS of Hvel(3, tread, nhyd)). */
void orc_geometry_accumulate(double *acc, int natoms, int P, const double *box, const double *RR,
                             const double *RRt);
void orc_geometry_report(const double *acc, int P, double *out);
void orc_msd_step(double *st, int natoms, int ntimes, const double *box, const double *RRc);
void orc_msd_report(const double *aMS, int ntimes, double timestep, double *out);
void orc_four1(float *data, int nn, int isign);
void orc_corr_function(const float *in, int tread, double *out);
void orc_calc_dft(const double *in, int tread, double timestep, double *out, double *freqs);
void orc_ir_spectrum(const float *dip, int tread, const double *box, double timestep, double temp,
                     int *npoints, double *freq, double *ir);
void orc_dos(const float *Hvel, int tread, int nhyd, double timestep, int *npoints, double *freq,
             double *dos);

#ifdef __cplusplus
}
#endif
