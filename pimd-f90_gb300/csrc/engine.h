// engine.h -- internal state of one force-engine context and the kernel launchers.
//
// One context holds the module state the reference keeps in pot_mod/system_mod
// (pot_ttm/pot_mod.f90:47-83, system_mod.f90:22-44): model parameters, Ewald k-vector
// tables, scratch arrays and the per-bead induced-dipole predictor history. All P beads of
// a ring polymer are evaluated together: every kernel has the bead as a grid axis.
//
// HBM layout (per context, P beads, N waters, S sites per bead = 4N for TTM / 3N for SPC,
// sites in the reference's block order O(0..N-1) H1(N..2N-1) H2(2N..3N-1) M(3N..4N-1)):
//   pos   [P][S]      double4_32a (x, y, z, q)   site positions and charges
//   posc  [S]         double4_32a                centroid sites (for the centroid virial)
//   F     [P][S]      double4_32a (Ex,Ey,Ez,phi) charge field Efq and potential phi
//   dR    [P][S][3]   gradient accumulator
//   dip   [P][S][3]   induced dipoles (non-zero on the dipole sites only)
//   Efdr  [P][S][3]   real-space dipole field of the current iteration
//   pairs [P][cap]    int2 half neighbour list of O-O pairs (i < j), ordered as find_neigh
//   Tdd   [P][cap][ND][6]  cached dipole-dipole tensors for the iterations
//   tab   [P][nx+ny+nz][S]  double2 e^{i 2pi n x/L} recurrence tables (ssincos)
//   Spart [P][tiles][nk]    double2 per-site-tile structure-factor partials
//   Sq, Sm [P][nk]          double2 charge / dipole structure factors
//   Sdip  [P][nk][3]        double2 sum mu_c e^{ik.r} for the reciprocal virial
//   acc   [P][NACC]         per-bead energy / virial accumulators
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/pimd_gb300.h"
#include "common.cuh"

namespace pimd {

enum { PIMD_PREC_FP64 = 0, PIMD_PREC_MIXED = 1 };

enum { ACC_UMON = 0, ACC_UVDW, ACC_UELEC2, ACC_UIND, ACC_VIRT, ACC_VIRIALC = ACC_VIRT + 9, ACC_DSQ,
       ACC_MUEFQ, ACC_DELTADIP, ACC_NITER, ACC_CONV, NACC = 24 };

// site-kind parameter tables, index [isp][jsp] with isp, jsp = 1..4 (O, H1, H2, M)
struct PairTables {
    double apol_qq[5][5];  // aCCaCD * polfac(i) * polfac(j) for the charge phase
    double ra_qq[5][5];    // apol_qq^(1/3)
    double apol_dd[5][5];  // aDD * polfac(i) * polfac(j)
    double apol_cd[5][5];  // aCCaCD * polfac(i) * polfac(j)
};

// FP32 copies of the pair constants for the mixed engine's pair kernels (converted once on the
// host, so no FP64-to-FP32 conversion -- an FP64-pipe instruction -- sits in a pair loop)
struct PairTablesF {
    float apol_qq[5][5], ra_qq[5][5], apol_dd[5][5], apol_cd[5][5];
    float vdw[5];            // vdwA .. vdwE
    float shiftA, shiftB, rc1;
    float box[3], boxi[3];
};

// k-space run: a maximal block of consecutive k-vectors with equal (kx, ky); kz runs over
// [kzlo, kzlo + nkz). kbeg is the index of the first k-vector of the run.
struct KRun {
    int kx, ky, kzlo, nkz, kbeg, pad0, pad1, pad2;
};
// structure-factor chunk: k in [k0, k1), runs [r0, r1)
struct KChunk {
    int k0, k1, r0, r1;
};

// Everything a kernel needs, passed by value.
struct KP {
    int model, N, S, P, natoms, cap, nk, nrun, nchunk, ntab, hmax, kmax, lmax;
    int fd, ld;          // dipole sites [fd, ld)
    int fq;              // first site of the Ewald charge sums (TTM: N, O is uncharged; SPC: 0)
    int ndd;             // dipole site pairs per molecule pair (TTM3 1, TTM2 9)
    int contraction, guess, t, polar_maxiter, same_acd;
    double polar_eps;
    double box[3], boxi[3], volume, rc2, rc1;
    float boxq[3];  // box / 2^32 (FP32): the length of one unit of ofix
    double vdwA, vdwB, vdwC, vdwD, vdwE, shiftA, shiftB;
    PairTablesF ptf;  // FP32 copies of pt, the vdW constants and the box (kp_float_tables)
    double gammaM, polar[5], dms1, dms2, dms3, polar_sor, stath, factor, Uvdw_lrc;
    double qO, qH, roh0, th0, harmkb, harmka;
    const double *c5z;   // NASA PES coefficients for non-default scale factors (null: published)
    double nasa_f5z;     // NASA scale factor of deoh / phh1
    EwC ew;
    EwCf ewf;  // FP32 copy for the mixed engine
    PairTables pt;
    // buffers
    const double *RRt, *RRc;
    double *dRRt, *dipI, *dipE, *chg;
    double4_32a *pos, *posc, *F;
    double *dR, *dip, *Efdr, *txdip, *grdq, *Tdd, *Tself;
    int2 *pairs;
    int *npair;
    double2 *tab, *Spart, *Sq, *Sm, *Sdip;
    const KRun *runs;
    const KChunk *chunks;
    const double4_32a *kinfo;  // (kx, ky, kz) vector, 4pi Ak / V
    const double *kAk;     // Ak = 2 exp(-k^2/4a^2)/k^2
    const int2 *kidx;      // (run index, kz) of each k-vector
    const float2 *runkf;   // FP32 (kx, ky) components of each run's k-vectors (mixed engine)
    const float *kzf;      // FP32 kz component of each k-vector (mixed engine)
    const float4 *kvirf;   // FP32 (k_x, k_y, k_z, Ak) of each k-vector (mixed engine)
    const float *kc2f;     // FP32 2 / k^2 + 1 / (2 alpha^2) of each k-vector (mixed engine)
    float2 *Wf;            // [P][2][nk] FP32 field weights 4pi Ak/V conj(S): slot 0 charge, 1 dipole
    const int *sfrun;      // runs in the order of the structure-factor tiles (sorted by nkz)
    const int4 *sftile;    // per tile: first ez slot, kz groups, runs, offset into sfrun
    int *nbrtmp;           // [P][N] neighbour counts / offsets
    // mixed-precision engine
    float2 *tabf;          // [P][ntab][S] FP32 copies of the FP64 recurrence tables
    float4 *posf;          // [P][S] (site - own O (min image), q)
    float4 *rhof;          // [P][S] centroid site - own bead O (raw difference)
    uint4 *ofix;           // [P][N] O sites as 32-bit fractions of the box edges: the wrapping
                           // unsigned difference of two of them is the minimum image
    float4 *orawf;         // [P][N] O sites (unwrapped) in FP32: force-phase centroid-virial lever
    // TTM3-F mixed engine: per molecule [P][N][2] the M site as 32-bit fractions of the box
    // edges (as float bits) and its FP32 dipole, the one record a real-space dipole-field entry
    // reads of its partner (null: other models)
    float4 *mrec;
    double4_32a *Fx;       // [P][S] reciprocal charge field / force-pass sums when those passes run
                           // beside the pair kernels (mixed engine): (x, y, z, potential)
    int fx_mode;           // bit 0: the charge field is in Fx (k_after_qq adds it to F); bit 1: the
                           // force pass is in Fx (k_finish adds it to dR and the potentials)
    int fx_s0;             // first site the tensor-core passes write (sites below are not in Fx)
    float4 *gq23;          // [GQ_N] cubic pieces of h(u) = Gamma(2/3) Q(2/3, u^3) exp(u^3) (mixed.cu)
    float4 *dipf;          // [P][S] FP32 copy of the induced dipoles (written with every update)
    // asynchronous real-space dipole field (mixed engine, TTM3-F, tensor-core field pass): the
    // field pass does not wait for k_dd_real_m; of the two, the last to finish a unit of 128
    // dipole sites runs the unit's SOR update, which writes the other FP32 dipole buffer (the
    // real-space gathers of the iteration may still be reading this one)
    int dd_async;          // the dipole iterations run so (0: the field pass runs the SOR)
    int unit_sbase, nunits;  // first site of unit 0 (a multiple of 32), units per bead
    float4 *dipf_alt;      // [P][S] the second FP32 dipole buffer
    float4 *Erec;          // [P][S] reciprocal field of the iteration at the dipole sites
    unsigned *unit_cnt;    // [P][nunits] arrivals at each unit (reset by the last)
    int *fcnt, *foff;      // [P][N] full neighbour list counts / offsets
    int *fnbr;             // [P][fcap] full neighbour list (j ascending per i)
    int *fntot;            // [P] full-list length
    float2 *Tf;            // [P][fcap][ndd] FP32 (t1, 3 t2) dipole-tensor scalars of the full list
    int *fj;               // [P][fcap] partner j of each full-list entry
    int l2keep;            // k_dd_real_m loads fj / Tf with the L2 evict-last policy
    int fcap;
    double4_32a *Fpart;    // [slices][P][S] per-k-slice partial fields of the Ewald field passes
    // cell lists of large boxes (N > 1024, >= 4 cells of width >= Rc per edge)
    int cl_n[3], cl_ncell;     // cells per edge, cells (0: no cell lists)
    int *cl_mol;               // [P][N] cell of each molecule
    float4 *cl_posf;           // [P][N] FP32 O sites wrapped into the box
    int *cl_cnt, *cl_start;    // [P][ncell] counts, [P][ncell + 1] starts
    int *cl_list;              // [P][N] molecules ordered by cell
    int *cl_row, *cl_rowlen;   // [P][N][256] sorted full rows, [P][N] their lengths
    double *acc;
    unsigned *err;
    int *allconv;
    const int *brep;              // replica of each bead when one context holds several ring
                                  // polymers (null: one replica); RRc and posc are per replica
    int nrep;                     // replicas in this context (>= 1)
    int *dstep;                   // [0] MD step t of the force call, [1] dipole iterations done
    unsigned *fin_counter;        // blocks done in the dipole field pass (fused convergence test)
    unsigned long long cond;      // CUDA-graph conditional handle of the dipole loop (0: host loop)
};

// refresh kp.ptf from the FP64 constants (after they are set or changed)
inline void kp_float_tables(KP &kp) {
    for (int i = 0; i < 5; i++)
        for (int j = 0; j < 5; j++) {
            kp.ptf.apol_qq[i][j] = (float)kp.pt.apol_qq[i][j];
            kp.ptf.ra_qq[i][j] = (float)kp.pt.ra_qq[i][j];
            kp.ptf.apol_dd[i][j] = (float)kp.pt.apol_dd[i][j];
            kp.ptf.apol_cd[i][j] = (float)kp.pt.apol_cd[i][j];
        }
    const double v[5] = {kp.vdwA, kp.vdwB, kp.vdwC, kp.vdwD, kp.vdwE};
    for (int i = 0; i < 5; i++) kp.ptf.vdw[i] = (float)v[i];
    kp.ptf.shiftA = (float)kp.shiftA;
    kp.ptf.shiftB = (float)kp.shiftB;
    kp.ptf.rc1 = (float)kp.rc1;
    for (int c = 0; c < 3; c++) {
        kp.ptf.box[c] = (float)kp.box[c];
        kp.ptf.boxi[c] = (float)kp.boxi[c];
    }
}

// acc[ACC_CONV] != 0.0 (bead b's dipoles converged) tested on the bits, without an FP64 compare
PIMD_D bool bead_converged(const KP &kp, int b) {
    const unsigned long long u = reinterpret_cast<const unsigned long long *>(kp.acc)[(size_t)b * NACC + ACC_CONV];
    return (u & 0x7fffffffffffffffULL) != 0ULL;
}

// The FP32 dipoles an iteration reads and the buffer its SOR update writes: the same buffer
// unless the real-space field runs asynchronously (then iteration d + 1 reads buffer d & 1).
PIMD_D const float4 *dipf_cur(const KP &kp) { return (kp.dd_async && (kp.dstep[1] & 1)) ? kp.dipf_alt : kp.dipf; }
PIMD_D float4 *dipf_next(const KP &kp) { return (kp.dd_async && !(kp.dstep[1] & 1)) ? kp.dipf_alt : kp.dipf; }
// the FP32 dipole of dipole site s of bead b into the molecule record (TTM3-F: s = fd + i)
PIMD_D void mrec_dipole(const KP &kp, int b, int s, float4 m) {
    if (kp.mrec && s >= kp.fd && s < kp.ld) kp.mrec[2 * ((size_t)b * kp.N + (s - kp.fd)) + 1] = m;
}

// replica of bead b and its centroid sites (posc[replica][S])
PIMD_HD int rep_of(const KP &kp, int b) { return kp.brep ? kp.brep[b] : 0; }
PIMD_HD const double4_32a *posc_of(const KP &kp, int b) { return kp.posc + (size_t)rep_of(kp, b) * kp.S; }

// Named phase timers (the reference's dans_timer.f90 start_timer/stop_timer), recorded as
// CUDA events on the engine stream and resolved lazily.
struct PhaseTimers {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<std::string> names;
    std::vector<double> ms;
    std::vector<long> count;
    cudaEvent_t cur0 = nullptr;
    int cur = -1;
};

struct Engine {
    KP kp;
    PhaseTimers timers;
    int precision = 0;
    int device = 0;
    cudaStream_t stream = 0;
    bool own_stream = false;
    int nchunk = 0, ntile_q = 0, ntile_d = 0, max_runs_chunk = 0;
    int max_slices = 16;  // k-slices of the Ewald field passes (Fpart capacity)
    bool sf_tiled = true;  // mixed engine: register-tiled structure factors (k_sfac_f)
    int sf_groups = 0;     // site groups of k_sfac_f (0: sized from the SM count)
    int sf_ntiles = 0, sf_nkg_max = 0;  // run tiles of k_sfac_f and the largest kz-group count
    int sp_cap = 1;        // site groups the structure-factor partial buffer (Spart) holds
    bool ff_regs = true;   // mixed engine: field passes with the kz row in registers (k_field_f)
    bool nbr_block = true; // one-launch neighbour lists per bead for N <= 1024 (k_nbr_block)
    bool nbr_cells = true; // cell lists for N > 1024 when the box holds >= 4 cells per edge
    bool wave_shapes = true;  // k-slices / site groups chosen by wave quantisation (occupancy API)
    bool dd_overlap = true;   // mixed engine: real-space dipole field beside the structure factor
    bool dd_async = false;    // ... and beside the field pass too, the SOR by the last to finish (TTM3-F)
    // tensor-core (tcgen05, 3xTF32) dipole structure factor of the mixed engine (ewald_tc.cu)
    bool sf_tc = true;        // use it when tc_ready
    bool tc_ready = false;    // run groups built and the table tensor map encoded
    bool tc_dip_ok = false;   // the dipole-component sums (three partials per k) fit too
    int tc_ntg = 0, tc_ncolmax = 0, tc_nabuf = 0;
    const int4 *d_tcslot = nullptr;   // per run slot: run, local k offset, kzlo, nkz
    const float2 *d_tcskv = nullptr;  // per run slot: FP32 (k_x, k_y)
    const void *d_tcgrp = nullptr;    // per run group (TcGroup): slots, columns, kz rows, k-vectors
    const void *d_tckloc = nullptr;   // (k-vector, weight) of each local index, group after group
    const float *d_tckzv = nullptr;   // FP32 k_z component by kz + lmax
    void *d_tcx = nullptr;            // X-operand cache of the dipole sites (uint4 blocks)
    int tc_xsub = 0, tc_xblock = 0;   // 16-site blocks per bead and run group, bytes per block
    bool tc_xcache = true;            // use the X cache in the dipole iterations
    bool tc_pdl = true;               // field pass and next structure factor as programmatic dependent launches
    int loop_unroll = 3;              // dipole iterations per body of the graph's conditional loop
    bool ewald_overlap = true;        // reciprocal charge / force passes beside the pair gathers
    bool dd_otf = false;              // real-space dipole tensors formed in each iteration (no cache)
    bool l2_keep = false;             // the iterations' cached operands (X blocks, dipole-pair scalars) loaded evict-last in L2
    bool ff_tc = true;                // tensor-core dipole field pass (k_field_tc) when tf_ready
    bool tf_ready = false;
    int tf_nr = 0, tf_nph = 0, tf_jm = 0, tf_ncol = 0, tf_kq = 0;
    bool tf_qd_ready = false;         // the force-pass modes (charge / dipole halves of ewald_std_qd)
    int tf_nphd = 0, tf_ncold = 0;    // runs per pass and V rows of the dipole-force mode
    int tf_vpp = 0, tf_wglob = 0;     // field passes: V built per pass (> 2 passes), weights read from global
    int tf_wglob_d = 0;               // the same for the dipole-force mode's weights
    const int2 *d_tfkpm = nullptr;    // per (run slot, j): k-vectors of kz = +j, -j
    alignas(64) unsigned char tc_map[128];  // CUtensorMap of the FP32 tables tabf
    size_t cap = 0;
    std::vector<KRun> h_runs;
    std::vector<KChunk> h_chunks;
    std::vector<int> h_khkl;
    std::vector<double> h_kvec, h_Ak;
    // host pinned staging
    double *h_pin = nullptr;
    size_t h_pin_bytes = 0;
    int *h_allconv = nullptr;
    double *d_out = nullptr;  // small device staging for per-bead scalar outputs
    double *d_md = nullptr;   // device MD state for the host-array step (pimd_md_step)
    std::vector<void *> allocs;
    std::string last_error;
    int last_niter_max = 0;
    long long nlaunch = 0;  // kernels launched by this context
    // CUDA-graph execution of the MD step (pimd_set_graph): captured once per set of device
    // pointers and replayed; the dipole iterations run in a conditional while node
    bool graph_mode = false;
    bool capturing = false;
    cudaStream_t body_stream = nullptr;
    // mixed engine: a second stream on which the real-space dipole field of an iteration runs
    // beside the structure factor (fork / join events; branches of the graph when captured)
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_nbr = nullptr;  // the neighbour lists built on the second stream beside k_sites
    bool nbr_overlap = true;       // (knob)
    // the dipole iterations' own pair (inside a graph they are captured into the conditional
    // loop's body, a graph of its own, which must not share a stream with the outer capture)
    cudaStream_t loop_aux = nullptr;
    cudaEvent_t loop_fork = nullptr, loop_join = nullptr;
    // at the start of a loop body the real-space field waits on this programmatic event of the
    // structure factor (all its CTAs resident), so that it does not take the SMs first
    cudaEvent_t loop_pev = nullptr;
    bool sfac_pev_req = false, sfac_pev_armed = false;
    bool dd_pev = true;  // use it (knob)
    // the field pass waits on this programmatic event of the real-space field (all its blocks
    // started) instead of its completion; griddepcontrol.wait in the field pass then waits for
    // the real-space grid before anything reads its output
    cudaEvent_t loop_jpev = nullptr;
    bool dd_jpev_req = false, dd_jpev_armed = false;
    bool dd_jpev = true;  // use it (knob)
    bool field_needs_join = false;  // a field pass launched without griddepcontrol.wait must first wait on loop_join
    cudaGraphExec_t gexec = nullptr;
    std::vector<const void *> gkey;
    long long graph_launches = 0, graph_captures = 0;
    // differentiation form (adjoint.cu): model parameters theta and the forward's tape
    double theta[PIMD_NTHETA];
    double *d_c5z = nullptr;     // NASA coefficients for the current theta
    bool tape_on = false;        // record the dipole iterations during the force call
    int tape_kmax = 0;           // iterations the tape holds
    double *d_tape = nullptr;    // [kmax + 1][P][N][3] dipoles of the dipole sites per iteration
    double *d_phiq = nullptr;    // [P][S] charge-only potential after the charge phase
    double2 *d_tapeS = nullptr;  // [kmax][P][nk] structure factor S(mu_k) of each iteration's dipoles (Sm form)
    double *d_adj = nullptr;     // backward scratch
    size_t adj_bytes = 0;
    bool tape_valid = false;
    double polfac[5] = {0, 0, 0, 0, 0};  // polfac^(-1/2) per site kind (potential.f90:157-160)
    double vdwA_model = 0, vdwB_model = 0, rc = 0;
    // normal modes (filled by pimd_nm_init)
    int nm_P = 0;
    double *d_nmC = nullptr, *d_nmA = nullptr;  // C(P,P), [A11,A12,A21,A22,msf,c1,c2] x P
    std::vector<double> h_nm;                     // host copy: A11..A22, omegalist, msf, C
    double nm_omegan = 0, nm_setfreq = 0;         // InitNormalModes' omegan and setNMfreq
    std::vector<double> h_nmC;                    // host copy of C(P,P), column-major
    unsigned long long host_rng = 20261203ull;    // splitmix64 state of the host normal draws
    // Nose-Hoover thermostats of the MD step (pimd_set_thermostat): the global chain
    // (MD.f90:43-46, 101-104) and the bead chains on the normal modes (main_stuff.f90:145-171)
    bool nh_global = false, nh_bead = false, nh_centroid = false;
    double nh_tau = 0, nh_temp = 0, nh_tau_centroid = 0;
    long long nh_gen = 0;          // configuration generation (part of the MD-step graph key)
    double *d_nh = nullptr;        // [vxi1, vxi2, uk, s_pre, s_post, uk_mid, K0, spare]
    double *d_vxib = nullptr;      // vxi_beads(2, Natoms, P, 3)
};

// Arguments of the normal-mode / thermostat / integrator kernels for one ring polymer
// (nm.cu); a context with several replicas launches them once per replica.
struct NMArgs {
    int P, natoms;
    const double *C;    // C(P,P) column-major: C[j + P*k] = C(j+1, k+1); then the same as FP32
                        // pairs (hi, lo) with hi + lo = C to 2^-48 (float2[P*P], fast transforms)
    const double *A;    // [A11, A12, A21, A22, msf, c1, c2, A12 / msf, A21 msf, c2 sqrt(msf), omegalist] x P
    double massO, massH;
    double delt, delt2, box0, boxi0;
    int langevin, evolve;
    const double *xi;   // (3, P, Natoms) standard normals, or null
    unsigned long long seed, counter;
    const int *tstep;   // device step word: when set, counter = 2 t + phase
    int phase;
    int fast;           // mixed engine: the MD-step kernels in FP32-pair arithmetic with FP32
                        // Box-Muller draws (FP64 state, not bit-identical to the FP64 kernels)
    double mass[2], minv[2], msqrt[2];  // O, H: m, 1/m, sqrt(m) (filled by nm_fast_args)
    float2 kick;                        // MASSCON dt/2 as an FP32 pair
    float2 hminv[2], pinv, boxf;        // 1/(2m) of O, H; 1/P; box edge (pairs)
    float boxif;                        // 1/box edge
    // Nose-Hoover chains on the normal modes instead of Langevin_NM (main_stuff.f90:145-171)
    int bead_nh, centroid_nh;
    double tau_centroid, nh_temp;       // chains couple to nh_temp = Nbeads T
    double *vxib;                       // vxi_beads(2, Natoms, P, 3)
    const double *s_pre;                // global chain's scale factor applied after the bead thermostat
    int nm_ke;                          // calc_uk in normal-mode space (setNMfreq != 0, P > 1)
    int nodrift;                        // k_md_pre without the drift (contracted MD: the inner steps drift)
};
// one replica of a batch for the batched MD-step kernels: its arguments and state pointers
struct NMBatchRep {
    NMArgs a;
    double *RRt, *PPt, *dRRt, *RRc, *uk;
};
struct NMSumRep {  // its step outputs (k_md_sum's inputs)
    int P;
    const double *Upott, *virialt, *virialct, *uk;
    double *out4;
};
// the batched phases of every replica's MD step (phase 0 before the force call, 1 after); with
// nblk = 0 only the shared-memory opt-in (call once outside any stream capture)
void nm_launch_md_batch(int phase, bool fast, int nblk, size_t smem, cudaStream_t st, const NMBatchRep *reps,
                        const int2 *blkmap);
__global__ void k_md_sum_batch(const NMSumRep *reps);
NMArgs nm_step_args(Engine &E, const pimd_md_params *mp, const double *xi1);
void nm_launch_evolve(const NMArgs &a, cudaStream_t st, double *RRt, double *PPt);
void nm_launch_ring_sums(const NMArgs &a, cudaStream_t st, const double *RRt, const double *PPt, double *sums);
void nm_launch_nh_global(Engine &E, const double *uk_end, int slot, double delt2);
void nm_launch_nh_scale(Engine &E, double *PPt);
void nm_launch_estimators(Engine &E, const double *uk, const double *uvv, double *out);
__global__ void k_md_pre(NMArgs a, double *RRt, double *PPt, const double *dRRt, double *RRc);
__global__ void k_md_post(NMArgs a, double *PPt, const double *dRRt, double *uk);
__global__ void k_md_sum(int P, const double *Upott, const double *virialt, const double *virialct, const double *uk,
                         double *out4);
void nm_launch_shape(int P, int natoms, int *threads, int *blocks, size_t *smem);
void nm_smem_optin(int P);
void nm_extend_A(std::vector<double> &A, int P, const std::vector<double> &omegalist);
void nm_fast_args(NMArgs &a);
size_t nm_fast_smem(int P, int G);
void nm_launch_md_pre(const NMArgs &a, cudaStream_t st, double *RRt, double *PPt, const double *dRRt, double *RRc);
void nm_launch_md_post(const NMArgs &a, cudaStream_t st, double *PPt, const double *dRRt, double *uk);
void nm_pair_copy(const std::vector<double> &C, std::vector<double> &out);  // C then its FP32 pairs
void nm_init_host(int P, double omegan, double delta, double setNMfreq, std::vector<double> &A11,
                  std::vector<double> &A12, std::vector<double> &A21, std::vector<double> &A22,
                  std::vector<double> &om, std::vector<double> &msf, std::vector<double> &C);
// context creation with nrep ring polymers sharing one box (brep: replica of each bead, host)
int create_context(Engine &E, const pimd_params *p, int nrep, const int *brep);

// phase timers (capi.cu)
void timer_begin(Engine &E, const char *name);
void timer_end(Engine &E);
int run_forces(Engine &E, int t, int check_every, double *Upott, double *virialt, double *virialct, double *virt9);

// differentiation form (adjoint.cu)
void tape_record(Engine &E, int iter);
int apply_theta(Engine &E);
void adjoint_init(Engine &E);
void adj_structure_factor(Engine &E, const double *dipbuf, const float4 *dipf32, double2 *Sout, double *bacc);
void launch_adj_pairs_m(Engine &E, const double pf[5], const double *ebar, const double *nu, double *grad, double *phin,
                        double *thacc);
void adj_dipole_field(Engine &E, double2 *Sm_u, double *bacc, double *Dr);
void adj_rec(Engine &E, int mode, const double *a, const double *bvec, const double2 *SA, const double2 *SB,
             const double *ebw, double *grad, double *phi);

// launchers (neighbors.cu)
void neighbors_init(Engine &E);
void launch_neighbors(Engine &E);
bool nbr_from_inputs(const Engine &E);
// launchers (pot.cu)
void pot_init_constants(Engine &E);
void launch_sites(Engine &E);
void launch_pair_qq(Engine &E);
void launch_after_qq(Engine &E);
void launch_dd_real(Engine &E);
void launch_dd_update(Engine &E);
void launch_set_step(Engine &E, int t);
void launch_pair_force(Engine &E);
void launch_finish(Engine &E);
void launch_totals(Engine &E, double *Upott, double *virialt, double *virialct, double *virt9);
// launchers (mixed.cu): FP32 pair arithmetic, FP64 accumulation
cudaError_t mixed_init(Engine &E);  // FP32 lookup tables of the mixed engine
void launch_site_offsets(Engine &E);
void launch_pair_qq_m(Engine &E);
void launch_dd_tensors_m(Engine &E);
void launch_dd_real_m(Engine &E);
bool dd_async_ok(const Engine &E);
void launch_dipf_sync(Engine &E);
void launch_pair_force_m(Engine &E);
// launchers (ewald.cu)
void ewald_init(Engine &E);
void launch_ewald_tables(Engine &E);
void launch_ewald_sq(Engine &E);
void launch_ewald_fq(Engine &E);
void launch_ewald_smu(Engine &E);
void launch_ewald_qd(Engine &E);
void launch_ewald_pw(Engine &E);
// tensor-core structure factors (ewald_tc.cu): setup once per context; per call the launch
// writes the sums of op (OP_Q: Sq + charge weights, OP_MU: Sm + dipole weights, OP_DIP: Sdip)
// and returns 1, or returns 0 (not applicable)
void tc_init(Engine &E);
int launch_sfac_tc(Engine &E, int op, int s0, int nsites, int skipconv);
// tensor-core field passes (ewald_tc.cu): mode F_D (dipole field, SOR update, convergence test)
// or F_Q (charge field and potential into F); 1 when launched
int launch_field_tc(Engine &E, int mode, int s0, int s1);
int launch_adj_field_tc(Engine &E);
int launch_adj_dforce_tc(Engine &E);
int launch_adj_qforce_tc(Engine &E);
bool field_pdl_ok(const Engine &E);
int launch_field_qd_tc(Engine &E, int s0, int s1);  // ewald_std_qd force pass on the tensor cores
// launchers (spc.cu): q-SPC/Fw and SPC/F
void launch_sites_spc(Engine &E);
void launch_pair_spc(Engine &E);
void launch_finish_spc(Engine &E);

}  // namespace pimd

// The opaque handle of the C ABI (include/pimd_gb300.h).
struct pimd_ctx {
    pimd::Engine E;
    int check_every = 1;  // host convergence check period of the dipole iterations
    pimd_params params{};  // as created
    // ring-polymer contraction / monomer PIMD (contracted.cu): a one-bead context of the
    // centroid, the mode (0 contracted MTS, 1 monomer PIMD) and the inner steps, device scratch
    pimd_ctx *cen = nullptr;
    int con_mode = -1, con_intra = 0;
    double *d_con = nullptr;
    // run analyses (analysis.cu): geometry accumulator and the centroid O-H pairs of a frame, MSD
    // state, spectra time series (device memory, freed with the context's allocations)
    double *an_geo = nullptr, *an_dcen = nullptr, *an_msd = nullptr;
    int an_msd_ntimes = 0;
    float *an_dip = nullptr, *an_hvel = nullptr;
    int an_nmax = 0, an_n = 0;
    double an_massH = 1.008;
};
