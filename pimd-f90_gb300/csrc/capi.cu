// capi.cu -- context set-up (init_pot / ewald_set) and the force-call C ABI.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/pimd_gb300.h"
#include "engine.h"
#include "nasa_tables.h"

namespace pimd {

// pot_mod.f90:7-44 parameter sets
struct ModelSet {
    double vdwA, vdwB, vdwC, vdwD, vdwE, aDD, aCCaCD, polfacO, polfacH, polfacM, polarO, polarH, polarM,
        gammaM, dms1, dms2, dms3;
};
static const ModelSet TTM21F = {-1.329565985e+6, 3.632560798e+5, -2.147141323e+3, 1.e13, 13.2, 0.3, 0.2,
                                0.837, 0.496, 0.837, 0.837, 0.496, 0.837, 0.426706882, 0.0, 0.0, 0.0};
static const ModelSet TTM3F = {0.0, 0.0, -0.72298855e+03, 0.10211829e+06, 0.37170376e+01, 0.175, 0.175,
                               0.837, 0.496, 0.837, 0.0, 0.0, 1.444, 0.46, 0.5, 0.9578, 0.012};
// q-SPC/Fw and SPC/F (pot_mod.f90:29-44): only the Lennard-Jones A/r^12 + C/r^6 terms are used
static const ModelSet QSPCFW = {629326.57249877361701443513, 0.0, -625.50206521141523463400, 0, 0, 0, 0,
                                0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
static const ModelSet SPCF = {628213.72817108343399678768, 0.0, -624.97858519194071637260, 0, 0, 0, 0,
                              0, 0, 0, 0, 0, 0, 0, 0, 0, 0};

static int fail(Engine &E, int code, const char *msg) {
    E.last_error = msg;
    return code;
}

static int cuda_check(Engine &E, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PIMD_OK;
    char buf[512];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    E.last_error = buf;
    return e == cudaErrorMemoryAllocation ? PIMD_ERR_NOMEM : PIMD_ERR_CUDA;
}

template <typename T>
static int dalloc(Engine &E, T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) return cuda_check(E, e, "cudaMalloc");
    E.allocs.push_back((void *)*p);
    return PIMD_OK;
}

// ewald.f90:293-378 (half-space k list in the reference's loop order) and the run/chunk
// structure used by the kernels.
static int setup_kspace(Engine &E, const pimd_params *p) {
    KP &kp = E.kp;
    const bool explicit_k = p->alpha > 0;
    double kcutsq = 0;
    if (!explicit_k) {
        const double PP = -std::log(p->eps_ewald);
        kp.ew.aewald = std::sqrt(PP) / p->rc;
        const double kcut = 2.0 * kp.ew.aewald * std::sqrt(PP);
        kcutsq = kcut * kcut;
        kp.hmax = (int)std::floor(kcut / TWOPI * p->box[0]);
        kp.kmax = (int)std::floor(kcut / TWOPI * p->box[1]);
        kp.lmax = (int)std::floor(kcut / TWOPI * p->box[2]);
    } else {
        kp.ew.aewald = p->alpha;
        kp.hmax = kp.kmax = kp.lmax = p->nmax;
    }
    if (kp.lmax > 127 || kp.kmax > 127 || kp.hmax > 127) return fail(E, PIMD_ERR_ARG, "k shell too large (max 127)");
    const double a = kp.ew.aewald;
    const double fac_ew2 = -0.25 / (a * a);
    E.h_khkl.clear();
    E.h_kvec.clear();
    E.h_Ak.clear();
    for (int kx = 0; kx <= kp.hmax; kx++) {
        const double k0 = TWOPI * kp.boxi[0] * (double)kx;
        for (int ky = (kx == 0 ? 0 : -kp.kmax); ky <= kp.kmax; ky++) {
            const double k1 = TWOPI * kp.boxi[1] * (double)ky;
            const double kvxy = k0 * k0 + k1 * k1;
            for (int kz = (kx == 0 && ky == 0) ? 1 : -kp.lmax; kz <= kp.lmax; kz++) {
                const double k2 = TWOPI * kp.boxi[2] * (double)kz;
                const double kvsq = kvxy + k2 * k2;
                const bool keep = explicit_k ? (kx * kx + ky * ky + kz * kz <= p->nmax * p->nmax && kvsq > 1.e-16)
                                             : (kvsq < kcutsq && kvsq > 1.e-16);
                if (!keep) continue;
                E.h_khkl.insert(E.h_khkl.end(), {kx, ky, kz});
                E.h_kvec.insert(E.h_kvec.end(), {k0, k1, k2});
                E.h_Ak.push_back(2.0 * std::exp(fac_ew2 * kvsq) / kvsq);
            }
        }
    }
    kp.nk = (int)E.h_Ak.size();
    if (kp.nk == 0) return fail(E, PIMD_ERR_ARG, "empty k-vector set");
    // runs of equal (kx, ky) with consecutive kz
    E.h_runs.clear();
    std::vector<int2> kidx(kp.nk);
    for (int k = 0; k < kp.nk; k++) {
        const int kx = E.h_khkl[3 * k], ky = E.h_khkl[3 * k + 1], kz = E.h_khkl[3 * k + 2];
        if (E.h_runs.empty() || E.h_runs.back().kx != kx || E.h_runs.back().ky != ky) {
            KRun r{};
            r.kx = kx;
            r.ky = ky;
            r.kzlo = kz;
            r.nkz = 0;
            r.kbeg = k;
            E.h_runs.push_back(r);
        }
        KRun &r = E.h_runs.back();
        if (kz != r.kzlo + r.nkz) return fail(E, PIMD_ERR_ARG, "non-contiguous kz run");
        r.nkz++;
        kidx[k] = make_int2((int)E.h_runs.size() - 1, kz);
    }
    kp.nrun = (int)E.h_runs.size();
    // chunks of <= 256 k-vectors and <= 64 runs
    E.h_chunks.clear();
    E.max_runs_chunk = 0;
    KChunk c{0, 0, 0, 0};
    for (int r = 0; r < kp.nrun; r++) {
        const KRun &run = E.h_runs[r];
        if (c.r1 > c.r0 && (run.kbeg + run.nkz - c.k0 > 256 || c.r1 - c.r0 >= 64)) {
            E.h_chunks.push_back(c);
            E.max_runs_chunk = std::max(E.max_runs_chunk, c.r1 - c.r0);
            c = KChunk{run.kbeg, run.kbeg, r, r};
        }
        c.k1 = run.kbeg + run.nkz;
        c.r1 = r + 1;
    }
    E.h_chunks.push_back(c);
    E.max_runs_chunk = std::max(E.max_runs_chunk, c.r1 - c.r0);
    E.nchunk = (int)E.h_chunks.size();
    kp.nchunk = E.nchunk;
    kp.ntab = kp.hmax + 1 + kp.kmax + 1 + kp.lmax + 1;
    // device copies
    int rc;
    KRun *d_runs;
    KChunk *d_chunks;
    double4_32a *d_kinfo;
    double *d_Ak;
    int2 *d_kidx;
    if ((rc = dalloc(E, &d_runs, kp.nrun)) || (rc = dalloc(E, &d_chunks, E.nchunk)) || (rc = dalloc(E, &d_kinfo, kp.nk)) ||
        (rc = dalloc(E, &d_Ak, kp.nk)) || (rc = dalloc(E, &d_kidx, kp.nk)))
        return rc;
    std::vector<double4_32a> kinfo(kp.nk);
    for (int k = 0; k < kp.nk; k++)
        kinfo[k] = make_double4_32a(E.h_kvec[3 * k], E.h_kvec[3 * k + 1], E.h_kvec[3 * k + 2], FOURPI * E.h_Ak[k] / kp.volume);
    cudaMemcpy(d_runs, E.h_runs.data(), sizeof(KRun) * kp.nrun, cudaMemcpyHostToDevice);
    cudaMemcpy(d_chunks, E.h_chunks.data(), sizeof(KChunk) * E.nchunk, cudaMemcpyHostToDevice);
    cudaMemcpy(d_kinfo, kinfo.data(), sizeof(double4_32a) * kp.nk, cudaMemcpyHostToDevice);
    cudaMemcpy(d_Ak, E.h_Ak.data(), sizeof(double) * kp.nk, cudaMemcpyHostToDevice);
    cudaMemcpy(d_kidx, kidx.data(), sizeof(int2) * kp.nk, cudaMemcpyHostToDevice);
    // FP32 copies of the k-vector components for the mixed engine's phase arithmetic
    std::vector<float2> runkf(kp.nrun);
    std::vector<float> kzf(kp.nk);
    for (int r = 0; r < kp.nrun; r++)
        runkf[r] = make_float2((float)E.h_kvec[3 * E.h_runs[r].kbeg], (float)E.h_kvec[3 * E.h_runs[r].kbeg + 1]);
    for (int k = 0; k < kp.nk; k++) kzf[k] = (float)E.h_kvec[3 * k + 2];
    float2 *d_runkf;
    float *d_kzf;
    if ((rc = dalloc(E, &d_runkf, kp.nrun)) || (rc = dalloc(E, &d_kzf, kp.nk))) return rc;
    cudaMemcpy(d_runkf, runkf.data(), sizeof(float2) * kp.nrun, cudaMemcpyHostToDevice);
    cudaMemcpy(d_kzf, kzf.data(), sizeof(float) * kp.nk, cudaMemcpyHostToDevice);
    // per k-vector (k_x, k_y, k_z, Ak) and 2 / k^2 + 1 / (2 alpha^2) in FP32 (mixed reciprocal virial)
    std::vector<float4> kvirf(kp.nk);
    std::vector<float> kc2f(kp.nk);
    for (int k = 0; k < kp.nk; k++) {
        const double kx = E.h_kvec[3 * k], ky = E.h_kvec[3 * k + 1], kz = E.h_kvec[3 * k + 2];
        kvirf[k] = make_float4((float)kx, (float)ky, (float)kz, (float)E.h_Ak[k]);
        kc2f[k] = (float)(2.0 / (kx * kx + ky * ky + kz * kz) + 0.5 / (kp.ew.aewald * kp.ew.aewald));
    }
    float4 *d_kvirf;
    float *d_kc2f;
    if ((rc = dalloc(E, &d_kvirf, kp.nk)) || (rc = dalloc(E, &d_kc2f, kp.nk))) return rc;
    cudaMemcpy(d_kvirf, kvirf.data(), sizeof(float4) * kp.nk, cudaMemcpyHostToDevice);
    cudaMemcpy(d_kc2f, kc2f.data(), sizeof(float) * kp.nk, cudaMemcpyHostToDevice);
    kp.kvirf = d_kvirf;
    kp.kc2f = d_kc2f;
    kp.runkf = d_runkf;
    kp.kzf = d_kzf;
    kp.runs = d_runs;
    kp.chunks = d_chunks;
    kp.kinfo = d_kinfo;
    kp.kAk = d_Ak;
    kp.kidx = d_kidx;
    return cuda_check(E, cudaGetLastError(), "k-space upload");
}

static int create(Engine &E, const pimd_params *p, int nrep, const int *brep) {
    if (!p || p->natoms <= 0 || p->natoms % 3 || p->nbeads < 1) return fail(E, PIMD_ERR_ARG, "natoms/nbeads");
    if (p->pot_model < 2 || p->pot_model > 5) return fail(E, PIMD_ERR_ARG, "pot_model must be 2, 3, 4 or 5");
    const bool spc = p->pot_model >= 4;
    if (spc && p->precision != PIMD_FP64) return fail(E, PIMD_ERR_ARG, "the SPC models run in FP64 only");
    if (!(p->box[0] > 0 && p->box[1] > 0 && p->box[2] > 0)) return fail(E, PIMD_ERR_ARG, "box");
    const double lmin = std::min(p->box[0], std::min(p->box[1], p->box[2]));
    // InputOutput.f90:277-281: the cutoff may not exceed half the box
    if (!(p->rc > 0) || p->rc > 0.5 * lmin) return fail(E, PIMD_ERR_ARG, "rc must be in (0, min(box)/2]");
    if (p->alpha <= 0 && !(p->eps_ewald > 0 && p->eps_ewald < 1)) return fail(E, PIMD_ERR_ARG, "eps_ewald");
    if (p->alpha > 0 && p->nmax < 1) return fail(E, PIMD_ERR_ARG, "nmax");
    if (p->polar_maxiter < 1) return fail(E, PIMD_ERR_ARG, "polar_maxiter must be >= 1");
    if (p->precision != PIMD_FP64 && p->precision != PIMD_MIXED) return fail(E, PIMD_ERR_ARG, "precision");
    int rc = cuda_check(E, cudaSetDevice(p->device), "cudaSetDevice");
    if (rc) return rc;
    E.device = p->device;
    E.precision = p->precision;
    rc = cuda_check(E, cudaStreamCreateWithFlags(&E.stream, cudaStreamNonBlocking), "stream");
    if (rc) return rc;
    E.own_stream = true;
    KP &kp = E.kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.model = p->pot_model;
    kp.natoms = p->natoms;
    kp.N = p->natoms / 3;
    kp.fx_s0 = (kp.model == 3) ? kp.N : 0;  // the first site of the charge field passes
    kp.S = (spc ? 3 : 4) * kp.N;  // potential.f90:53-80: no M site in the SPC models
    kp.fq = spc ? 0 : kp.N;
    kp.P = p->nbeads;
    kp.nrep = nrep;
    for (int c = 0; c < 3; c++) {
        kp.box[c] = p->box[c];
        kp.boxi[c] = 1.0 / p->box[c];
        kp.boxq[c] = (float)(p->box[c] * 0x1p-32);
    }
    kp.volume = p->box[0] * p->box[1] * p->box[2];
    kp.rc2 = p->rc * p->rc;
    kp.rc1 = p->rc1;
    kp.contraction = p->contraction;
    kp.guess = p->guess_initdip;
    kp.polar_maxiter = p->polar_maxiter;
    kp.polar_sor = p->polar_sor;
    kp.polar_eps = p->polar_eps;
    const ModelSet &m = (p->pot_model == 2) ? TTM21F : (p->pot_model == 3) ? TTM3F : (p->pot_model == 4) ? QSPCFW : SPCF;
    kp.vdwA = m.vdwA;
    kp.vdwB = m.vdwB;
    kp.vdwC = m.vdwC;
    kp.vdwD = m.vdwD;
    kp.vdwE = m.vdwE;
    kp.gammaM = m.gammaM;
    kp.dms1 = m.dms1;
    kp.dms2 = m.dms2;
    kp.dms3 = m.dms3;
    kp.polar[1] = m.polarO;
    kp.polar[2] = m.polarH;
    kp.polar[3] = m.polarH;
    kp.polar[4] = m.polarM;
    kp.same_acd = std::fabs(m.aCCaCD - m.aDD) < 1.e-12 ? 1 : 0;
    if (p->pot_model == 3 && p->rc != p->rc1) {
        // potential.f90:106-113 GROMACS-style vdW force switch
        const double Rc = p->rc, r1 = p->rc1;
        const double rc8 = Rc * Rc * Rc * Rc * Rc * Rc * Rc * Rc;
        kp.shiftA = -(10 * Rc - 7 * r1) / (rc8 * ((Rc - r1) * (Rc - r1)));
        kp.shiftB = (9 * Rc - 7 * r1) / (rc8 * ((Rc - r1) * (Rc - r1) * (Rc - r1)));
    }
    if (spc) {  // pot_mod.f90:29-44
        const bool q = p->pot_model == 4;
        kp.qO = q ? -0.84 : -0.82;
        kp.qH = q ? 0.42 : 0.41;
        kp.roh0 = q ? 1.012 : 1.0;
        kp.th0 = q ? 1.95476876223364912614 : 1.91061193215819258784;
        kp.harmkb = q ? 529.581 : 0.0;
        kp.harmka = q ? 37.95 : 0.0;
        kp.fd = kp.ld = 0;
        kp.ndd = 0;
    } else if (p->pot_model == 2) {
        kp.fd = 0;
        kp.ld = 3 * kp.N;
        kp.ndd = 9;
    } else {
        kp.fd = 3 * kp.N;
        kp.ld = 4 * kp.N;
        kp.ndd = 1;
    }
    {  // potential.f90:152-154 long-range vdW correction
        const double Rc = p->rc, r3 = Rc * Rc * Rc, r7 = r3 * r3 * Rc, r9 = r7 * Rc * Rc;
        kp.Uvdw_lrc = TWOPI * (double)(kp.N * kp.N) / kp.volume * (m.vdwA / (9.0 * r9) + m.vdwB / (7.0 * r7) + m.vdwC / (3.0 * r3));
    }
    // potential.f90:157-160 polfac = polfac^(-1/2) by way of the sixth root
    double pf[5];
    const double base[5] = {0, m.polfacO, m.polfacH, m.polfacH, m.polfacM};
    for (int i = 1; i <= 4; i++) {
        const double r = std::pow(base[i], 1.0 / 6.0);
        pf[i] = spc ? 0.0 : 1.0 / (r * r * r);
    }
    for (int i = 1; i <= 4; i++) E.polfac[i] = pf[i];
    // the differentiable parameters start at the published values
    E.theta[PIMD_TH_POLAR_M] = m.polarM;
    E.theta[PIMD_TH_A_DD] = m.aDD;
    E.theta[PIMD_TH_A_CC] = m.aCCaCD;
    E.theta[PIMD_TH_VDW_C] = m.vdwC;
    E.theta[PIMD_TH_VDW_D] = m.vdwD;
    E.theta[PIMD_TH_VDW_E] = m.vdwE;
    E.theta[PIMD_TH_DMS1] = m.dms1;
    E.theta[PIMD_TH_DMS2] = m.dms2;
    E.theta[PIMD_TH_DMS3] = m.dms3;
    E.theta[PIMD_TH_GAMMA_M] = m.gammaM;
    E.theta[PIMD_TH_F5Z] = PIMD_NASA_F5Z;
    E.theta[PIMD_TH_FBASIS] = PIMD_NASA_FBASIS;
    E.theta[PIMD_TH_FCORE] = PIMD_NASA_FCORE;
    E.theta[PIMD_TH_FREST] = PIMD_NASA_FREST;
    kp.nasa_f5z = PIMD_NASA_F5Z;
    E.vdwA_model = m.vdwA;
    E.vdwB_model = m.vdwB;
    E.rc = p->rc;
    for (int i = 1; i <= 4; i++)
        for (int j = 1; j <= 4; j++) {
            kp.pt.apol_qq[i][j] = (m.aCCaCD * pf[i]) * pf[j];
            kp.pt.ra_qq[i][j] = std::pow(kp.pt.apol_qq[i][j], 1.0 / 3.0);
            kp.pt.apol_dd[i][j] = (m.aDD * pf[i]) * pf[j];
            kp.pt.apol_cd[i][j] = (m.aCCaCD * pf[i]) * pf[j];
        }
    if ((rc = setup_kspace(E, p))) return rc;
    const double a = kp.ew.aewald;
    kp.ew.a2 = a * a;
    kp.ew.cts1 = 2.0 * a / SQPI;
    kp.ew.cts2 = 4.0 * a * a * a / (3.0 * SQPI);
    kp.ew.cts3 = 8.0 * (a * a * a * a * a) / (15.0 * SQPI);
    kp.ewf = EwCf{(float)kp.ew.aewald, (float)kp.ew.a2, (float)kp.ew.cts1, (float)kp.ew.cts2, (float)kp.ew.cts3};
    kp_float_tables(kp);
    kp.stath = DEBYE / CHARGECON / std::sqrt((double)kp.natoms);
    kp.factor = 4.0 * (a * a * a) / (3.0 * std::sqrt(PI));
    // neighbour-list capacity: 3x the expected O-O pairs, at most all pairs
    const double shell = 4.0 / 3.0 * PI * p->rc * p->rc * p->rc / kp.volume;
    const double est = 0.5 * kp.N * (double)kp.N * shell;
    const double all = 0.5 * kp.N * (double)(kp.N - 1);
    E.cap = (size_t)std::max(1.0, std::min(all, std::max(1024.0, 3.0 * est)));
    kp.cap = (int)E.cap;
    const size_t P = kp.P, S = kp.S, N = kp.N;
    const int nsq = kp.S - kp.fq, nsd = kp.ld - kp.fd;
    // structure-factor partials: at most one site group per 32-site tile, at most 32 groups, and
    // at most ~256 MB for all beads (large boxes have enough k-vectors to fill the GPU anyway)
    const size_t tiles = (size_t)std::max((nsq + 31) / 32, (nsd + 31) / 32);
    const size_t memcap = std::max<size_t>(1, (256ull << 20) / (P * (size_t)kp.nk * 3 * sizeof(double2)));
    const size_t maxgroups = std::max<size_t>(1, std::min<size_t>(std::min<size_t>(tiles, 32), memcap));
    E.sp_cap = (int)maxgroups;
    if ((rc = dalloc(E, (double **)&kp.RRt, P * kp.natoms * 3)) || (rc = dalloc(E, (double **)&kp.RRc, (size_t)kp.nrep * kp.natoms * 3)) ||
        (rc = dalloc(E, &kp.dRRt, P * kp.natoms * 3)) || (rc = dalloc(E, &kp.dipI, P * N * 3)) ||
        (rc = dalloc(E, &kp.dipE, P * N * 3)) || (rc = dalloc(E, &kp.chg, P * kp.natoms)) ||
        (rc = dalloc(E, &kp.pos, P * S)) || (rc = dalloc(E, &kp.posc, (size_t)kp.nrep * S)) || (rc = dalloc(E, &kp.F, P * S)) ||
        (rc = dalloc(E, &kp.dR, P * S * 3)) || (rc = dalloc(E, &kp.dip, P * S * 3)) || (rc = dalloc(E, &kp.Efdr, P * S * 3)) ||
        (rc = dalloc(E, &kp.txdip, P * 4 * S * 3)) || (rc = dalloc(E, &kp.grdq, P * N * 27)) ||
        (rc = dalloc(E, &kp.Tdd, P * E.cap * kp.ndd * 6)) || (rc = dalloc(E, &kp.Tself, P * N * 18)) ||
        (rc = dalloc(E, &kp.pairs, P * E.cap)) || (rc = dalloc(E, &kp.npair, P)) ||
        (rc = dalloc(E, &kp.tab, P * kp.ntab * S)) || (rc = dalloc(E, &kp.Spart, P * maxgroups * kp.nk * 3)) ||
        (rc = dalloc(E, &kp.Sq, P * kp.nk)) || (rc = dalloc(E, &kp.Sm, P * kp.nk)) || (rc = dalloc(E, &kp.Sdip, P * kp.nk * 3)) ||
        (rc = dalloc(E, &kp.acc, P * NACC)) || (rc = dalloc(E, &kp.err, 1)) || (rc = dalloc(E, &kp.allconv, 1)) ||
        (rc = dalloc(E, &kp.dstep, 2)) || (rc = dalloc(E, &kp.fin_counter, 1)) ||
        (rc = dalloc(E, &kp.nbrtmp, P * N)) || (rc = dalloc(E, &E.d_out, 3 * P + 16)) ||
        (rc = dalloc(E, &kp.Fpart, (size_t)E.max_slices * P * S)))
        return rc;
    if (E.precision == PIMD_MIXED) {
        kp.fcap = (int)std::min(2.0 * E.cap, (double)kp.N * (kp.N - 1));
        if ((rc = dalloc(E, &kp.tabf, P * kp.ntab * S)) || (rc = dalloc(E, &kp.posf, P * S)) ||
            (rc = dalloc(E, &kp.rhof, P * S)) || (rc = dalloc(E, &kp.fcnt, P * N)) || (rc = dalloc(E, &kp.foff, P * N)) ||
            (rc = dalloc(E, &kp.fnbr, P * (size_t)kp.fcap * 2)) || (rc = dalloc(E, &kp.fntot, P)) ||
            (rc = dalloc(E, &kp.Tf, P * (size_t)kp.fcap * kp.ndd)) || (rc = dalloc(E, &kp.fj, P * (size_t)kp.fcap)) || (rc = dalloc(E, &kp.Wf, P * 2 * (size_t)kp.nk)) || (rc = dalloc(E, &kp.dipf, P * S)) ||
            (rc = dalloc(E, &kp.ofix, P * N)) || (rc = dalloc(E, &kp.orawf, P * N)) || (rc = dalloc(E, &kp.Fx, P * S)) ||
            (rc = dalloc(E, &kp.dipf_alt, P * S)) || (rc = dalloc(E, &kp.Erec, P * S)) ||
            (kp.model == 3 && (rc = dalloc(E, &kp.mrec, P * 2 * (size_t)N))) ||
            (rc = dalloc(E, &kp.unit_cnt, P * ((size_t)S / 128 + 2))))
            return rc;
        cudaMemset(kp.unit_cnt, 0, sizeof(unsigned) * P * ((size_t)S / 128 + 2));
        kp.unit_sbase = kp.fd & ~31;  // the field pass's first CTA (TMA-aligned site base)
        kp.nunits = (kp.ld - kp.unit_sbase + 127) / 128;
    }
    // cell lists for boxes beyond the one-block neighbour kernel (cells of width >= Rc + 1e-3 A)
    kp.cl_ncell = 0;
    if (N > 1024) {
        bool ok = true;
        for (int d = 0; d < 3; d++) {
            kp.cl_n[d] = (int)std::floor(p->box[d] / (p->rc + 1e-3));
            ok = ok && kp.cl_n[d] >= 4;
        }
        if (ok) {
            kp.cl_ncell = kp.cl_n[0] * kp.cl_n[1] * kp.cl_n[2];
            if ((rc = dalloc(E, &kp.cl_mol, P * N)) || (rc = dalloc(E, &kp.cl_posf, P * N)) ||
                (rc = dalloc(E, &kp.cl_cnt, P * (size_t)kp.cl_ncell)) ||
                (rc = dalloc(E, &kp.cl_start, P * (size_t)(kp.cl_ncell + 1))) || (rc = dalloc(E, &kp.cl_list, P * N)) ||
                (rc = dalloc(E, &kp.cl_row, P * N * 256)) || (rc = dalloc(E, &kp.cl_rowlen, P * N)))
                return rc;
        }
    }
    cudaMemset(kp.txdip, 0, sizeof(double) * P * 4 * S * 3);
    cudaMemset(kp.Sm, 0, sizeof(double2) * P * kp.nk);
    if (kp.Wf) cudaMemset(kp.Wf, 0, sizeof(float2) * P * 2 * kp.nk);
    cudaMemset(kp.err, 0, sizeof(unsigned));
    if ((rc = cuda_check(E, cudaMallocHost((void **)&E.h_allconv, sizeof(int)), "cudaMallocHost"))) return rc;
    cudaMemset(kp.dstep, 0, sizeof(int) * 2);
    cudaMemset(kp.fin_counter, 0, sizeof(unsigned));
    if (nrep > 1) {
        int *d_brep;
        if ((rc = dalloc(E, &d_brep, P))) return rc;
        cudaMemcpy(d_brep, brep, sizeof(int) * P, cudaMemcpyHostToDevice);
        kp.brep = d_brep;
    }
    pot_init_constants(E);
    ewald_init(E);
    if (E.precision == PIMD_MIXED && (rc = cuda_check(E, mixed_init(E), "mixed tables"))) return rc;
    neighbors_init(E);
    if (kp.model == 3) adjoint_init(E);
    return cuda_check(E, cudaDeviceSynchronize(), "init");
}

int create_context(Engine &E, const pimd_params *p, int nrep, const int *brep) {
    if (nrep < 1 || (nrep > 1 && !brep)) return fail(E, PIMD_ERR_ARG, "replicas");
    return create(E, p, nrep, brep);
}

// ---------------------------------------------------------------------------------------
// Phase timers: a pair of events around each named phase on the engine stream.
static int timer_slot(PhaseTimers &T, const char *name) {
    for (size_t i = 0; i < T.names.size(); i++)
        if (T.names[i] == name) return (int)i;
    T.names.push_back(name);
    T.ms.push_back(0.0);
    T.count.push_back(0);
    return (int)T.names.size() - 1;
}

static cudaEvent_t timer_event(PhaseTimers &T) {
    if (!T.pool.empty()) {
        cudaEvent_t e = T.pool.back();
        T.pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

static void timer_resolve(Engine &E) {
    PhaseTimers &T = E.timers;
    if (T.pending.empty()) return;
    cudaEventSynchronize(T.pending.back().second.second);
    for (auto &p : T.pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.second.first, p.second.second);
        T.ms[p.first] += ms;
        T.count[p.first] += 1;
        T.pool.push_back(p.second.first);
        T.pool.push_back(p.second.second);
    }
    T.pending.clear();
}

void timer_begin(Engine &E, const char *name) {
    PhaseTimers &T = E.timers;
    if (!T.on) return;
    if (T.pending.size() > 8192) timer_resolve(E);
    T.cur = timer_slot(T, name);
    T.cur0 = timer_event(T);
    cudaEventRecord(T.cur0, E.stream);
}

void timer_end(Engine &E) {
    PhaseTimers &T = E.timers;
    if (!T.on || T.cur < 0) return;
    cudaEvent_t e1 = timer_event(T);
    cudaEventRecord(e1, E.stream);
    T.pending.push_back({T.cur, {T.cur0, e1}});
    T.cur = -1;
}

#define PHASE(name, call) \
    do {                  \
        timer_begin(E, name); \
        call;             \
        timer_end(E);     \
    } while (0)

// One induced-dipole iteration (pot_ttm.f90:298-390): real-space dipole field, ewald_std_dd
// structure factor, field + SOR update, convergence test.
static void dipole_iteration(Engine &E, bool mixed, bool body_start = false) {
    if (mixed && E.loop_aux && E.dd_overlap) {
        // the real-space field runs on the second stream beside the structure factor (both only
        // read the iteration's dipoles); the field + SOR pass waits for both
        cudaEventRecord(E.loop_fork, E.stream);
        cudaStreamWaitEvent(E.loop_aux, E.loop_fork, 0);
        // first iteration of a graph loop body: nothing gives the structure factor a head start
        // (later ones are programmatic dependents of the field pass), so the real-space blocks
        // would fill the SMs first; they wait until the structure factor's CTAs are resident
        E.sfac_pev_req = body_start && E.dd_pev && E.loop_pev;
        E.sfac_pev_armed = false;
        PHASE("dd_smu", launch_ewald_smu(E));
        if (E.sfac_pev_armed) cudaStreamWaitEvent(E.loop_aux, E.loop_pev, 0);
        E.sfac_pev_req = false;
        cudaStream_t keep = E.stream;
        E.stream = E.loop_aux;
        // the field pass, a programmatic dependent of the structure factor, may also start as
        // the real-space field drains when its griddepcontrol.wait covers that grid too
        E.dd_jpev_req = E.dd_jpev && !E.kp.dd_async && field_pdl_ok(E);
        E.dd_jpev_armed = false;
        PHASE("dd_real", launch_dd_real_m(E));
        E.dd_jpev_req = false;
        E.stream = keep;
        cudaEventRecord(E.loop_join, E.loop_aux);
        // asynchronous: the field pass runs beside the real-space field as well (whichever ends
        // a unit of sites last updates its dipoles); the iteration ends when both are done
        if (E.dd_jpev_armed)
            cudaStreamWaitEvent(E.stream, E.loop_jpev, 0);
        else if (!E.kp.dd_async)
            cudaStreamWaitEvent(E.stream, E.loop_join, 0);
        E.field_needs_join = E.dd_jpev_armed;
        PHASE("dd_update", launch_dd_update(E));  // includes the convergence test (last block)
        E.field_needs_join = false;
        if (E.kp.dd_async || E.dd_jpev_armed) cudaStreamWaitEvent(E.stream, E.loop_join, 0);
        return;
    }
    if (mixed)
        PHASE("dd_real", launch_dd_real_m(E));
    else
        PHASE("dd_real", launch_dd_real(E));
    PHASE("dd_smu", launch_ewald_smu(E));
    PHASE("dd_update", launch_dd_update(E));  // includes the convergence test (last block)
}

// While capturing a CUDA graph: the dipole iterations become a conditional while node whose
// body is one iteration; the convergence test in the field pass's last block sets the condition
// on the device, so the loop runs with
// no host round trip and stops at convergence (or polar_maxiter) exactly like the host loop.
static int capture_dipole_loop(Engine &E, bool mixed) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(E.stream, &st, nullptr, &g, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return cuda_check(E, e, "cudaStreamGetCaptureInfo");
    if (st != cudaStreamCaptureStatusActive) return fail(E, PIMD_ERR_STATE, "dipole loop capture outside a capture");
    cudaGraphConditionalHandle h;
    e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return cuda_check(E, e, "cudaGraphConditionalHandleCreate");
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};  // aggregate init zeroes the rest
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp);
    if (e != cudaSuccess) return cuda_check(E, e, "conditional node");
    e = cudaStreamUpdateCaptureDependencies(E.stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return cuda_check(E, e, "cudaStreamUpdateCaptureDependencies");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(E.body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_check(E, e, "body capture");
    cudaStream_t keep = E.stream;
    E.stream = E.body_stream;
    E.kp.cond = h;
    // iterations per body: 3 divides the conditional's relaunches by three; an iteration after every bead
    // has converged is empty (each kernel returns at the bead's flag, the test leaves the
    // per-bead counts alone)
    for (int u = 0; u < std::max(1, E.loop_unroll); u++) dipole_iteration(E, mixed, u == 0);
    E.kp.cond = 0;
    E.stream = keep;
    cudaGraph_t out = nullptr;
    e = cudaStreamEndCapture(E.body_stream, &out);
    return cuda_check(E, e, "body capture end");
}

// One force call for all beads of the context (pot_ttm.f90:3-630 per bead).
int run_forces(Engine &E, int t, int check_every, double *Upott, double *virialt, double *virialct, double *virt9) {
    KP &kp = E.kp;
    kp.t = t;
    cudaMemsetAsync(kp.acc, 0, sizeof(double) * kp.P * NACC, E.stream);
    cudaMemsetAsync(kp.err, 0, sizeof(unsigned), E.stream);
    if (E.capturing)
        cudaMemsetAsync(kp.dstep + 1, 0, sizeof(int), E.stream);  // t is set before each graph launch
    else
        launch_set_step(E, t);
    const bool mixed = E.precision == PIMD_MIXED;
    if (kp.model >= 4) {  // pot_spc.f90: no induced dipoles
        PHASE("sites", launch_sites_spc(E));
        PHASE("neighbors", launch_neighbors(E));
        PHASE("pair_qq", launch_pair_spc(E));
        PHASE("ewald_tables", launch_ewald_tables(E));
        PHASE("ewald_pw", launch_ewald_pw(E));
        PHASE("finish", launch_finish_spc(E));
        E.last_niter_max = 0;
        PHASE("totals", launch_totals(E, Upott, virialt, virialct, virt9));
        return cuda_check(E, cudaGetLastError(), "force kernels");
    }
    // mixed engine with the tensor-core field passes: the reciprocal charge passes run on the
    // second stream beside the neighbour list and the charge pair gather, and the force pass
    // beside the force pair gather; their field / gradient sums go to the scratch Fx, which
    // k_after_qq and k_finish add (the pair kernels update F and dR in place). The neighbour
    // lists, which need only the input O sites, are built on the second stream beside k_sites.
    const bool ovl = mixed && E.ewald_overlap && E.aux_stream && kp.Fx && E.tc_ready && E.tf_ready && E.ff_tc;
    const bool ovq = ovl, ovf = ovl && E.tf_qd_ready;
    const bool nbe = ovq && E.nbr_overlap && E.ev_nbr && nbr_from_inputs(E);
    if (nbe) {
        cudaEventRecord(E.ev_fork, E.stream);
        cudaStreamWaitEvent(E.aux_stream, E.ev_fork, 0);
        cudaStream_t keep = E.stream;
        E.stream = E.aux_stream;
        PHASE("neighbors", launch_neighbors(E));
        E.stream = keep;
        cudaEventRecord(E.ev_nbr, E.aux_stream);
    }
    PHASE("sites", launch_sites(E));
    kp.fx_mode = 0;
    if (mixed) {
        PHASE("site_offsets", launch_site_offsets(E));
        if (ovq) {
            cudaEventRecord(E.ev_fork, E.stream);
            cudaStreamWaitEvent(E.aux_stream, E.ev_fork, 0);
            cudaStream_t keep = E.stream;
            E.stream = E.aux_stream;
            kp.fx_mode = 1;
            PHASE("ewald_tables", launch_ewald_tables(E));
            PHASE("ewald_sq", launch_ewald_sq(E));
            PHASE("ewald_fq", launch_ewald_fq(E));
            kp.fx_mode = 0;
            // the iterations' dipole-pair scalars fill this stream's slack beside the charge
            // gather (after the full lists this stream built)
            if (nbe) PHASE("dd_tensors", launch_dd_tensors_m(E));
            E.stream = keep;
            cudaEventRecord(E.ev_join, E.aux_stream);
        }
        if (nbe)
            cudaStreamWaitEvent(E.stream, E.ev_nbr, 0);
        else
            PHASE("neighbors", launch_neighbors(E));
        PHASE("pair_qq", launch_pair_qq_m(E));
        if (!nbe) PHASE("dd_tensors", launch_dd_tensors_m(E));
    } else {
        PHASE("neighbors", launch_neighbors(E));
        PHASE("pair_qq", launch_pair_qq(E));
    }
    if (ovq) {
        cudaStreamWaitEvent(E.stream, E.ev_join, 0);
        kp.fx_mode = 1;
    } else {
        PHASE("ewald_tables", launch_ewald_tables(E));
        PHASE("ewald_sq", launch_ewald_sq(E));
        PHASE("ewald_fq", launch_ewald_fq(E));
    }
    PHASE("after_qq", launch_after_qq(E));
    kp.fx_mode = 0;
    if (E.tape_on) tape_record(E, 0);
    kp.dd_async = (mixed && dd_async_ok(E)) ? 1 : 0;
    if (E.capturing) {
        int rc = capture_dipole_loop(E, mixed);
        if (rc) {
            kp.dd_async = 0;
            return rc;
        }
        E.last_niter_max = -1;  // known on the device only
    } else {
        int iter = 1;
        for (; iter <= kp.polar_maxiter; iter++) {
            dipole_iteration(E, mixed);
            if (E.tape_on) tape_record(E, iter);
            if (check_every > 0 && (iter % check_every) == 0 && iter < kp.polar_maxiter) {
                cudaMemcpyAsync(E.h_allconv, kp.allconv, sizeof(int), cudaMemcpyDeviceToHost, E.stream);
                cudaError_t e = cudaStreamSynchronize(E.stream);
                if (e != cudaSuccess) return cuda_check(E, e, "dipole iteration");
                if (*E.h_allconv) break;
            }
        }
        E.last_niter_max = std::min(iter, kp.polar_maxiter);
    }
    if (kp.dd_async) {
        PHASE("dipf_sync", launch_dipf_sync(E));
        kp.dd_async = 0;
    }
    if (ovf) {
        cudaEventRecord(E.ev_fork, E.stream);
        cudaStreamWaitEvent(E.aux_stream, E.ev_fork, 0);
        cudaStream_t keep = E.stream;
        E.stream = E.aux_stream;
        kp.fx_mode = 2;
        PHASE("ewald_qd", launch_ewald_qd(E));
        kp.fx_mode = 0;
        E.stream = keep;
        cudaEventRecord(E.ev_join, E.aux_stream);
        PHASE("pair_force", launch_pair_force_m(E));
        cudaStreamWaitEvent(E.stream, E.ev_join, 0);
        kp.fx_mode = 2;
    } else {
        if (mixed)
            PHASE("pair_force", launch_pair_force_m(E));
        else
            PHASE("pair_force", launch_pair_force(E));
        PHASE("ewald_qd", launch_ewald_qd(E));
    }
    PHASE("finish", launch_finish(E));
    kp.fx_mode = 0;
    PHASE("totals", launch_totals(E, Upott, virialt, virialct, virt9));
    return cuda_check(E, cudaGetLastError(), "force kernels");
}

static int read_err(Engine &E) {
    unsigned err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, E.kp.err, sizeof(unsigned), cudaMemcpyDeviceToHost, E.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(E.stream);
    if (e != cudaSuccess) return cuda_check(E, e, "force call");
    if (err & 1u) return fail(E, PIMD_ERR_NEIGHBOR_OVERFLOW, "neighbour list capacity exceeded");
    if (err & 4u) return fail(E, PIMD_ERR_GAMMQ, "gammq2_3 did not converge");
    if (err & 8u) return fail(E, PIMD_ERR_CUDA, "tensor-core structure factor: pipeline wait timed out");
    return PIMD_OK;
}

}  // namespace pimd

using namespace pimd;

extern "C" {

int pimd_create(pimd_ctx **ctx, const pimd_params *p) {
    if (!ctx) return PIMD_ERR_ARG;
    *ctx = nullptr;
    pimd_ctx *c = new pimd_ctx();
    if (p) c->params = *p;
    int rc = create(c->E, p, 1, nullptr);
    if (rc) {
        fprintf(stderr, "pimd_create: %s\n", c->E.last_error.c_str());
        pimd_destroy(c);
        return rc;
    }
    *ctx = c;
    return PIMD_OK;
}

int pimd_destroy(pimd_ctx *ctx) {
    if (!ctx) return PIMD_OK;
    if (ctx->cen) pimd_destroy(ctx->cen);
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    if (E.stream) cudaStreamSynchronize(E.stream);
    for (void *p : E.allocs) cudaFree(p);
    if (E.d_nmC) cudaFree(E.d_nmC);
    if (E.d_nmA) cudaFree(E.d_nmA);
    for (cudaEvent_t e : E.timers.pool) cudaEventDestroy(e);
    for (auto &pe : E.timers.pending) {
        cudaEventDestroy(pe.second.first);
        cudaEventDestroy(pe.second.second);
    }
    if (E.h_allconv) cudaFreeHost(E.h_allconv);
    if (E.h_pin) cudaFreeHost(E.h_pin);
    if (E.d_tape) cudaFree(E.d_tape);
    if (E.d_phiq) cudaFree(E.d_phiq);
    if (E.d_tapeS) cudaFree(E.d_tapeS);
    if (E.d_adj) cudaFree(E.d_adj);
    if (E.gexec) cudaGraphExecDestroy(E.gexec);
    if (E.body_stream) cudaStreamDestroy(E.body_stream);
    if (E.aux_stream) cudaStreamDestroy(E.aux_stream);
    if (E.ev_fork) cudaEventDestroy(E.ev_fork);
    if (E.ev_join) cudaEventDestroy(E.ev_join);
    if (E.ev_nbr) cudaEventDestroy(E.ev_nbr);
    if (E.loop_aux) cudaStreamDestroy(E.loop_aux);
    if (E.loop_fork) cudaEventDestroy(E.loop_fork);
    if (E.loop_pev) cudaEventDestroy(E.loop_pev);
    if (E.loop_jpev) cudaEventDestroy(E.loop_jpev);
    if (E.loop_join) cudaEventDestroy(E.loop_join);
    if (E.own_stream && E.stream) cudaStreamDestroy(E.stream);
    delete ctx;
    return PIMD_OK;
}

int pimd_set_stream(pimd_ctx *ctx, void *s) {
    if (!ctx) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (s && (cudaStream_t)s != E.stream) {
        if (E.own_stream && E.stream) cudaStreamDestroy(E.stream);
        E.stream = (cudaStream_t)s;
        E.own_stream = false;
    }
    return PIMD_OK;
}

const char *pimd_last_error(pimd_ctx *ctx) { return ctx ? ctx->E.last_error.c_str() : "null context"; }

int pimd_ewald_info(pimd_ctx *ctx, double *alpha, int *nk, int *hkl_max) {
    if (!ctx) return PIMD_ERR_ARG;
    const KP &kp = ctx->E.kp;
    if (alpha) *alpha = kp.ew.aewald;
    if (nk) *nk = kp.nk;
    if (hkl_max) {
        hkl_max[0] = kp.hmax;
        hkl_max[1] = kp.kmax;
        hkl_max[2] = kp.lmax;
    }
    return PIMD_OK;
}

int pimd_set_dipole_check(pimd_ctx *ctx, int every) {
    if (!ctx || every < 0) return PIMD_ERR_ARG;
    ctx->check_every = every;
    return PIMD_OK;
}

int pimd_full_bead_forces_device(pimd_ctx *ctx, const double *RRt, const double *RRc, double *Upott, double *dRRt,
                                 double *virialt, double *virialct, double *dip_momIt, double *dip_momEt, double *chg,
                                 int t) {
    if (!ctx || !RRt || !RRc) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    KP saved = E.kp;
    E.kp.RRt = RRt;
    E.kp.RRc = RRc;
    if (dRRt) E.kp.dRRt = dRRt;
    if (dip_momIt) E.kp.dipI = dip_momIt;
    if (dip_momEt) E.kp.dipE = dip_momEt;
    int rc = run_forces(E, t, ctx->check_every, Upott, virialt, virialct, nullptr);
    if (!rc && chg)
        rc = cuda_check(E, cudaMemcpyAsync(chg, E.kp.chg + (size_t)(E.kp.P - 1) * E.kp.natoms, sizeof(double) * E.kp.natoms,
                                           cudaMemcpyDeviceToDevice, E.stream), "chg");
    const double *keepRRt = saved.RRt, *keepRRc = saved.RRc;
    double *kd = saved.dRRt, *ki = saved.dipI, *ke = saved.dipE;
    E.kp.RRt = keepRRt;
    E.kp.RRc = keepRRc;
    E.kp.dRRt = kd;
    E.kp.dipI = ki;
    E.kp.dipE = ke;
    return rc;
}

int pimd_full_bead_forces(pimd_ctx *ctx, const double *RRt, const double *RRc, double *Upott, double *dRRt,
                          double *virialt, double *virialct, double *dip_momIt, double *dip_momEt, double *chg, int t) {
    if (!ctx || !RRt || !RRc) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    KP &kp = E.kp;
    const size_t P = kp.P, na = kp.natoms, nw = kp.N;
    cudaMemcpyAsync((void *)kp.RRt, RRt, sizeof(double) * P * na * 3, cudaMemcpyHostToDevice, E.stream);
    cudaMemcpyAsync((void *)kp.RRc, RRc, sizeof(double) * na * 3, cudaMemcpyHostToDevice, E.stream);
    double *d_out = E.d_out;  // Upott, virialt, virialct staged on the device
    int rc = run_forces(E, t, ctx->check_every, d_out, d_out + P, d_out + 2 * P, nullptr);
    if (!rc) {
        std::vector<double> h(3 * P);
        cudaMemcpyAsync(h.data(), d_out, sizeof(double) * 3 * P, cudaMemcpyDeviceToHost, E.stream);
        if (dRRt) cudaMemcpyAsync(dRRt, kp.dRRt, sizeof(double) * P * na * 3, cudaMemcpyDeviceToHost, E.stream);
        if (dip_momIt) cudaMemcpyAsync(dip_momIt, kp.dipI, sizeof(double) * P * nw * 3, cudaMemcpyDeviceToHost, E.stream);
        if (dip_momEt) cudaMemcpyAsync(dip_momEt, kp.dipE, sizeof(double) * P * nw * 3, cudaMemcpyDeviceToHost, E.stream);
        if (chg) cudaMemcpyAsync(chg, kp.chg + (P - 1) * na, sizeof(double) * na, cudaMemcpyDeviceToHost, E.stream);
        rc = read_err(E);
        if (!rc) {
            if (Upott) std::copy(h.begin(), h.begin() + P, Upott);
            if (virialt) std::copy(h.begin() + P, h.begin() + 2 * P, virialt);
            if (virialct) std::copy(h.begin() + 2 * P, h.end(), virialct);
        }
    }
    cudaStreamSynchronize(E.stream);
    return rc;
}

int pimd_pot_ttm(pimd_ctx *ctx, const double *RR, const double *RRc, double *En, double *dRR, double *virt,
                 double *virialc, double *dip_momI, double *Edip_mom, double *chg, int t) {
    if (!ctx || !RR || !RRc) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    KP saved = E.kp;
    E.kp.P = 1;  // bead-0 view of the context
    const size_t na = E.kp.natoms, nw = E.kp.N;
    cudaMemcpyAsync((void *)E.kp.RRt, RR, sizeof(double) * na * 3, cudaMemcpyHostToDevice, E.stream);
    cudaMemcpyAsync((void *)E.kp.RRc, RRc, sizeof(double) * na * 3, cudaMemcpyHostToDevice, E.stream);
    double *d_out = E.d_out;  // En, virialc, virt(9)
    int rc = run_forces(E, t, ctx->check_every, d_out, nullptr, d_out + 1, d_out + 2);
    if (!rc) {
        double h[12];
        cudaMemcpyAsync(h, d_out, sizeof(h) - sizeof(double), cudaMemcpyDeviceToHost, E.stream);
        if (dRR) cudaMemcpyAsync(dRR, E.kp.dRRt, sizeof(double) * na * 3, cudaMemcpyDeviceToHost, E.stream);
        if (dip_momI) cudaMemcpyAsync(dip_momI, E.kp.dipI, sizeof(double) * nw * 3, cudaMemcpyDeviceToHost, E.stream);
        if (Edip_mom) cudaMemcpyAsync(Edip_mom, E.kp.dipE, sizeof(double) * nw * 3, cudaMemcpyDeviceToHost, E.stream);
        if (chg) cudaMemcpyAsync(chg, E.kp.chg, sizeof(double) * na, cudaMemcpyDeviceToHost, E.stream);
        rc = read_err(E);
        if (!rc) {
            if (En) *En = h[0];
            if (virialc) *virialc = h[1];
            if (virt) std::copy(h + 2, h + 11, virt);
        }
    }
    cudaStreamSynchronize(E.stream);
    E.kp = saved;
    return rc;
}

int pimd_pot_spc(pimd_ctx *ctx, const double *RR, double *En, double *dRR, double *virt, double *dip_momI,
                 double *chg) {
    if (!ctx || !RR) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (E.kp.model < 4) return fail(E, PIMD_ERR_ARG, "context was not created for pot_model 4/5");
    cudaSetDevice(E.device);
    KP saved = E.kp;
    E.kp.P = 1;  // bead-0 view of the context
    const size_t na = E.kp.natoms, nw = E.kp.N;
    cudaMemcpyAsync((void *)E.kp.RRt, RR, sizeof(double) * na * 3, cudaMemcpyHostToDevice, E.stream);
    double *d_out = E.d_out;  // En, (unused), virt(9)
    int rc = run_forces(E, 0, ctx->check_every, d_out, nullptr, nullptr, d_out + 2);
    if (!rc) {
        double h[11];
        cudaMemcpyAsync(h, d_out, sizeof(h), cudaMemcpyDeviceToHost, E.stream);
        if (dRR) cudaMemcpyAsync(dRR, E.kp.dRRt, sizeof(double) * na * 3, cudaMemcpyDeviceToHost, E.stream);
        if (dip_momI) cudaMemcpyAsync(dip_momI, E.kp.dipI, sizeof(double) * nw * 3, cudaMemcpyDeviceToHost, E.stream);
        if (chg) cudaMemcpyAsync(chg, E.kp.chg, sizeof(double) * na, cudaMemcpyDeviceToHost, E.stream);
        rc = read_err(E);
        if (!rc) {
            if (En) *En = h[0];
            if (virt) std::copy(h + 2, h + 11, virt);
        }
    }
    cudaStreamSynchronize(E.stream);
    E.kp = saved;
    return rc;
}

int pimd_get_energies(pimd_ctx *ctx, int bead, double U[4]) {
    if (!ctx || bead < 0 || bead >= ctx->E.kp.P || !U) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    double a[NACC];
    cudaMemcpyAsync(a, E.kp.acc + (size_t)bead * NACC, sizeof(a), cudaMemcpyDeviceToHost, E.stream);
    int rc = cuda_check(E, cudaStreamSynchronize(E.stream), "get_energies");
    if (rc) return rc;
    U[0] = a[ACC_UMON];
    U[1] = a[ACC_UVDW];
    U[2] = 0.5 * a[ACC_UELEC2];
    U[3] = a[ACC_UIND];
    return PIMD_OK;
}

int pimd_get_virial(pimd_ctx *ctx, int bead, double virt[9]) {
    if (!ctx || bead < 0 || bead >= ctx->E.kp.P || !virt) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    double a[NACC];
    cudaMemcpyAsync(a, E.kp.acc + (size_t)bead * NACC, sizeof(a), cudaMemcpyDeviceToHost, E.stream);
    int rc = cuda_check(E, cudaStreamSynchronize(E.stream), "get_virial");
    if (rc) return rc;
    for (int i = 0; i < 9; i++) virt[i] = a[ACC_VIRT + i];
    virt[0] -= E.kp.Uvdw_lrc;
    virt[4] -= E.kp.Uvdw_lrc;
    virt[8] -= E.kp.Uvdw_lrc;
    return PIMD_OK;
}

long long pimd_launch_count(pimd_ctx *ctx) { return ctx ? ctx->E.nlaunch : -1; }

int pimd_timers_reset(pimd_ctx *ctx, int enable) {
    if (!ctx) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    timer_resolve(E);
    PhaseTimers &T = E.timers;
    for (size_t i = 0; i < T.ms.size(); i++) {
        T.ms[i] = 0.0;
        T.count[i] = 0;
    }
    T.on = enable != 0;
    return PIMD_OK;
}

int pimd_timers_get(pimd_ctx *ctx, int i, char *name, int namelen, double *ms, long long *count) {
    if (!ctx) return -1;
    Engine &E = ctx->E;
    timer_resolve(E);
    PhaseTimers &T = E.timers;
    if (i < 0 || i >= (int)T.names.size()) return (int)T.names.size();
    if (name && namelen > 0) {
        std::strncpy(name, T.names[i].c_str(), namelen - 1);
        name[namelen - 1] = 0;
    }
    if (ms) *ms = T.ms[i];
    if (count) *count = T.count[i];
    return (int)T.names.size();
}

int pimd_get_neighbors(pimd_ctx *ctx, int bead, int *ij, int cap, int *npairs) {
    if (!ctx || bead < 0 || bead >= ctx->E.kp.P || cap < 0) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    int n = 0;
    cudaMemcpyAsync(&n, E.kp.npair + bead, sizeof(int), cudaMemcpyDeviceToHost, E.stream);
    int rc = cuda_check(E, cudaStreamSynchronize(E.stream), "get_neighbors");
    if (rc) return rc;
    if (npairs) *npairs = n;
    const int m = std::min(n, cap);
    if (ij && m > 0) {
        cudaMemcpyAsync(ij, E.kp.pairs + (size_t)bead * E.kp.cap, sizeof(int2) * m, cudaMemcpyDeviceToHost, E.stream);
        rc = cuda_check(E, cudaStreamSynchronize(E.stream), "get_neighbors");
    }
    return rc;
}

int pimd_get_dipole_info(pimd_ctx *ctx, int bead, int *niter, double *deltadip) {
    if (!ctx || bead < 0 || bead >= ctx->E.kp.P) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    double a[NACC];
    cudaMemcpyAsync(a, E.kp.acc + (size_t)bead * NACC, sizeof(a), cudaMemcpyDeviceToHost, E.stream);
    int rc = cuda_check(E, cudaStreamSynchronize(E.stream), "get_dipole_info");
    if (rc) return rc;
    if (niter) *niter = (int)a[ACC_NITER];
    if (deltadip) *deltadip = a[ACC_DELTADIP];
    return PIMD_OK;
}

// ---------------------------------------------------------------------------------------
// Autotuner: coordinate descent over the launch-shape knobs, each candidate timed as the best of
// two force calls (after one warm-up) with CUDA events on the context's stream.
static int tune_time(pimd_ctx *ctx, float *ms) {
    Engine &E = ctx->E;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double *d = E.d_out;
    float best = 1e30f;
    int rc = PIMD_OK;
    for (int rep = 0; rep < 3 && !rc; rep++) {
        cudaEventRecord(a, E.stream);
        rc = run_forces(E, 0, ctx->check_every, d, d + E.kp.P, d + 2 * E.kp.P, nullptr);
        cudaEventRecord(b, E.stream);
        cudaError_t e = cudaEventSynchronize(b);
        if (!rc && e != cudaSuccess) rc = cuda_check(E, e, "autotune");
        float t = 0.f;
        cudaEventElapsedTime(&t, a, b);
        if (rep > 0) best = std::min(best, t);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = best;
    return rc;
}

int pimd_autotune(pimd_ctx *ctx, const double *RRt, const double *RRc) {
    if (!ctx) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    KP saved = E.kp;
    if (RRt) E.kp.RRt = RRt;
    if (RRc) E.kp.RRc = RRc;
    const bool timers_on = E.timers.on;
    E.timers.on = false;
    struct Knob {
        int *v;
        std::vector<int> cand;
    };
    int sf_tiled = E.sf_tiled, ff_regs = E.ff_regs, nbr_block = E.nbr_block, wave = E.wave_shapes;
    int nbr_cells = E.nbr_cells, sf_tc = E.sf_tc, ff_tc = E.ff_tc, dd_overlap = E.dd_overlap, xcache = E.tc_xcache, pdl = E.tc_pdl,
        ewo = E.ewald_overlap, otf = E.dd_otf, dda = E.dd_async;
    std::vector<Knob> knobs;
    const bool mixed = E.precision == PIMD_MIXED && E.kp.model < 4;
    if (mixed) {
        if (E.tc_ready) knobs.push_back({&sf_tc, {1, 0}});
        if (E.tf_ready) knobs.push_back({&ff_tc, {1, 0}});
        knobs.push_back({&sf_tiled, {1, 0}});
        knobs.push_back({&E.sf_groups, {0, 4, 8, 16, 32}});
        knobs.push_back({&ff_regs, {1, 0}});
        if (E.loop_aux) knobs.push_back({&dd_overlap, {1, 0}});
        if (dd_async_ok(E)) knobs.push_back({&dda, {1, 0}});
        if (E.d_tcx) knobs.push_back({&xcache, {1, 0}});
        if (E.tf_ready) knobs.push_back({&pdl, {1, 0}});
        if (E.kp.Fx) knobs.push_back({&ewo, {1, 0}});
        knobs.push_back({&otf, {1, 0}});
    }
    knobs.push_back({&wave, {1, 0}});
    knobs.push_back({&E.max_slices, {16, 8, 4, 2}});
    knobs.push_back({&nbr_block, {1, 0}});
    if (E.kp.cl_ncell > 0) knobs.push_back({&nbr_cells, {1, 0}});
    auto apply = [&]() {
        E.sf_tiled = sf_tiled != 0;
        E.ff_regs = ff_regs != 0;
        E.nbr_block = nbr_block != 0;
        E.wave_shapes = wave != 0;
        E.nbr_cells = nbr_cells != 0;
        E.sf_tc = sf_tc != 0;
        E.ff_tc = ff_tc != 0;
        E.dd_overlap = dd_overlap != 0;
        E.tc_xcache = xcache != 0;
        E.tc_pdl = pdl != 0;
        E.ewald_overlap = ewo != 0;
        E.dd_otf = otf != 0;
        E.dd_async = dda != 0;
    };
    int rc = PIMD_OK;
    float best;
    apply();
    rc = tune_time(ctx, &best);
    for (size_t k = 0; k < knobs.size() && !rc; k++) {
        int keep = *knobs[k].v;
        for (int c : knobs[k].cand) {
            if (c == keep) continue;
            *knobs[k].v = c;
            apply();
            float t;
            if ((rc = tune_time(ctx, &t))) break;
            if (t < best) {
                best = t;
                keep = c;
            }
        }
        *knobs[k].v = keep;
        apply();
    }
    // the Fpart buffer holds max_slices slices: never exceed the allocated 16
    E.max_slices = std::min(E.max_slices, 16);
    E.gkey.clear();  // a captured MD-step graph holds the old launches: capture again
    E.timers.on = timers_on;
    const double *kr = saved.RRt, *kc = saved.RRc;
    E.kp.RRt = kr;
    E.kp.RRc = kc;
    return rc;
}

int pimd_get_tuning(pimd_ctx *ctx, int *k, int n) {
    if (!ctx || !k || n < 5) return PIMD_ERR_ARG;
    const Engine &E = ctx->E;
    k[0] = E.sf_tiled;
    k[1] = E.sf_groups;
    k[2] = E.ff_regs;
    k[3] = E.max_slices;
    k[4] = E.nbr_block;
    if (n >= 6) k[5] = E.wave_shapes;
    if (n >= 7) k[6] = E.sf_tc && E.tc_ready;
    if (n >= 8) k[7] = E.ff_tc && E.tf_ready;
    if (n >= 9) k[8] = E.dd_overlap && E.loop_aux != nullptr && E.precision == PIMD_MIXED;
    if (n >= 10) k[9] = E.tc_xcache && E.d_tcx != nullptr && E.sf_tc && E.tc_ready;
    if (n >= 11) k[10] = E.tc_pdl && E.ff_tc && E.tf_ready && E.sf_tc && E.tc_ready;
    if (n >= 12) k[11] = E.loop_unroll;
    if (n >= 13) k[12] = E.ewald_overlap && E.aux_stream != nullptr && E.kp.Fx != nullptr;
    if (n >= 14) k[13] = E.dd_otf && E.precision == PIMD_MIXED;
    if (n >= 15) k[14] = E.ff_tc && E.tf_ready && E.tf_qd_ready;
    if (n >= 16) k[15] = E.l2_keep && E.precision == PIMD_MIXED;
    if (n >= 17) k[16] = dd_async_ok(E);
    if (n >= 18) k[17] = E.dd_pev && E.loop_pev != nullptr;
    if (n >= 19) k[18] = E.dd_jpev && E.loop_jpev != nullptr && field_pdl_ok(E);
    if (n >= 20) k[19] = E.nbr_overlap && E.ev_nbr != nullptr && E.precision == PIMD_MIXED && nbr_from_inputs(E);
    return PIMD_OK;
}

int pimd_set_tuning(pimd_ctx *ctx, const int *k, int n) {
    if (!ctx || !k || n < 5) return PIMD_ERR_ARG;
    if (k[1] < 0 || k[1] > 1024 || k[3] < 1 || k[3] > 16) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    E.sf_tiled = k[0] != 0;
    E.sf_groups = k[1];
    E.ff_regs = k[2] != 0;
    E.max_slices = k[3];
    E.nbr_block = k[4] != 0;
    if (n >= 6) E.wave_shapes = k[5] != 0;
    if (n >= 7) E.sf_tc = k[6] != 0;
    if (n >= 8) E.ff_tc = k[7] != 0;
    if (n >= 9) E.dd_overlap = k[8] != 0;
    if (n >= 10) E.tc_xcache = k[9] != 0;
    if (n >= 11) E.tc_pdl = k[10] != 0;
    if (n >= 12) {
        if (k[11] < 1 || k[11] > 4) return PIMD_ERR_ARG;
        E.loop_unroll = k[11];
    }
    if (n >= 13) E.ewald_overlap = k[12] != 0;
    if (n >= 14) E.dd_otf = k[13] != 0;
    if (n >= 16) E.l2_keep = k[15] != 0;
    if (n >= 17) E.dd_async = k[16] != 0;
    if (n >= 18) E.dd_pev = k[17] != 0;
    if (n >= 19) E.dd_jpev = k[18] != 0;
    if (n >= 20) E.nbr_overlap = k[19] != 0;
    E.gkey.clear();  // a captured MD-step graph holds the old launches: capture again
    return PIMD_OK;
}

}  // extern "C"
