// pimd_oracle.cpp -- CPU FP64 restatement of the PIMD-F90 hot path.
//
// TEST INFRASTRUCTURE ONLY: the checker the CUDA engine is compared against. Nothing in the
// engine links to or calls this file. Parity unpinned by the reference's own outputs (no
// Fortran compiler is available to build the reference); pinned by physics known-answer
// tests in tests/.
//
// Conventions: Fortran arrays A(3,n) are stored column-major as A[3*(i-1)+(c-1)]; site
// indices below are 0-based (O block 0..N-1, H1 N..2N-1, H2 2N..3N-1, M 3N..4N-1), which
// is the reference's OOO..HHH..HHH..MMM layout shifted by one. Every expression keeps the
// reference's evaluation order; the library is built with -ffp-contract=off so no FMA is
// formed (the reference is assumed built by gfortran -O3 on baseline x86-64, no FMA).
#include "pimd_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "../pimd-f90_gb300/csrc/nasa_tables.h"

namespace {

// consts.f90:22-55
const double CHARGECON = 18.22234397655801030455;
const double DEBYE = 4.8033324;
const double MASSCON = 418.4;
const double PI = 3.14159265358979323844;
const double TWOPI = 6.28318530717958647688;
const double FOURPI = 12.56637061435917295376;
const double TSP = 1.12837916709551257390;
const double SQPI = 1.77245385090551602729;
const double KB_AMU = 0.831447148;  // KB_amuA2ps2perK

// pot_mod.f90:7-44 model parameters
struct ModelParams {
    double vdwA, vdwB, vdwC, vdwD, vdwE, aDD, aCCaCD, polfacO, polfacH, polfacM, polarO, polarH,
        polarM, gammaM, dms1, dms2, dms3;
};
const ModelParams TTM21F = {-1.329565985e+6, 3.632560798e+5, -2.147141323e+3, 1.e13, 13.2, 0.3, 0.2,
                            0.837, 0.496, 0.837, 0.837, 0.496, 0.837, 0.426706882, 0.0, 0.0, 0.0};
const ModelParams TTM3F = {0.0, 0.0, -0.72298855e+03, 0.10211829e+06, 0.37170376e+01, 0.175, 0.175,
                           0.837, 0.496, 0.837, 0.0, 0.0, 1.444, 0.46, 0.5, 0.9578, 0.012};

inline double anint(double x) { return std::round(x); }  // Fortran anint: half away from zero

// math.f90:287-314 Abramowitz-Stegun 7.1.26
double erfc_as(double X) {
    const double A1 = 0.254829592, A2 = -0.284496736, A3 = 1.421413741, A4 = -1.453152027,
                 A5 = 1.061405429, P = 0.3275911;
    double T = 1.0 / (1.0 + P * X);
    double XSQ = X * X;
    double TP = T * (A1 + T * (A2 + T * (A3 + T * (A4 + T * A5))));
    return TP * std::exp(-XSQ);
}

// math.f90:211-247 gser2_3
double gser2_3(double x, int *err) {
    const double a = 2.0 / 3.0, gln = 0.303150275147547, EPS = 3.e-7;
    if (x <= 0.0) {
        if (x < 0.0) *err |= 1;
        return 0.0;
    }
    double ap = a, ssum = 1.0 / a, del = ssum;
    for (int n = 1; n <= 800; n++) {
        ap = ap + 1.0;
        del = del * x / ap;
        ssum = ssum + del;
        if (std::fabs(del) < std::fabs(ssum) * EPS) return ssum * std::exp(-x + a * std::log(x) - gln);
    }
    *err |= 2;
    return NAN;
}

// math.f90:250-285 gcf2_3 (modified Lentz)
double gcf2_3(double x, int *err) {
    const double a = 2.0 / 3.0, gln = 0.303150275147547, EPS = 3.e-7, FPMIN = 1.e-30;
    double b = x + 1.0 - a, c = 1.0 / FPMIN, d = 1.0 / b, h = d;
    for (int i = 1; i <= 100; i++) {
        double an = -(double)i * ((double)i - a);
        b = b + 2.0;
        d = an * d + b;
        if (std::fabs(d) < FPMIN) d = FPMIN;
        c = b + an / c;
        if (std::fabs(c) < FPMIN) c = FPMIN;
        d = 1.0 / d;
        double del = d * c;
        h = h * del;
        if (std::fabs(del - 1.0) < EPS) return std::exp(-x + a * std::log(x) - gln) * h;
    }
    *err |= 4;
    return NAN;
}

// math.f90:188-208
double gammq2_3(double x, int *err) {
    const double a = 2.0 / 3.0;
    if (x < 0.0) {
        *err |= 1;
        return NAN;
    }
    if (x < a + 1.0) return 1.0 - gser2_3(x, err);
    return gcf2_3(x, err);
}

struct Orc {
    orc_params p;
    ModelParams m;
    bool polar;
    int N, NM, Natoms;
    int fd, ld;    // 0-based dipole site range [fd, ld]
    int fdI, ldI;  // 1-based dipole site kinds
    double box[3], boxi[3], volume, rc, rc1, Rc2;
    double shiftA = 0, shiftB = 0, Uvdw_lrc = 0;
    double qO = 0, qH = 0, roh0 = 0, th0 = 0, harmkb = 0, harmka = 0;
    double polfac[5];
    double aewald, const_ts1, const_ts2, const_ts3;
    // Ewald tables
    int nkvec = 0, hmax = 0, kmax = 0, lmax = 0;
    std::vector<int> k_hkl;
    std::vector<double> kvec, Ak, rQq, iQq, rQm, iQm;
    std::vector<double> coskx, sinkx, cosky, sinky, coskz, sinkz;  // [s][n]
    std::vector<double> coskxky, sinkxky, coskr, sinkr, dKk;
    // state
    std::vector<double> R, RRRc, dR, Efq, Efd, dip, olddip, charge, phi, grdq, tx_dip;
    double c5z[245];
    double Umon, Uvdw, Uelec, Uind, vir_rec[9];
    int niter = 0;
    double deltadip_last = 0;
    int err = 0;

    double &Rx(std::vector<double> &a, int c, int s) { return a[3 * s + c]; }

    int ncx() const { return hmax + 1; }
    int ncy() const { return 2 * kmax + 1; }
    int ncz() const { return 2 * lmax + 1; }
    double &CX(std::vector<double> &t, int s, int n) { return t[s * ncx() + n]; }
    double &CY(std::vector<double> &t, int s, int n) { return t[s * ncy() + n + kmax]; }
    double &CZ(std::vector<double> &t, int s, int n) { return t[s * ncz() + n + lmax]; }

    explicit Orc(const orc_params *pp);
    void ewald_set();
    void ssincos();
    void ewald_std_qq();
    void ewald_std_dd();
    void ewald_std_qd();
    void ewald_pw_std_qq();
    void find_neigh(int iO, std::vector<int> &nj, std::vector<double> &nR, std::vector<double> &nR2);
    void smear01(double drsq, double a_pol12, double *ts0, double *ts1);
    void smear2(double drsq, double a_pol12, double *ts1, double *ts2);
    void smear3(double drsq, double a_pol12, double *ts1, double *ts2, double *ts3);
    void self1(double drsq, double *ts0, double *ts1);
    void self2(double drsq, double *ts1, double *ts2);
    void pot_nasa(const double r1[3][3], double dr1[3][3], double *e1);
    void dms_nasa(const double r1[3][3], double q3[3], double gradq[3][3][3]);
    void pot_ttm(int bead, const double *RR, const double *RRc, double *En, double *dRR, double *virt,
                 double *virialc, double *dip_momI, double *Edip_mom, double *chg, int t);
    void pot_spc(const double *RR, double *En, double *dRR, double *virt, double *dip_momI,
                 double *chg);
};

// potential.f90:43-199 init_pot
Orc::Orc(const orc_params *pp) : p(*pp) {
    Natoms = p.natoms;
    N = Natoms / 3;
    polar = (p.pot_model == 2 || p.pot_model == 3);
    NM = polar ? 4 * N : 3 * N;
    for (int c = 0; c < 3; c++) box[c] = p.box[c];
    rc = p.rc;
    rc1 = p.rc1;
    Rc2 = rc * rc;
    if (p.pot_model == 2) {
        m = TTM21F;
        fd = 0;
        ld = 3 * N - 1;
        fdI = 1;
        ldI = 3;
    } else if (p.pot_model == 3) {
        m = TTM3F;
        fd = 3 * N;
        ld = 4 * N - 1;
        fdI = 4;
        ldI = 4;
        if (rc == rc1) {
            shiftA = 0;
            shiftB = 0;
        } else {
            // potential.f90:106-113 (integer powers as repeated products)
            double rc8 = rc * rc * rc * rc * rc * rc * rc * rc;
            shiftA = -(10 * rc - 7 * rc1) / (rc8 * ((rc - rc1) * (rc - rc1)));
            shiftB = (9 * rc - 7 * rc1) / (rc8 * ((rc - rc1) * (rc - rc1) * (rc - rc1)));
        }
    } else {
        std::memset(&m, 0, sizeof(m));
        fd = 0;
        ld = -1;
        fdI = 1;
        ldI = 0;
        if (p.pot_model == 4) {  // pot_mod.f90:31-35
            m.vdwA = 629326.57249877361701443513;
            m.vdwC = -625.50206521141523463400;
            qO = -0.84;
            qH = 0.42;
            roh0 = 1.012;
            th0 = 1.95476876223364912614;
            harmkb = 529.581;
            harmka = 37.95;
        } else {  // pot_mod.f90:40-44
            m.vdwA = 628213.72817108343399678768;
            m.vdwC = -624.97858519194071637260;
            qO = -0.82;
            qH = 0.41;
            roh0 = 1.0;
            th0 = 1.91061193215819258784;
        }
    }
    volume = box[0] * box[1] * box[2];
    for (int c = 0; c < 3; c++) boxi[c] = 1.0 / box[c];
    {
        double r3 = rc * rc * rc, r7 = r3 * r3 * rc, r9 = r7 * rc * rc;
        Uvdw_lrc = TWOPI * (double)(N * N) / volume *
                   (m.vdwA / (9.0 * r9) + m.vdwB / (7.0 * r7) + m.vdwC / (3.0 * r3));
    }
    if (polar) {
        double pf[4] = {std::pow(m.polfacO, 1.0 / 6.0), std::pow(m.polfacH, 1.0 / 6.0),
                        std::pow(m.polfacH, 1.0 / 6.0), std::pow(m.polfacM, 1.0 / 6.0)};
        for (int i = 0; i < 4; i++) polfac[i + 1] = 1.0 / (pf[i] * pf[i] * pf[i]);
    }
    R.assign(3 * NM, 0.0);
    RRRc.assign(3 * NM, 0.0);
    dR.assign(3 * NM, 0.0);
    Efq.assign(3 * NM, 0.0);
    Efd.assign(3 * NM, 0.0);
    dip.assign(3 * NM, 0.0);
    olddip.assign(3 * NM, 0.0);
    charge.assign(NM, 0.0);
    phi.assign(NM, 0.0);
    grdq.assign(27 * N, 0.0);
    int nslots = p.shared_history ? 1 : std::max(1, p.nbeads);
    tx_dip.assign((size_t)nslots * 4 * 3 * NM, 0.0);
    if (!polar) {  // potential.f90:186-192
        for (int iw = 0; iw < N; iw++) {
            charge[iw] = qO * CHARGECON;
            charge[iw + N] = qH * CHARGECON;
            charge[iw + 2 * N] = qH * CHARGECON;
        }
    }
    // nasa.f90:45 c5z = f5z*c5zA + fbasis*cbasis + fcore*ccore + frest*crest
    for (int j = 0; j < 245; j++)
        c5z[j] = PIMD_NASA_F5Z * PIMD_NASA_C5ZA[j] + PIMD_NASA_FBASIS * PIMD_NASA_CBASIS[j] +
                 PIMD_NASA_FCORE * PIMD_NASA_CCORE[j] + PIMD_NASA_FREST * PIMD_NASA_CREST[j];
    ewald_set();
    const_ts1 = 2.0 * aewald / SQPI;
    const_ts2 = 4.0 * aewald * aewald * aewald / (3.0 * SQPI);
    double a5 = aewald * aewald * aewald * aewald * aewald;
    const_ts3 = 8.0 * a5 / (15.0 * SQPI);
}

// ewald.f90:293-378 ewald_set(.true.). With p.alpha > 0 the Ewald alpha and the integer
// shell |n|^2 <= nmax^2 are taken as given instead of the eps_ewald rule.
void Orc::ewald_set() {
    double kvec_cutSQ = 0;
    bool explicit_k = p.alpha > 0;
    if (!explicit_k) {
        double PP = -std::log(p.eps_ewald);
        aewald = std::sqrt(PP) / rc;
        double kvec_cut = 2.0 * aewald * std::sqrt(PP);
        kvec_cutSQ = kvec_cut * kvec_cut;
        hmax = (int)std::floor(kvec_cut / TWOPI * box[0]);
        kmax = (int)std::floor(kvec_cut / TWOPI * box[1]);
        lmax = (int)std::floor(kvec_cut / TWOPI * box[2]);
    } else {
        aewald = p.alpha;
        hmax = kmax = lmax = p.nmax;
    }
    double fac_ew2 = -0.25 / (aewald * aewald);
    const double factor = 2.0;
    nkvec = 0;
    k_hkl.clear();
    kvec.clear();
    Ak.clear();
    double kv[3];
    for (int kx = 0; kx <= hmax; kx++) {
        kv[0] = TWOPI * boxi[0] * (double)kx;
        int ky1 = (kx == 0) ? 0 : -kmax;
        for (int ky = ky1; ky <= kmax; ky++) {
            kv[1] = TWOPI * boxi[1] * (double)ky;
            int kz1 = (kx == 0 && ky == 0) ? 1 : -lmax;
            double kvxy = kv[0] * kv[0] + kv[1] * kv[1];
            for (int kz = kz1; kz <= lmax; kz++) {
                kv[2] = TWOPI * boxi[2] * (double)kz;
                double kvsq = kvxy + kv[2] * kv[2];
                bool keep = explicit_k ? (kx * kx + ky * ky + kz * kz <= p.nmax * p.nmax && kvsq > 1.e-16)
                                       : (kvsq < kvec_cutSQ && kvsq > 1.e-16);
                if (keep) {
                    nkvec++;
                    k_hkl.push_back(kx);
                    k_hkl.push_back(ky);
                    k_hkl.push_back(kz);
                    kvec.push_back(kv[0]);
                    kvec.push_back(kv[1]);
                    kvec.push_back(kv[2]);
                    Ak.push_back(factor * std::exp(fac_ew2 * kvsq) / kvsq);
                }
            }
        }
    }
    coskx.assign((size_t)NM * ncx(), 0.0);
    sinkx.assign((size_t)NM * ncx(), 0.0);
    cosky.assign((size_t)NM * ncy(), 0.0);
    sinky.assign((size_t)NM * ncy(), 0.0);
    coskz.assign((size_t)NM * ncz(), 0.0);
    sinkz.assign((size_t)NM * ncz(), 0.0);
    coskxky.assign(NM, 0.0);
    sinkxky.assign(NM, 0.0);
    coskr.assign(NM, 0.0);
    sinkr.assign(NM, 0.0);
    dKk.assign(NM, 0.0);
    rQq.assign(nkvec, 0.0);
    iQq.assign(nkvec, 0.0);
    rQm.assign(nkvec, 0.0);
    iQm.assign(nkvec, 0.0);
}

// ewald.f90:403-437 ssincos (angle-addition recurrence from n = 1)
void Orc::ssincos() {
    for (int s = 0; s < NM; s++) {
        CX(coskx, s, 0) = 1.0;
        CY(cosky, s, 0) = 1.0;
        CZ(coskz, s, 0) = 1.0;
        CX(sinkx, s, 0) = 0.0;
        CY(sinky, s, 0) = 0.0;
        CZ(sinkz, s, 0) = 0.0;
        if (hmax >= 1) {
            CX(coskx, s, 1) = std::cos(TWOPI * boxi[0] * R[3 * s + 0]);
            CX(sinkx, s, 1) = std::sin(TWOPI * boxi[0] * R[3 * s + 0]);
        }
        if (kmax >= 1) {
            CY(cosky, s, 1) = std::cos(TWOPI * boxi[1] * R[3 * s + 1]);
            CY(cosky, s, -1) = CY(cosky, s, 1);
            CY(sinky, s, 1) = std::sin(TWOPI * boxi[1] * R[3 * s + 1]);
            CY(sinky, s, -1) = -CY(sinky, s, 1);
        }
        if (lmax >= 1) {
            CZ(coskz, s, 1) = std::cos(TWOPI * boxi[2] * R[3 * s + 2]);
            CZ(coskz, s, -1) = CZ(coskz, s, 1);
            CZ(sinkz, s, 1) = std::sin(TWOPI * boxi[2] * R[3 * s + 2]);
            CZ(sinkz, s, -1) = -CZ(sinkz, s, 1);
        }
        for (int kx = 2; kx <= hmax; kx++) {
            CX(coskx, s, kx) = CX(coskx, s, kx - 1) * CX(coskx, s, 1) - CX(sinkx, s, kx - 1) * CX(sinkx, s, 1);
            CX(sinkx, s, kx) = CX(coskx, s, kx - 1) * CX(sinkx, s, 1) + CX(sinkx, s, kx - 1) * CX(coskx, s, 1);
        }
        for (int ky = 2; ky <= kmax; ky++) {
            CY(cosky, s, ky) = CY(cosky, s, ky - 1) * CY(cosky, s, 1) - CY(sinky, s, ky - 1) * CY(sinky, s, 1);
            CY(sinky, s, ky) = CY(cosky, s, ky - 1) * CY(sinky, s, 1) + CY(sinky, s, ky - 1) * CY(cosky, s, 1);
            CY(cosky, s, -ky) = CY(cosky, s, ky);
            CY(sinky, s, -ky) = -CY(sinky, s, ky);
        }
        for (int kz = 2; kz <= lmax; kz++) {
            CZ(coskz, s, kz) = CZ(coskz, s, kz - 1) * CZ(coskz, s, 1) - CZ(sinkz, s, kz - 1) * CZ(sinkz, s, 1);
            CZ(sinkz, s, kz) = CZ(coskz, s, kz - 1) * CZ(sinkz, s, 1) + CZ(sinkz, s, kz - 1) * CZ(coskz, s, 1);
            CZ(coskz, s, -kz) = CZ(coskz, s, kz);
            CZ(sinkz, s, -kz) = -CZ(sinkz, s, kz);
        }
    }
}

// ewald.f90:1-52 ewald_std_qq (TTM site layout: sites fO..lM, charges fH..lM)
void Orc::ewald_std_qq() {
    ssincos();
    int lastkx = -1000, lastky = -1000;
    for (int k = 0; k < nkvec; k++) {
        int kx = k_hkl[3 * k], ky = k_hkl[3 * k + 1], kz = k_hkl[3 * k + 2];
        const double *kv = &kvec[3 * k];
        double p4vAkk = FOURPI * Ak[k] / volume;
        if (!(kx == lastkx && ky == lastky)) {
            for (int s = 0; s < NM; s++) {
                double tmp = CX(sinkx, s, kx) * CY(cosky, s, ky) + CX(coskx, s, kx) * CY(sinky, s, ky);
                coskxky[s] = CX(coskx, s, kx) * CY(cosky, s, ky) - CX(sinkx, s, kx) * CY(sinky, s, ky);
                sinkxky[s] = tmp;
            }
        }
        lastkx = kx;
        lastky = ky;
        for (int s = 0; s < NM; s++) {
            double tmp = sinkxky[s] * CZ(coskz, s, kz) + coskxky[s] * CZ(sinkz, s, kz);
            coskr[s] = coskxky[s] * CZ(coskz, s, kz) - sinkxky[s] * CZ(sinkz, s, kz);
            sinkr[s] = tmp;
        }
        double rQqk = 0, iQqk = 0;
        for (int s = N; s < NM; s++) rQqk += charge[s] * coskr[s];
        for (int s = N; s < NM; s++) iQqk += charge[s] * sinkr[s];
        rQq[k] = rQqk;
        iQq[k] = iQqk;
        for (int s = 0; s < NM; s++) {
            double tmp = p4vAkk * (coskr[s] * iQqk - sinkr[s] * rQqk);
            for (int c = 0; c < 3; c++) Efq[3 * s + c] = Efq[3 * s + c] - tmp * kv[c];
        }
        for (int s = N; s < NM; s++) phi[s] = phi[s] + p4vAkk * (coskr[s] * rQqk + sinkr[s] * iQqk);
    }
}

// ewald.f90:56-119 ewald_std_dd
void Orc::ewald_std_dd() {
    int lastkx = -1000, lastky = -1000;
    for (int k = 0; k < nkvec; k++) {
        int kx = k_hkl[3 * k], ky = k_hkl[3 * k + 1], kz = k_hkl[3 * k + 2];
        const double *kv = &kvec[3 * k];
        double p4vAkk = FOURPI * Ak[k] / volume;
        if (!(kx == lastkx && ky == lastky)) {
            for (int i = fd; i <= ld; i++) {
                double tmp = CX(sinkx, i, kx) * CY(cosky, i, ky) + CX(coskx, i, kx) * CY(sinky, i, ky);
                coskxky[i] = CX(coskx, i, kx) * CY(cosky, i, ky) - CX(sinkx, i, kx) * CY(sinky, i, ky);
                sinkxky[i] = tmp;
            }
        }
        for (int i = fd; i <= ld; i++)
            dKk[i] = (kv[0] * dip[3 * i] + kv[1] * dip[3 * i + 1]) + kv[2] * dip[3 * i + 2];
        double rQmk = 0, iQmk = 0;
        for (int i = fd; i <= ld; i++) {
            double tmp = sinkxky[i] * CZ(coskz, i, kz) + coskxky[i] * CZ(sinkz, i, kz);
            coskr[i] = coskxky[i] * CZ(coskz, i, kz) - sinkxky[i] * CZ(sinkz, i, kz);
            sinkr[i] = tmp;
            rQmk = rQmk - dKk[i] * sinkr[i];
            iQmk = iQmk + dKk[i] * coskr[i];
        }
        rQm[k] = rQmk;
        iQm[k] = iQmk;
        lastkx = kx;
        lastky = ky;
        for (int i = fd; i <= ld; i++) {
            double tmp = p4vAkk * (coskr[i] * iQmk - sinkr[i] * rQmk);
            for (int c = 0; c < 3; c++) Efd[3 * i + c] = Efd[3 * i + c] - kv[c] * tmp;
        }
    }
}

// ewald.f90:123-226 ewald_std_qd. Uses rQm/iQm stored by the LAST ewald_std_dd call
// (i.e. the dipoles before the final SOR update) and dKk from the final dipoles.
void Orc::ewald_std_qd() {
    double virtmp[9] = {0}, virtmp1[9] = {0};  // (row,col) -> [row + 3*col]
    int lastkx = -1000, lastky = -1000;
    for (int k = 0; k < nkvec; k++) {
        int kx = k_hkl[3 * k], ky = k_hkl[3 * k + 1], kz = k_hkl[3 * k + 2];
        const double *kv = &kvec[3 * k];
        double Akk = Ak[k];
        double p4vAkk = FOURPI * Akk / volume;
        if (!(kx == lastkx && ky == lastky)) {
            for (int i = 0; i < NM; i++) {
                double tmp = CX(sinkx, i, kx) * CY(cosky, i, ky) + CX(coskx, i, kx) * CY(sinky, i, ky);
                coskxky[i] = CX(coskx, i, kx) * CY(cosky, i, ky) - CX(sinkx, i, kx) * CY(sinky, i, ky);
                sinkxky[i] = tmp;
            }
        }
        for (int i = fd; i <= ld; i++)
            dKk[i] = (kv[0] * dip[3 * i] + kv[1] * dip[3 * i + 1]) + kv[2] * dip[3 * i + 2];
        for (int i = 0; i < NM; i++) {
            double tmp = sinkxky[i] * CZ(coskz, i, kz) + coskxky[i] * CZ(sinkz, i, kz);
            coskr[i] = coskxky[i] * CZ(coskz, i, kz) - sinkxky[i] * CZ(sinkz, i, kz);
            sinkr[i] = tmp;
        }
        lastkx = kx;
        lastky = ky;
        double rQmk = rQm[k], iQmk = iQm[k];
        double rQqmk = rQq[k] + rQm[k], iQqmk = iQq[k] + iQm[k];
        for (int iat = N; iat < NM; iat++) {
            double tmp = charge[iat] * p4vAkk * (coskr[iat] * iQmk - sinkr[iat] * rQmk);
            phi[iat] = phi[iat] + p4vAkk * (coskr[iat] * rQmk + sinkr[iat] * iQmk);
            for (int c = 0; c < 3; c++) dR[3 * iat + c] = dR[3 * iat + c] + tmp * kv[c];
        }
        for (int iat = fd; iat <= ld; iat++) {
            double tmp = dKk[iat] * p4vAkk * (coskr[iat] * rQqmk + sinkr[iat] * iQqmk);
            for (int c = 0; c < 3; c++) dR[3 * iat + c] = dR[3 * iat + c] - tmp * kv[c];
        }
        double ksq = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
        double coeff2 = 2.0 / ksq + 0.5 / (aewald * aewald);
        double Ureck = Akk * (rQqmk * rQqmk + iQqmk * iQqmk);
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double t = Ureck * coeff2 * kv[std::min(a, b)] * kv[std::max(a, b)];
                virtmp[a + 3 * b] = (a == b) ? virtmp[a + 3 * b] + Ureck - t : virtmp[a + 3 * b] - t;
            }
        double rdipQ[3], idipQ[3];
        for (int c = 0; c < 3; c++) {
            double sr = 0, si = 0;
            for (int i = fd; i <= ld; i++) sr += sinkr[i] * dip[3 * i + c];
            for (int i = fd; i <= ld; i++) si += coskr[i] * dip[3 * i + c];
            rdipQ[c] = -sr;
            idipQ[c] = si;
        }
        for (int ix = 0; ix < 3; ix++) {
            double tmp = 2.0 * Akk * kv[ix];
            for (int iy = 0; iy < 3; iy++)
                virtmp1[ix + 3 * iy] = virtmp1[ix + 3 * iy] + tmp * (rQqmk * rdipQ[iy] + iQqmk * idipQ[iy]);
        }
    }
    for (int i = 0; i < 9; i++) {
        virtmp[i] = -0.5 * virtmp[i] * FOURPI / volume;
        virtmp1[i] = -0.5 * virtmp1[i] * FOURPI / volume;
        vir_rec[i] = vir_rec[i] + virtmp[i] + virtmp1[i];
    }
}

// ewald.f90:230-291 ewald_pw_std_qq (non-polarizable: sites fO..lH, also the virial)
void Orc::ewald_pw_std_qq() {
    for (int i = 0; i < 9; i++) vir_rec[i] = 0.0;
    ssincos();
    int lastkx = -1000, lastky = -1000;
    for (int k = 0; k < nkvec; k++) {
        int kx = k_hkl[3 * k], ky = k_hkl[3 * k + 1], kz = k_hkl[3 * k + 2];
        const double *kv = &kvec[3 * k];
        double p4vAkk = FOURPI * Ak[k] / volume;
        if (!(kx == lastkx && ky == lastky)) {
            for (int s = 0; s < NM; s++) {
                double tmp = CX(sinkx, s, kx) * CY(cosky, s, ky) + CX(coskx, s, kx) * CY(sinky, s, ky);
                coskxky[s] = CX(coskx, s, kx) * CY(cosky, s, ky) - CX(sinkx, s, kx) * CY(sinky, s, ky);
                sinkxky[s] = tmp;
            }
        }
        lastkx = kx;
        lastky = ky;
        for (int s = 0; s < NM; s++) {
            double tmp = sinkxky[s] * CZ(coskz, s, kz) + coskxky[s] * CZ(sinkz, s, kz);
            coskr[s] = coskxky[s] * CZ(coskz, s, kz) - sinkxky[s] * CZ(sinkz, s, kz);
            sinkr[s] = tmp;
        }
        double rQqk = 0, iQqk = 0;
        for (int s = 0; s < NM; s++) rQqk += charge[s] * coskr[s];
        for (int s = 0; s < NM; s++) iQqk += charge[s] * sinkr[s];
        for (int s = 0; s < NM; s++) {
            double tmp = p4vAkk * (coskr[s] * iQqk - sinkr[s] * rQqk);
            for (int c = 0; c < 3; c++) Efq[3 * s + c] = Efq[3 * s + c] - tmp * kv[c];
        }
        for (int s = 0; s < NM; s++) phi[s] = phi[s] + p4vAkk * (coskr[s] * rQqk + sinkr[s] * iQqk);
        double ksq = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
        double coeff2 = 2.0 / ksq + 0.5 / (aewald * aewald);
        double Ureck = -0.5 * p4vAkk * (rQqk * rQqk + iQqk * iQqk);
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double t = Ureck * coeff2 * kv[std::min(a, b)] * kv[std::max(a, b)];
                vir_rec[a + 3 * b] = (a == b) ? vir_rec[a + 3 * b] + Ureck - t : vir_rec[a + 3 * b] - t;
            }
    }
}

// find_neigh.f90:14-120: all j > iO within Rc (strict), anint min-image, ascending j
void Orc::find_neigh(int iO, std::vector<int> &nj, std::vector<double> &nR, std::vector<double> &nR2) {
    nj.clear();
    nR.clear();
    nR2.clear();
    double Ri[3] = {R[3 * iO], R[3 * iO + 1], R[3 * iO + 2]};
    for (int j = iO + 1; j < N; j++) {
        double Rij[3];
        for (int c = 0; c < 3; c++) {
            Rij[c] = Ri[c] - R[3 * j + c];
            Rij[c] = Rij[c] - box[c] * anint(Rij[c] * boxi[c]);
        }
        double R2 = Rij[0] * Rij[0] + Rij[1] * Rij[1] + Rij[2] * Rij[2];
        if (R2 < Rc2) {
            nj.push_back(j);
            nR.push_back(Rij[0]);
            nR.push_back(Rij[1]);
            nR.push_back(Rij[2]);
            nR2.push_back(R2);
        }
    }
}

// smear.f90:2-34
void Orc::smear01(double drsq, double a_pol12, double *ts0, double *ts1) {
    const double g23 = 1.3541179394264;
    double dd = std::sqrt(drsq);
    double dri = 1.0 / dd;
    double drsqi = dri * dri;
    double expon = std::exp(-(aewald * aewald * drsq));
    double er = erfc_as(aewald * dd);
    *ts0 = er * dri;
    *ts1 = (*ts0 + const_ts1 * expon) * drsqi;
    if (drsq < 25.0) {
        double rA3 = dd * drsq * a_pol12;
        double rA = std::pow(a_pol12, 1.0 / 3.0);
        double exp1 = std::exp(-rA3);
        double ch1 = -1.0 * dri * drsqi;
        double sr1 = (1.0 - exp1) * dri * drsqi;
        *ts1 = *ts1 + ch1 + sr1;
        *ts0 = *ts0 - exp1 * dri + rA * g23 * gammq2_3(rA3, &err);
    }
}

// smear.f90:36-69
void Orc::smear2(double drsq, double a_pol12, double *ts1, double *ts2) {
    double dd = std::sqrt(drsq);
    double dri = 1.0 / dd;
    double drsqi = dri * dri;
    double expon = std::exp(-(aewald * aewald * drsq));
    double er = erfc_as(aewald * dd);
    *ts1 = (er * dri + const_ts1 * expon) * drsqi;
    *ts2 = (*ts1 + const_ts2 * expon) * drsqi;
    if (drsq < 25.0) {
        double rA3 = (dd * drsq) * a_pol12;
        double exp1 = std::exp(-rA3);
        double ch1 = -1.0 * dri * drsqi;
        double ch2 = ch1 * drsqi;
        double sr1 = (1.0 - exp1) * dri * drsqi;
        double sr2 = (sr1 - exp1 * a_pol12) * drsqi;
        *ts1 = *ts1 + ch1 + sr1;
        *ts2 = *ts2 + ch2 + sr2;
    }
}

// smear.f90:71-107
void Orc::smear3(double drsq, double a_pol12, double *ts1, double *ts2, double *ts3) {
    double dd = std::sqrt(drsq);
    double dri = 1.0 / dd;
    double drsqi = dri * dri;
    double expon = std::exp(-(aewald * aewald * drsq));
    double er = erfc_as(aewald * dd);
    *ts1 = (er * dri + const_ts1 * expon) * drsqi;
    *ts2 = (*ts1 + const_ts2 * expon) * drsqi;
    *ts3 = (*ts2 + const_ts3 * expon) * drsqi;
    if (drsq < 25.0) {
        double rA3 = (dd * drsq) * a_pol12;
        double exp1 = std::exp(-rA3);
        double ch1 = -1.0 * dri * drsqi;
        double ch2 = ch1 * drsqi;
        double ch3 = ch2 * drsqi;
        double sr1 = (1.0 - exp1) * dri * drsqi;
        double sr2 = (sr1 - exp1 * a_pol12) * drsqi;
        double sr3 = (sr2 - 0.6 * exp1 * dd * a_pol12 * a_pol12) * drsqi;
        *ts1 = *ts1 + ch1 + sr1;
        *ts2 = *ts2 + ch2 + sr2;
        *ts3 = *ts3 + ch3 + sr3;
    }
}

// smear.f90:110-131
void Orc::self1(double drsq, double *ts0, double *ts1) {
    double dd = std::sqrt(drsq);
    double drsqi = 1.0 / drsq;
    double dri = std::sqrt(drsqi);
    double expon = std::exp(-(aewald * aewald * drsq));
    double kr0 = (erfc_as(aewald * dd)) * dri;
    double kr1 = (kr0 + const_ts1 * expon) * drsqi;
    double ch0 = -dri;
    double ch1 = ch0 * drsqi;
    *ts0 = ch0 + kr0;
    *ts1 = kr1 + ch1;
}

// smear.f90:133-156
void Orc::self2(double drsq, double *ts1, double *ts2) {
    double dd = std::sqrt(drsq);
    double drsqi = 1.0 / drsq;
    double dri = std::sqrt(drsqi);
    double expon = std::exp(-(aewald * aewald * drsq));
    double kr0 = (erfc_as(aewald * dd)) * dri;
    double kr1 = (kr0 + const_ts1 * expon) * drsqi;
    double kr2 = (kr1 + const_ts2 * expon) * drsqi;
    double ch0 = -dri;
    double ch1 = ch0 * drsqi;
    double ch2 = ch1 * drsqi;
    *ts1 = kr1 + ch1;
    *ts2 = kr2 + ch2;
}

// nasa.f90:2-103 pot_nasa. r1[atom][comp] = r1(comp, atom); atoms O, H1, H2.
void Orc::pot_nasa(const double r1[3][3], double dr1[3][3], double *e1) {
    double ROH1[3], ROH2[3], RHH[3];
    for (int c = 0; c < 3; c++) {
        ROH1[c] = r1[1][c] - r1[0][c];
        ROH1[c] = ROH1[c] - box[c] * anint(ROH1[c] * boxi[c]);
        ROH2[c] = r1[2][c] - r1[0][c];
        ROH2[c] = ROH2[c] - box[c] * anint(ROH2[c] * boxi[c]);
        RHH[c] = r1[1][c] - r1[2][c];
        RHH[c] = RHH[c] - box[c] * anint(RHH[c] * boxi[c]);
    }
    double dROH1 = std::sqrt(ROH1[0] * ROH1[0] + ROH1[1] * ROH1[1] + ROH1[2] * ROH1[2]);
    double dROH2 = std::sqrt(ROH2[0] * ROH2[0] + ROH2[1] * ROH2[1] + ROH2[2] * ROH2[2]);
    double dRHH = std::sqrt(RHH[0] * RHH[0] + RHH[1] * RHH[1] + RHH[2] * RHH[2]);
    double costh = (ROH1[0] * ROH2[0] + ROH1[1] * ROH2[1] + ROH1[2] * ROH2[2]) / (dROH1 * dROH2);
    const double reoh = PIMD_NASA_REOH, b1 = PIMD_NASA_B1, roh = PIMD_NASA_ROH, alphaoh = PIMD_NASA_ALPHAOH,
                 phh2 = PIMD_NASA_PHH2;
    double deoh = PIMD_NASA_F5Z * PIMD_NASA_DEOHA;
    double phh1 = PIMD_NASA_F5Z * PIMD_NASA_PHH1A;
    phh1 = phh1 * std::exp(phh2);
    const double costhe = -.24780227221366464506;
    double exp1 = std::exp(-alphaoh * (dROH1 - roh));
    double exp2 = std::exp(-alphaoh * (dROH2 - roh));
    double Va = deoh * (exp1 * (exp1 - 2.0) + exp2 * (exp2 - 2.0));
    double Vb = phh1 * std::exp(-phh2 * dRHH);
    double dVa1 = 2.0 * alphaoh * deoh * exp1 * (1.0 - exp1) / dROH1;
    double dVa2 = 2.0 * alphaoh * deoh * exp2 * (1.0 - exp2) / dROH2;
    double dVb = -phh2 * Vb / dRHH;
    double x1 = (dROH1 - reoh) / reoh;
    double x2 = (dROH2 - reoh) / reoh;
    double x3 = costh - costhe;
    double fmat[16][3];
    for (int c = 0; c < 3; c++) {
        fmat[0][c] = 0.0;
        fmat[1][c] = 1.0;
    }
    for (int j = 2; j <= 15; j++) {
        fmat[j][0] = fmat[j - 1][0] * x1;
        fmat[j][1] = fmat[j - 1][1] * x2;
        fmat[j][2] = fmat[j - 1][2] * x3;
    }
    double efac = std::exp(-b1 * ((dROH1 - reoh) * (dROH1 - reoh) + (dROH2 - reoh) * (dROH2 - reoh)));
    double sum0 = 0, sum1 = 0, sum2 = 0, sum3 = 0;
    for (int j = 1; j < 245; j++) {
        int inI = PIMD_NASA_IDX1[j], inJ = PIMD_NASA_IDX2[j], inK = PIMD_NASA_IDX3[j];
        sum0 = sum0 + c5z[j] * (fmat[inI][0] * fmat[inJ][1] + fmat[inJ][0] * fmat[inI][1]) * fmat[inK][2];
        sum1 = sum1 + c5z[j] * ((double)(inI - 1) * fmat[inI - 1][0] * fmat[inJ][1] +
                                (double)(inJ - 1) * fmat[inJ - 1][0] * fmat[inI][1]) * fmat[inK][2];
        sum2 = sum2 + c5z[j] * ((double)(inJ - 1) * fmat[inI][0] * fmat[inJ - 1][1] +
                                (double)(inI - 1) * fmat[inJ][0] * fmat[inI - 1][1]) * fmat[inK][2];
        sum3 = sum3 + c5z[j] * (fmat[inI][0] * fmat[inJ][1] + fmat[inJ][0] * fmat[inI][1]) *
                          (double)(inK - 1) * fmat[inK - 1][2];
    }
    double Vc = 2.0 * c5z[0] + efac * sum0;
    double e = Va + Vb + Vc;
    e = e + 0.44739574026257;
    e = e * 0.00285914375100642899;
    *e1 = e;
    double dVcdr1 = (-2.0 * b1 * efac * (dROH1 - reoh) * sum0 + efac * sum1 / reoh) / dROH1;
    double dVcdr2 = (-2.0 * b1 * efac * (dROH2 - reoh) * sum0 + efac * sum2 / reoh) / dROH2;
    double dVcdcth = efac * sum3;
    for (int c = 0; c < 3; c++) {
        dr1[1][c] = dVa1 * ROH1[c] + dVb * RHH[c] + dVcdr1 * ROH1[c] +
                    dVcdcth * (ROH2[c] / (dROH1 * dROH2) - costh * ROH1[c] / (dROH1 * dROH1));
        dr1[2][c] = dVa2 * ROH2[c] - dVb * RHH[c] + dVcdr2 * ROH2[c] +
                    dVcdcth * (ROH1[c] / (dROH1 * dROH2) - costh * ROH2[c] / (dROH2 * dROH2));
        dr1[0][c] = -(dr1[1][c] + dr1[2][c]);
    }
    for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++) dr1[a][c] = dr1[a][c] * .00285914375100642899;
}

// nasa.f90:105-293 dms_nasa. gradq[a][b][c] = gradq(a+1, b+1, c+1).
void Orc::dms_nasa(const double r1[3][3], double q3[3], double gradq[3][3][3]) {
    const double reoh = PIMD_NASA_REOH, b1D = PIMD_NASA_B1D, a = PIMD_NASA_A, b = PIMD_NASA_B,
                 c0 = PIMD_NASA_C0, c1 = PIMD_NASA_C1, c2 = PIMD_NASA_C2;
    const double ath0 = 1.82400520401572996557;
    const double costhe = -.24780227221366464506;
    const double B2A = 0.529177249;
    double ROH1[3], ROH2[3], RHH[3];
    for (int c = 0; c < 3; c++) {
        ROH1[c] = r1[1][c] - r1[0][c];
        ROH1[c] = ROH1[c] - box[c] * anint(ROH1[c] * boxi[c]);
        ROH2[c] = r1[2][c] - r1[0][c];
        ROH2[c] = ROH2[c] - box[c] * anint(ROH2[c] * boxi[c]);
        RHH[c] = r1[1][c] - r1[2][c];
        RHH[c] = RHH[c] - box[c] * anint(RHH[c] * boxi[c]);
    }
    double dROH1 = std::sqrt(ROH1[0] * ROH1[0] + ROH1[1] * ROH1[1] + ROH1[2] * ROH1[2]);
    double dROH2 = std::sqrt(ROH2[0] * ROH2[0] + ROH2[1] * ROH2[1] + ROH2[2] * ROH2[2]);
    double costh = (ROH1[0] * ROH2[0] + ROH1[1] * ROH2[1] + ROH1[2] * ROH2[2]) / (dROH1 * dROH2);
    double efac = std::exp(-b1D * ((dROH1 - reoh) * (dROH1 - reoh) + (dROH2 - reoh) * (dROH2 - reoh)));
    double x1 = (dROH1 - reoh) / reoh;
    double x2 = (dROH2 - reoh) / reoh;
    double x3 = costh - costhe;
    double fmat[16][3];
    for (int c = 0; c < 3; c++) {
        fmat[0][c] = 0.0;
        fmat[1][c] = 1.0;
    }
    for (int j = 2; j <= 15; j++) {
        fmat[j][0] = fmat[j - 1][0] * x1;
        fmat[j][1] = fmat[j - 1][1] * x2;
        fmat[j][2] = fmat[j - 1][2] * x3;
    }
    double P1 = 0, P2 = 0, PL1 = costh, PL2 = 0.5 * (3.0 * PL1 * PL1 - 1.0);
    double dp1dr1 = 0, dp1dr2 = 0, dp1dcabc = 0, dp2dr1 = 0, dp2dr2 = 0, dp2dcabc = 0;
    for (int j = 1; j < 84; j++) {
        int inI = PIMD_NASA_IDXD1[j], inJ = PIMD_NASA_IDXD2[j], inK = PIMD_NASA_IDXD3[j];
        double cf = PIMD_NASA_COEFD[j];
        P1 = P1 + cf * fmat[inI][0] * fmat[inJ][1] * fmat[inK][2];
        P2 = P2 + cf * fmat[inJ][0] * fmat[inI][1] * fmat[inK][2];
        dp1dr1 = dp1dr1 + cf * ((double)(inI - 1) * fmat[inI - 1][0] * fmat[inJ][1] * fmat[inK][2]);
        dp1dr2 = dp1dr2 + cf * ((double)(inJ - 1) * fmat[inI][0] * fmat[inJ - 1][1] * fmat[inK][2]);
        dp1dcabc = dp1dcabc + cf * ((double)(inK - 1) * fmat[inI][0] * fmat[inJ][1] * fmat[inK - 1][2]);
        dp2dr1 = dp2dr1 + cf * ((double)(inJ - 1) * fmat[inJ - 1][0] * fmat[inI][1] * fmat[inK][2]);
        dp2dr2 = dp2dr2 + cf * ((double)(inI - 1) * fmat[inJ][0] * fmat[inI - 1][1] * fmat[inK][2]);
        dp2dcabc = dp2dcabc + cf * ((double)(inK - 1) * fmat[inJ][0] * fmat[inI][1] * fmat[inK - 1][2]);
    }
    dp1dr1 = dp1dr1 / reoh * B2A;
    dp1dr2 = dp1dr2 / reoh * B2A;
    dp2dr1 = dp2dr1 / reoh * B2A;
    dp2dr2 = dp2dr2 / reoh * B2A;
    double PC0 = a * (std::pow(dROH1, b) + std::pow(dROH2, b)) * (c0 + PL1 * c1 + PL2 * c2);
    double dpc0dr1 = a * (b * std::pow(dROH1, b - 1)) * (c0 + PL1 * c1 + PL2 * c2) * B2A * B2A;
    double dpc0dr2 = a * (b * std::pow(dROH2, b - 1)) * (c0 + PL1 * c1 + PL2 * c2) * B2A * B2A;
    double dpc0dcabc = a * (std::pow(dROH1, b) + std::pow(dROH2, b)) * (c1 + 0.5 * (6.0 * PL1) * c2) * B2A;
    double defacdr1 = -2.0 * b1D * (dROH1 - reoh) * efac * B2A;
    double defacdr2 = -2.0 * b1D * (dROH2 - reoh) * efac * B2A;
    dp1dr1 = dp1dr1 * efac + P1 * defacdr1 + dpc0dr1;
    dp1dr2 = dp1dr2 * efac + P1 * defacdr2 + dpc0dr2;
    dp1dcabc = dp1dcabc * efac + dpc0dcabc;
    dp2dr1 = dp2dr1 * efac + P2 * defacdr1 + dpc0dr1;
    dp2dr2 = dp2dr2 * efac + P2 * defacdr2 + dpc0dr2;
    dp2dcabc = dp2dcabc * efac + dpc0dcabc;
    P1 = PIMD_NASA_COEFD[0] + P1 * efac + PC0 * B2A;
    P2 = PIMD_NASA_COEFD[0] + P2 * efac + PC0 * B2A;
    // nasa.f90:218 bfac = 1.d0/0.529177249 -- the divisor is a single-precision literal
    double bfac = 1.0 / (double)0.529177249f;
    q3[0] = -(P1 + P2);
    q3[1] = P1;
    q3[2] = P2;
    dp1dr1 = dp1dr1 * bfac;
    dp1dr2 = dp1dr2 * bfac;
    dp2dr1 = dp2dr1 * bfac;
    dp2dr2 = dp2dr2 * bfac;
    double AxB[3];
    AxB[0] = ROH1[1] * ROH2[2] - ROH1[2] * ROH2[1];
    AxB[1] = -ROH1[0] * ROH2[2] + ROH1[2] * ROH2[0];
    AxB[2] = ROH1[0] * ROH2[1] - ROH1[1] * ROH2[0];
    double dAxB = std::sqrt(AxB[0] * AxB[0] + AxB[1] * AxB[1] + AxB[2] * AxB[2]);
    double sinth = dAxB / (dROH1 * dROH2);
    double ang = std::atan2(sinth, costh);
    P1 = m.dms1 * (dROH1 - m.dms2) + m.dms3 * (ang - ath0);
    P2 = m.dms1 * (dROH2 - m.dms2) + m.dms3 * (ang - ath0);
    q3[0] = q3[0] - (P1 + P2);
    q3[1] = q3[1] + P1;
    q3[2] = q3[2] + P2;
    dp1dr1 = dp1dr1 + m.dms1;
    dp2dr2 = dp2dr2 + m.dms1;
    dp1dcabc = dp1dcabc - m.dms3 / sinth;
    dp2dcabc = dp2dcabc - m.dms3 / sinth;
    double f1q1r13 = (dp1dr1 - (dp1dcabc * costh / dROH1)) / dROH1;
    double f1q1r23 = dp1dcabc / (dROH1 * dROH2);
    double f2q1r23 = (dp1dr2 - (dp1dcabc * costh / dROH2)) / dROH2;
    double f2q1r13 = dp1dcabc / (dROH2 * dROH1);
    double f1q2r13 = (dp2dr1 - (dp2dcabc * costh / dROH1)) / dROH1;
    double f1q2r23 = dp2dcabc / (dROH1 * dROH2);
    double f2q2r23 = (dp2dr2 - (dp2dcabc * costh / dROH2)) / dROH2;
    double f2q2r13 = dp2dcabc / (dROH2 * dROH1);
    for (int c = 0; c < 3; c++) {
        gradq[0][0][c] = f1q1r13 * ROH1[c] + f1q1r23 * ROH2[c];
        gradq[1][0][c] = f2q1r13 * ROH1[c] + f2q1r23 * ROH2[c];
        gradq[2][0][c] = -(gradq[0][0][c] + gradq[1][0][c]);
        gradq[0][1][c] = f1q2r13 * ROH1[c] + f1q2r23 * ROH2[c];
        gradq[1][1][c] = f2q2r13 * ROH1[c] + f2q2r23 * ROH2[c];
        gradq[2][1][c] = -(gradq[0][1][c] + gradq[1][1][c]);
        gradq[0][2][c] = -(gradq[0][0][c] + gradq[0][1][c]);
        gradq[1][2][c] = -(gradq[1][0][c] + gradq[1][1][c]);
        gradq[2][2][c] = -(gradq[2][0][c] + gradq[2][1][c]);
    }
}

static void get_dd3(const double R[3], double ts1, double ts2, double dd3[3][3]) {
    // pot_ttm.f90:633-647 (dd3 symmetric, [a][b] = dd3(a+1,b+1))
    dd3[0][0] = 3.0 * ts2 * R[0] * R[0] - ts1;
    dd3[1][1] = 3.0 * ts2 * R[1] * R[1] - ts1;
    dd3[2][2] = 3.0 * ts2 * R[2] * R[2] - ts1;
    dd3[0][1] = 3.0 * ts2 * R[0] * R[1];
    dd3[0][2] = 3.0 * ts2 * R[0] * R[2];
    dd3[1][2] = 3.0 * ts2 * R[1] * R[2];
    dd3[1][0] = dd3[0][1];
    dd3[2][0] = dd3[0][2];
    dd3[2][1] = dd3[1][2];
}

// pot_ttm.f90:649-675
static void calc_dpcf(int md_step, double dpcf[4]) {
    static const double t0[4] = {-1, 4, -6, 4}, t1[4] = {4, -1, 4, -6}, t2[4] = {-6, 4, -1, 4},
                        t3[4] = {4, -6, 4, -1};
    const double *src = t0;
    if (md_step < 4) {
        static const double s1[4] = {1, 0, 0, 0}, s2[4] = {-1, 2, 0, 0}, s3[4] = {1, -3, 3, 0};
        src = md_step == 1 ? s1 : md_step == 2 ? s2 : s3;
    } else {
        int itmp = md_step % 4;
        src = itmp == 0 ? t0 : itmp == 1 ? t1 : itmp == 2 ? t2 : t3;
    }
    for (int i = 0; i < 4; i++) dpcf[i] = src[i];
}

// pot_ttm.f90:3-630
void Orc::pot_ttm(int bead, const double *RR, const double *RRc, double *En, double *dRR, double *virt,
                  double *virialc_out, double *dip_momI, double *Edip_mom, double *chg, int t) {
    // virt(a,b) -> virt[a + 3*b]
    for (int i = 0; i < 9; i++) {
        virt[i] = 0.0;
        vir_rec[i] = 0.0;
    }
    double virialc = 0.0;
    Umon = Uvdw = Uelec = 0.0;
    std::fill(phi.begin(), phi.end(), 0.0);
    std::fill(Efq.begin(), Efq.end(), 0.0);
    std::fill(dip.begin(), dip.end(), 0.0);
    std::fill(olddip.begin(), olddip.end(), 0.0);
    std::fill(dR.begin(), dR.end(), 0.0);
    const double gammaM = m.gammaM;
    // 56-80 reorder and M sites
    for (int iw = 0; iw < N; iw++) {
        int ia[3] = {3 * iw, 3 * iw + 1, 3 * iw + 2};
        int is[3] = {iw, iw + N, iw + 2 * N};
        int iM = iw + 3 * N;
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++) {
                R[3 * is[k] + c] = RR[3 * ia[k] + c];
                RRRc[3 * is[k] + c] = RRc[3 * ia[k] + c];
            }
        for (int pass = 0; pass < 2; pass++) {
            std::vector<double> &A = pass == 0 ? R : RRRc;
            double roh1[3], roh2[3];
            for (int c = 0; c < 3; c++) {
                roh1[c] = A[3 * is[1] + c] - A[3 * is[0] + c];
                roh1[c] = roh1[c] - box[c] * anint(roh1[c] * boxi[c]);
                roh2[c] = A[3 * is[2] + c] - A[3 * is[0] + c];
                roh2[c] = roh2[c] - box[c] * anint(roh2[c] * boxi[c]);
            }
            for (int c = 0; c < 3; c++) A[3 * iM + c] = 0.5 * gammaM * (roh1[c] + roh2[c]) + A[3 * is[0] + c];
        }
    }
    // 84-151 monomer PES, DMS charges
    double tmp = 0.5 * gammaM / (1.0 - gammaM);
    std::fill(charge.begin(), charge.end(), 0.0);
    std::fill(grdq.begin(), grdq.end(), 0.0);
    std::fill(dR.begin(), dR.end(), 0.0);
    for (int iw = 0; iw < N; iw++) {
        int iO = iw, iH1 = iw + N, iH2 = iw + 2 * N, iM = iw + 3 * N;
        double r1[3][3], dr1[3][3], e1, q3[3], dq3[3][3][3];
        int sidx[3] = {iO, iH1, iH2};
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++) r1[k][c] = R[3 * sidx[k] + c];
        if (!p.contraction) {
            pot_nasa(r1, dr1, &e1);
            Umon = Umon + e1;
            for (int k = 0; k < 3; k++)
                for (int c = 0; c < 3; c++) dR[3 * sidx[k] + c] = dr1[k][c];
        } else {
            for (int k = 0; k < 3; k++)
                for (int c = 0; c < 3; c++) dr1[k][c] = 0.0;
            Umon = 0;
        }
        dms_nasa(r1, q3, dq3);
        for (int k = 0; k < 3; k++) q3[k] = q3[k] * CHARGECON;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                for (int c = 0; c < 3; c++) dq3[a][b][c] = dq3[a][b][c] * CHARGECON;
        for (int k = 0; k < 3; k++) chg[3 * iw + k] = q3[k];
        if (!p.contraction) {
            double roh1[3], roh2[3];
            for (int c = 0; c < 3; c++) {
                roh1[c] = r1[1][c] - r1[0][c];
                roh1[c] = roh1[c] - box[c] * anint(roh1[c] * boxi[c]);
                roh2[c] = r1[2][c] - r1[0][c];
                roh2[c] = roh2[c] - box[c] * anint(roh2[c] * boxi[c]);
            }
            for (int col = 0; col < 3; col++)
                for (int c = 0; c < 3; c++)
                    virt[c + 3 * col] = virt[c + 3 * col] + roh1[c] * dr1[1][col] + roh2[c] * dr1[2][col];
            for (int k = 0; k < 3; k++)
                for (int c = 0; c < 3; c++) r1[k][c] = RRRc[3 * sidx[k] + c];
            for (int c = 0; c < 3; c++) {
                roh1[c] = r1[1][c] - r1[0][c];
                roh1[c] = roh1[c] - box[c] * anint(roh1[c] * boxi[c]);
                roh2[c] = r1[2][c] - r1[0][c];
                roh2[c] = roh2[c] - box[c] * anint(roh2[c] * boxi[c]);
            }
            virialc = virialc + (roh1[0] * dr1[1][0] + roh1[1] * dr1[1][1] + roh1[2] * dr1[1][2]);
            virialc = virialc + (roh2[0] * dr1[2][0] + roh2[1] * dr1[2][1] + roh2[2] * dr1[2][2]);
        }
        charge[iO] = 0.0;
        charge[iH1] = q3[1] + tmp * (q3[1] + q3[2]);
        charge[iH2] = q3[2] + tmp * (q3[1] + q3[2]);
        charge[iM] = q3[0] / (1.0 - gammaM);
        // grdq(iw, a, b, c) -> grdq[27*iw + 9*a + 3*b + c]
        double *g = &grdq[27 * iw];
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) {
                g[9 * a + 3 * 0 + c] = dq3[a][0][c] + tmp * (dq3[a][0][c] + dq3[a][1][c]);
                g[9 * a + 3 * 1 + c] = dq3[a][1][c] + tmp * (dq3[a][0][c] + dq3[a][1][c]);
                g[9 * a + 3 * 2 + c] = dq3[a][2][c] - 2.0 * tmp * (dq3[a][0][c] + dq3[a][1][c]);
            }
    }

    std::vector<int> nj;
    std::vector<double> nR, nR2;
    double ts0 = 0, ts1 = 0, ts2 = 0, ts3 = 0;  // persist across phases like the Fortran locals
    // 159-228 real space vdW + charge-charge
    for (int iw = 0; iw < N; iw++) {
        int iO = iw;
        find_neigh(iO, nj, nR, nR2);
        for (size_t j = 0; j < nj.size(); j++) {
            int jO = nj[j];
            double Rij[3] = {nR[3 * j], nR[3 * j + 1], nR[3 * j + 2]};
            double dRsq = nR2[j];
            double dRij = std::sqrt(dRsq);
            double R2i = 1.0 / dRsq, R4i = R2i * R2i, R6i = R2i * R2i * R2i, R8i = R6i * R2i;
            double tmpv = m.vdwD * std::exp(-m.vdwE * dRij);
            double uij = R6i * ((m.vdwA * R6i + m.vdwB * R4i) + m.vdwC) + tmpv;
            double xr = dRij - rc1;
            double sc = R8i * 6.0 * m.vdwC + tmpv * m.vdwE / dRij + shiftA * (xr * xr) + shiftB * (xr * xr * xr);
            double dij[3];
            for (int c = 0; c < 3; c++) dij[c] = -(sc * Rij[c]);
            Uvdw = Uvdw + uij;
            for (int c = 0; c < 3; c++) {
                dR[3 * iO + c] = dR[3 * iO + c] + dij[c];
                dR[3 * jO + c] = dR[3 * jO + c] - dij[c];
            }
            double Rcij[3];
            for (int c = 0; c < 3; c++) {
                Rcij[c] = RRRc[3 * iO + c] - RRRc[3 * jO + c];
                Rcij[c] = Rcij[c] - box[c] * anint(Rcij[c] * boxi[c]);
            }
            virialc = virialc + (Rcij[0] * dij[0] + Rcij[1] * dij[1] + Rcij[2] * dij[2]);
            for (int col = 0; col < 3; col++)
                for (int c = 0; c < 3; c++) virt[c + 3 * col] = virt[c + 3 * col] + dij[col] * Rij[c];
            double Rij0[3];
            for (int c = 0; c < 3; c++) Rij0[c] = Rij[c] - R[3 * iO + c] + R[3 * jO + c];
            for (int isp = 1; isp <= 4; isp++) {
                int iat = iw + (isp - 1) * N;
                double Ri[3];
                for (int c = 0; c < 3; c++) Ri[c] = R[3 * iat + c] + Rij0[c];
                double qi = charge[iat];
                double polfacI = m.aCCaCD * polfac[isp];
                int jsp0 = (isp == 1) ? 2 : 1;
                for (int jsp = jsp0; jsp <= 4; jsp++) {
                    int jat = jO + (jsp - 1) * N;
                    double qj = charge[jat];
                    double Rs[3];
                    for (int c = 0; c < 3; c++) {
                        Rs[c] = Ri[c] - R[3 * jat + c];
                        Rs[c] = Rs[c] - box[c] * anint(Rs[c] * boxi[c]);
                    }
                    double d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                    smear01(d2, polfacI * polfac[jsp], &ts0, &ts1);
                    phi[iat] = phi[iat] + ts0 * qj;
                    phi[jat] = phi[jat] + ts0 * qi;
                    double d[3];
                    for (int c = 0; c < 3; c++) {
                        Efq[3 * iat + c] = Efq[3 * iat + c] + ts1 * qj * Rs[c];
                        Efq[3 * jat + c] = Efq[3 * jat + c] - ts1 * qi * Rs[c];
                        d[c] = -ts1 * qi * qj * Rs[c];
                    }
                    double Rc2v[3];
                    for (int c = 0; c < 3; c++) Rc2v[c] = RRRc[3 * iat + c] - RRRc[3 * jat + c] + Rij0[c];
                    virialc = virialc + (Rc2v[0] * d[0] + Rc2v[1] * d[1] + Rc2v[2] * d[2]);
                    for (int col = 0; col < 3; col++)
                        for (int c = 0; c < 3; c++) virt[c + 3 * col] = virt[c + 3 * col] + d[col] * Rs[c];
                }
            }
        }
    }
    // 232-261 self energy
    for (int iat = N; iat < 4 * N; iat++) phi[iat] = phi[iat] - aewald * TSP * charge[iat];
    for (int iw = 0; iw < N; iw++)
        for (int isp = 1; isp <= 3; isp++) {
            int iat = iw + (isp - 1) * N;
            for (int jsp = isp + 1; jsp <= 4; jsp++) {
                int jat = iw + (jsp - 1) * N;
                double Rs[3];
                for (int c = 0; c < 3; c++) {
                    Rs[c] = R[3 * iat + c] - R[3 * jat + c];
                    Rs[c] = Rs[c] - box[c] * anint(Rs[c] * boxi[c]);
                }
                double d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                self1(d2, &ts0, &ts1);
                phi[iat] = phi[iat] + ts0 * charge[jat];
                phi[jat] = phi[jat] + ts0 * charge[iat];
                double d[3];
                for (int c = 0; c < 3; c++) {
                    Efq[3 * iat + c] = Efq[3 * iat + c] + ts1 * charge[jat] * Rs[c];
                    Efq[3 * jat + c] = Efq[3 * jat + c] - ts1 * charge[iat] * Rs[c];
                    d[c] = -ts1 * charge[iat] * charge[jat] * Rs[c];
                }
                double Rcij[3];
                for (int c = 0; c < 3; c++) {
                    Rcij[c] = RRRc[3 * iat + c] - RRRc[3 * jat + c];
                    Rcij[c] = Rcij[c] - box[c] * anint(Rcij[c] * boxi[c]);
                }
                virialc = virialc + (Rcij[0] * d[0] + Rcij[1] * d[1] + Rcij[2] * d[2]);
                for (int col = 0; col < 3; col++)
                    for (int c = 0; c < 3; c++) virt[c + 3 * col] = virt[c + 3 * col] + d[col] * Rs[c];
            }
        }
    // 269-277 reciprocal space (charges)
    ewald_std_qq();
    {
        double s = 0;
        for (int iat = N; iat < 4 * N; iat++) s += charge[iat] * phi[iat];
        Uelec = 0.5 * s;
    }
    for (int iat = N; iat < 4 * N; iat++)
        for (int c = 0; c < 3; c++) dR[3 * iat + c] = dR[3 * iat + c] - charge[iat] * Efq[3 * iat + c];
    // 281-297 initial guess of the induced dipoles
    int slot = p.shared_history ? 0 : bead;
    double *hist = &tx_dip[(size_t)slot * 4 * 3 * NM];  // [h][3*NM]
    int predict_step = t;
    if (predict_step > 4 && p.guess_initdip) {
        double dpcf[4];
        calc_dpcf(predict_step, dpcf);
        for (int i = 3 * fd; i < 3 * (ld + 1); i++)
            dip[i] = dpcf[0] * hist[i] + dpcf[1] * hist[3 * NM + i] + dpcf[2] * hist[6 * NM + i] +
                     dpcf[3] * hist[9 * NM + i];
    } else {
        if (p.pot_model == 2) {
            for (int i = 0; i < 3 * N; i++) dip[i] = m.polarO * Efq[i];
            for (int i = 3 * N; i < 9 * N; i++) dip[i] = m.polarH * Efq[i];
        } else {
            for (int i = 9 * N; i < 12 * N; i++) dip[i] = m.polarM * Efq[i];
        }
    }
    // 306-386 induced dipole iterations
    double stath = DEBYE / CHARGECON / std::sqrt((double)Natoms);
    double factor = 4.0 * (aewald * aewald * aewald) / (3.0 * std::sqrt(PI));
    int iter;
    double deltadip = 0;
    for (iter = 1; iter <= p.polar_maxiter; iter++) {
        std::fill(Efd.begin(), Efd.end(), 0.0);
        for (int i = 0; i < N; i++) {
            int iO = i;
            find_neigh(iO, nj, nR, nR2);
            for (size_t j = 0; j < nj.size(); j++) {
                int jO = nj[j];
                double Rij0[3];
                for (int c = 0; c < 3; c++) {
                    Rij0[c] = nR[3 * j + c] - R[3 * iO + c] + R[3 * jO + c];
                    Rij0[c] = Rij0[c] - box[c] * anint(Rij0[c] * boxi[c]);
                }
                for (int isp = fdI; isp <= ldI; isp++) {
                    int iat = iO + (isp - 1) * N;
                    double polfacI = m.aDD * polfac[isp];
                    double di[3] = {dip[3 * iat], dip[3 * iat + 1], dip[3 * iat + 2]};
                    double Ri[3];
                    for (int c = 0; c < 3; c++) Ri[c] = R[3 * iat + c] + Rij0[c];
                    for (int jsp = fdI; jsp <= ldI; jsp++) {
                        int jat = jO + (jsp - 1) * N;
                        double dj[3] = {dip[3 * jat], dip[3 * jat + 1], dip[3 * jat + 2]};
                        double Rs[3];
                        for (int c = 0; c < 3; c++) {
                            Rs[c] = Ri[c] - R[3 * jat + c];
                            Rs[c] = Rs[c] - box[c] * anint(Rs[c] * boxi[c]);
                        }
                        double d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                        double t1, t2, dd3[3][3];
                        smear2(d2, polfacI * polfac[jsp], &t1, &t2);
                        get_dd3(Rs, t1, t2, dd3);
                        for (int c = 0; c < 3; c++) {
                            Efd[3 * iat + c] = Efd[3 * iat + c] + dd3[0][c] * dj[0] + dd3[1][c] * dj[1] + dd3[2][c] * dj[2];
                        }
                        for (int c = 0; c < 3; c++) {
                            Efd[3 * jat + c] = Efd[3 * jat + c] + dd3[0][c] * di[0] + dd3[1][c] * di[1] + dd3[2][c] * di[2];
                        }
                    }
                }
            }
        }
        for (int iw = 0; iw < N; iw++)
            for (int isp = fdI; isp <= ldI - 1; isp++) {
                int iat = iw + (isp - 1) * N;
                double di[3] = {dip[3 * iat], dip[3 * iat + 1], dip[3 * iat + 2]};
                double polfacI = m.aDD * polfac[isp];
                for (int jsp = isp + 1; jsp <= ldI; jsp++) {
                    int jat = iw + (jsp - 1) * N;
                    double dj[3] = {dip[3 * jat], dip[3 * jat + 1], dip[3 * jat + 2]};
                    double Rs[3];
                    for (int c = 0; c < 3; c++) {
                        Rs[c] = (R[3 * iat + c] - R[3 * jat + c]);
                        Rs[c] = Rs[c] - box[c] * anint(Rs[c] * boxi[c]);
                    }
                    double d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                    double t1, t2, dd3[3][3];
                    smear2(d2, polfacI * polfac[jsp], &t1, &t2);
                    get_dd3(Rs, t1, t2, dd3);
                    for (int c = 0; c < 3; c++)
                        Efd[3 * iat + c] = Efd[3 * iat + c] + dd3[0][c] * dj[0] + dd3[1][c] * dj[1] + dd3[2][c] * dj[2];
                    for (int c = 0; c < 3; c++)
                        Efd[3 * jat + c] = Efd[3 * jat + c] + dd3[0][c] * di[0] + dd3[1][c] * di[1] + dd3[2][c] * di[2];
                }
            }
        ewald_std_dd();
        for (int i = 3 * fd; i < 3 * (ld + 1); i++) Efd[i] = Efd[i] + Efq[i] + factor * dip[i];
        if (p.pot_model == 2) {
            for (int i = 0; i < 3 * N; i++) dip[i] = (1.0 - p.polar_sor) * dip[i] + p.polar_sor * m.polarO * Efd[i];
            for (int i = 3 * N; i < 9 * N; i++) dip[i] = (1.0 - p.polar_sor) * dip[i] + p.polar_sor * m.polarH * Efd[i];
        } else {
            for (int i = 9 * N; i < 12 * N; i++) dip[i] = (1.0 - p.polar_sor) * dip[i] + p.polar_sor * m.polarM * Efd[i];
        }
        {
            double s = 0;
            for (int i = 3 * fd; i < 3 * (ld + 1); i++) s += dip[i] * Efq[i];
            Uind = -0.5 * s;
        }
        {
            double s = 0;
            for (int i = 3 * fd; i < 3 * (ld + 1); i++) s += (dip[i] - olddip[i]) * (dip[i] - olddip[i]);
            deltadip = stath * std::sqrt(s);
        }
        if (deltadip < p.polar_eps) break;
        olddip = dip;
    }
    niter = iter;
    deltadip_last = deltadip;
    {
        double s = 0;
        for (int i = 3 * fd; i < 3 * (ld + 1); i++) s += dip[i] * Efq[i];
        Uind = -0.5 * s;
    }
    int itmp = predict_step % 4;
    if (p.guess_initdip)
        for (int i = 3 * fd; i < 3 * (ld + 1); i++) hist[(size_t)itmp * 3 * NM + i] = dip[i];

    // 399-478 forces for dipoles (real space)
    for (int iw = 0; iw < N; iw++) {
        int iO = iw;
        find_neigh(iO, nj, nR, nR2);
        for (size_t j = 0; j < nj.size(); j++) {
            int jO = nj[j];
            double Rij0[3];
            for (int c = 0; c < 3; c++) {
                Rij0[c] = nR[3 * j + c] - R[3 * iO + c] + R[3 * jO + c];
                Rij0[c] = Rij0[c] - box[c] * anint(Rij0[c] * boxi[c]);
            }
            for (int isp = 1; isp <= 4; isp++) {
                int iat = iO + (isp - 1) * N;
                double Ri[3];
                for (int c = 0; c < 3; c++) Ri[c] = R[3 * iat + c] + Rij0[c];
                double qi = charge[iat];
                bool idip = (isp >= fdI && isp <= ldI);
                double di[3] = {0, 0, 0};
                if (idip)
                    for (int c = 0; c < 3; c++) di[c] = dip[3 * iat + c];
                double polfacI = polfac[isp];
                for (int jsp = 1; jsp <= 4; jsp++) {
                    int jat = jO + (jsp - 1) * N;
                    double Rs[3];
                    for (int c = 0; c < 3; c++) {
                        Rs[c] = Ri[c] - R[3 * jat + c];
                        Rs[c] = Rs[c] - box[c] * anint(Rs[c] * boxi[c]);
                    }
                    double d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                    double qj = charge[jat];
                    bool jdip = (jsp >= fdI && jsp <= ldI);
                    double dj[3] = {0, 0, 0};
                    if (jdip)
                        for (int c = 0; c < 3; c++) dj[c] = dip[3 * jat + c];
                    double dij[3] = {0, 0, 0};
                    double qdqd[3];
                    for (int c = 0; c < 3; c++) qdqd[c] = qj * di[c] - qi * dj[c];
                    double qdqd_sq = qdqd[0] * qdqd[0] + qdqd[1] * qdqd[1] + qdqd[2] * qdqd[2];
                    if (idip && jdip) {
                        double t1DD, t2DD, t3DD;
                        smear3(d2, m.aDD * polfacI * polfac[jsp], &t1DD, &t2DD, &t3DD);
                        double TS[3][3][3];
                        for (int a = 0; a < 3; a++)
                            for (int b = 0; b < 3; b++)
                                for (int c = 0; c < 3; c++) TS[a][b][c] = 15.0 * Rs[a] * Rs[b] * Rs[c] * t3DD;
                        for (int jj = 0; jj < 3; jj++) {
                            for (int a = 0; a < 3; a++) TS[a][jj][jj] = TS[a][jj][jj] - 3.0 * t2DD * Rs[a];
                            for (int a = 0; a < 3; a++) TS[jj][a][jj] = TS[jj][a][jj] - 3.0 * t2DD * Rs[a];
                            for (int a = 0; a < 3; a++) TS[jj][jj][a] = TS[jj][jj][a] - 3.0 * t2DD * Rs[a];
                        }
                        double arr33[3][3];
                        for (int a = 0; a < 3; a++)
                            for (int b = 0; b < 3; b++)
                                arr33[a][b] = TS[a][b][0] * dj[0] + TS[a][b][1] * dj[1] + TS[a][b][2] * dj[2];
                        for (int c = 0; c < 3; c++)
                            dij[c] = dij[c] + di[0] * arr33[0][c] + di[1] * arr33[1][c] + di[2] * arr33[2][c];
                        if (qdqd_sq > 1.e-9) {
                            if (std::fabs(m.aCCaCD - m.aDD) < 1.e-12) {
                                ts1 = t1DD;
                                ts2 = t2DD;
                            } else {
                                smear2(d2, m.aCCaCD * polfacI * polfac[jsp], &ts1, &ts2);
                            }
                            double dd3[3][3];
                            get_dd3(Rs, ts1, ts2, dd3);
                            for (int c = 0; c < 3; c++)
                                dij[c] = dij[c] + dd3[0][c] * qdqd[0] + dd3[1][c] * qdqd[1] + dd3[2][c] * qdqd[2];
                        }
                    } else {
                        if (qdqd_sq > 1.e-9) {
                            smear2(d2, m.aCCaCD * polfacI * polfac[jsp], &ts1, &ts2);
                            double dd3[3][3];
                            get_dd3(Rs, ts1, ts2, dd3);
                            for (int c = 0; c < 3; c++)
                                dij[c] = dij[c] + dd3[0][c] * qdqd[0] + dd3[1][c] * qdqd[1] + dd3[2][c] * qdqd[2];
                        }
                    }
                    phi[iat] = phi[iat] + ts1 * (Rs[0] * dj[0] + Rs[1] * dj[1] + Rs[2] * dj[2]);
                    phi[jat] = phi[jat] - ts1 * (Rs[0] * di[0] + Rs[1] * di[1] + Rs[2] * di[2]);
                    for (int c = 0; c < 3; c++) {
                        dR[3 * iat + c] = dR[3 * iat + c] + dij[c];
                        dR[3 * jat + c] = dR[3 * jat + c] - dij[c];
                    }
                    double Rcij[3];
                    for (int c = 0; c < 3; c++) Rcij[c] = RRRc[3 * iat + c] - RRRc[3 * jat + c] + Rij0[c];
                    virialc = virialc + (Rcij[0] * dij[0] + Rcij[1] * dij[1] + Rcij[2] * dij[2]);
                    for (int col = 0; col < 3; col++)
                        for (int c = 0; c < 3; c++) virt[c + 3 * col] = virt[c + 3 * col] + dij[c] * Rs[col];
                }
            }
        }
    }
    // 482-542 intramolecular (self) dipole forces
    for (int iw = 0; iw < N; iw++)
        for (int isp = 1; isp <= 3; isp++) {
            int iat = iw + (isp - 1) * N;
            double qi = charge[iat];
            bool idip = (isp >= fdI && isp <= ldI);
            double di[3] = {0, 0, 0};
            if (idip)
                for (int c = 0; c < 3; c++) di[c] = dip[3 * iat + c];
            for (int jsp = isp + 1; jsp <= 4; jsp++) {
                int jat = iw + (jsp - 1) * N;
                double qj = charge[jat];
                bool jdip = (jsp >= fdI && jsp <= ldI);
                double dj[3] = {0, 0, 0};
                if (jdip)
                    for (int c = 0; c < 3; c++) dj[c] = dip[3 * jat + c];
                double Rs[3], Rcij[3];
                for (int c = 0; c < 3; c++) {
                    Rs[c] = R[3 * iat + c] - R[3 * jat + c];
                    Rs[c] = Rs[c] - box[c] * anint(Rs[c] * boxi[c]);
                    Rcij[c] = RRRc[3 * iat + c] - RRRc[3 * jat + c];
                    Rcij[c] = Rcij[c] - box[c] * anint(Rcij[c] * boxi[c]);
                }
                double d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                double dij[3];
                if (idip && jdip) {
                    smear3(d2, m.aDD * polfac[isp] * polfac[jsp], &ts1, &ts2, &ts3);
                    double TS[3][3][3];
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++)
                            for (int c = 0; c < 3; c++) {
                                double tt = 0.0;
                                if (b == c) tt = tt + Rs[a];
                                if (a == c) tt = tt + Rs[b];
                                if (a == b) tt = tt + Rs[c];
                                TS[a][b][c] = 15.0 * Rs[a] * Rs[b] * Rs[c] * ts3 - 3.0 * tt * ts2;
                            }
                    double arr33[3][3];
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++)
                            arr33[a][b] = TS[a][b][0] * dj[0] + TS[a][b][1] * dj[1] + TS[a][b][2] * dj[2];
                    for (int c = 0; c < 3; c++) dij[c] = di[0] * arr33[0][c] + di[1] * arr33[1][c] + di[2] * arr33[2][c];
                    for (int c = 0; c < 3; c++) {
                        dR[3 * iat + c] = dR[3 * iat + c] + dij[c];
                        dR[3 * jat + c] = dR[3 * jat + c] - dij[c];
                    }
                    virialc = virialc + (Rcij[0] * dij[0] + Rcij[1] * dij[1] + Rcij[2] * dij[2]);
                    for (int col = 0; col < 3; col++)
                        for (int c = 0; c < 3; c++) virt[c + 3 * col] = virt[c + 3 * col] + dij[c] * Rs[col];
                }
                double qdqd[3];
                for (int c = 0; c < 3; c++) qdqd[c] = qj * di[c] - qi * dj[c];
                self2(d2, &ts1, &ts2);
                double dd3[3][3];
                get_dd3(Rs, ts1, ts2, dd3);
                for (int c = 0; c < 3; c++) dij[c] = dd3[0][c] * qdqd[0] + dd3[1][c] * qdqd[1] + dd3[2][c] * qdqd[2];
                phi[iat] = phi[iat] + ts1 * (Rs[0] * dj[0] + Rs[1] * dj[1] + Rs[2] * dj[2]);
                phi[jat] = phi[jat] - ts1 * (Rs[0] * di[0] + Rs[1] * di[1] + Rs[2] * di[2]);
                for (int c = 0; c < 3; c++) {
                    dR[3 * iat + c] = dR[3 * iat + c] + dij[c];
                    dR[3 * jat + c] = dR[3 * jat + c] - dij[c];
                }
                virialc = virialc + (Rcij[0] * dij[0] + Rcij[1] * dij[1] + Rcij[2] * dij[2]);
                for (int col = 0; col < 3; col++)
                    for (int c = 0; c < 3; c++) virt[c + 3 * col] = virt[c + 3 * col] + dij[c] * Rs[col];
            }
        }
    // 551-553 reciprocal space (dipoles)
    ewald_std_qd();
    for (int i = 0; i < 9; i++) virt[i] = virt[i] + vir_rec[i];
    virialc = virialc + vir_rec[0] + vir_rec[4] + vir_rec[8];
    // 556-584 charge-derivative forces
    for (int iw = 0; iw < N; iw++) {
        int iO = iw, iH1 = iw + N, iH2 = iw + 2 * N, iM = iw + 3 * N;
        const double *g = &grdq[27 * iw];
        double dgrad[3][3];  // dgrad(c, k) -> dgrad[k][c]
        for (int c = 0; c < 3; c++) {
            dgrad[1][c] = g[9 * 0 + 0 + c] * phi[iH1] + g[9 * 0 + 3 + c] * phi[iH2] + g[9 * 0 + 6 + c] * phi[iM];
            dgrad[2][c] = g[9 * 1 + 0 + c] * phi[iH1] + g[9 * 1 + 3 + c] * phi[iH2] + g[9 * 1 + 6 + c] * phi[iM];
            dgrad[0][c] = g[9 * 2 + 0 + c] * phi[iH1] + g[9 * 2 + 3 + c] * phi[iH2] + g[9 * 2 + 6 + c] * phi[iM];
        }
        for (int c = 0; c < 3; c++) {
            dR[3 * iH1 + c] = dR[3 * iH1 + c] + dgrad[1][c];
            dR[3 * iH2 + c] = dR[3 * iH2 + c] + dgrad[2][c];
            dR[3 * iO + c] = dR[3 * iO + c] + dgrad[0][c];
        }
        double roh1[3], roh2[3];
        for (int c = 0; c < 3; c++) {
            roh1[c] = R[3 * iH1 + c] - R[3 * iO + c];
            roh1[c] = roh1[c] - box[c] * anint(roh1[c] * boxi[c]);
            roh2[c] = R[3 * iH2 + c] - R[3 * iO + c];
            roh2[c] = roh2[c] - box[c] * anint(roh2[c] * boxi[c]);
        }
        for (int ix = 0; ix < 3; ix++)
            for (int iy = 0; iy < 3; iy++)
                virt[ix + 3 * iy] = virt[ix + 3 * iy] + roh1[ix] * dgrad[1][iy] + roh2[ix] * dgrad[2][iy];
        for (int c = 0; c < 3; c++) {
            roh1[c] = RRRc[3 * iH1 + c] - RRRc[3 * iO + c];
            roh1[c] = roh1[c] - box[c] * anint(roh1[c] * boxi[c]);
            roh2[c] = RRRc[3 * iH2 + c] - RRRc[3 * iO + c];
            roh2[c] = roh2[c] - box[c] * anint(roh2[c] * boxi[c]);
        }
        for (int c = 0; c < 3; c++) virialc = virialc + roh1[c] * dgrad[1][c] + roh2[c] * dgrad[2][c];
    }
    // 588-591 long-range correction
    virt[0] = virt[0] - Uvdw_lrc;
    virt[4] = virt[4] - Uvdw_lrc;
    virt[8] = virt[8] - Uvdw_lrc;
    virialc = virialc - 3 * Uvdw_lrc;
    // 597-602 M-site force redistribution
    for (int iw = 0; iw < N; iw++) {
        int iO = iw, iH1 = iw + N, iH2 = iw + 2 * N, iM = iw + 3 * N;
        for (int c = 0; c < 3; c++) {
            dRR[3 * (3 * iw + 1) + c] = dR[3 * iH1 + c] + 0.5 * gammaM * dR[3 * iM + c];
            dRR[3 * (3 * iw + 2) + c] = dR[3 * iH2 + c] + 0.5 * gammaM * dR[3 * iM + c];
            dRR[3 * (3 * iw + 0) + c] = dR[3 * iO + c] + (1.0 - gammaM) * dR[3 * iM + c];
        }
    }
    // 605-627 dipole outputs
    for (int iw = 0; iw < N; iw++) {
        int iO = iw, iH1 = iw + N, iH2 = iw + 2 * N, iM = iw + 3 * N;
        double rh1m[3], rh2m[3];
        for (int c = 0; c < 3; c++) {
            rh1m[c] = R[3 * iH1 + c] - R[3 * iM + c];
            rh1m[c] = rh1m[c] - box[c] * anint(rh1m[c] * boxi[c]);
            rh2m[c] = R[3 * iH2 + c] - R[3 * iM + c];
            rh2m[c] = rh2m[c] - box[c] * anint(rh2m[c] * boxi[c]);
        }
        (void)iO;
        for (int c = 0; c < 3; c++) dip_momI[3 * iw + c] = charge[iH1] * rh1m[c] + charge[iH2] * rh2m[c];
        for (int isp = fdI; isp <= ldI; isp++) {
            int iat = iw + (isp - 1) * N;
            for (int c = 0; c < 3; c++) {
                dip_momI[3 * iw + c] = dip[3 * iat + c] + dip_momI[3 * iw + c];
                Edip_mom[3 * iw + c] = dip[3 * iat + c];
            }
        }
    }
    *En = Umon + Uvdw + Uelec + Uind + Uvdw_lrc;
    *virialc_out = virialc;
}

// pot_spc.f90:1-277 (q-SPC/Fw, pot_model 4; SPC/F, pot_model 5)
void Orc::pot_spc(const double *RR, double *En, double *dRR, double *virt, double *dip_momI, double *chg) {
    for (int i = 0; i < 9; i++) {
        virt[i] = 0.0;
        vir_rec[i] = 0.0;
    }
    Umon = Uvdw = Uelec = 0.0;
    Uind = 0.0;
    std::fill(phi.begin(), phi.end(), 0.0);
    std::fill(Efq.begin(), Efq.end(), 0.0);
    std::fill(dR.begin(), dR.end(), 0.0);
    for (int iw = 0; iw < N; iw++) {
        int ia[3] = {3 * iw, 3 * iw + 1, 3 * iw + 2};
        int is[3] = {iw, iw + N, iw + 2 * N};
        for (int k = 0; k < 3; k++) {
            for (int c = 0; c < 3; c++) R[3 * is[k] + c] = RR[3 * ia[k] + c];
            chg[ia[k]] = charge[is[k]];
        }
    }
    if (p.pot_model == 4) {
        for (int iw = 0; iw < N; iw++) {
            int sidx[3] = {iw, iw + N, iw + 2 * N};
            double r1[3][3];
            for (int k = 0; k < 3; k++)
                for (int c = 0; c < 3; c++) r1[k][c] = R[3 * sidx[k] + c];
            double ROH1[3], ROH2[3];
            for (int c = 0; c < 3; c++) {
                ROH1[c] = r1[1][c] - r1[0][c];
                ROH1[c] = ROH1[c] - box[c] * anint(ROH1[c] / box[c]);
            }
            double dROH1 = std::sqrt(ROH1[0] * ROH1[0] + ROH1[1] * ROH1[1] + ROH1[2] * ROH1[2]);
            for (int c = 0; c < 3; c++) {
                ROH2[c] = r1[2][c] - r1[0][c];
                ROH2[c] = ROH2[c] - box[c] * anint(ROH2[c] / box[c]);
            }
            double dROH2 = std::sqrt(ROH2[0] * ROH2[0] + ROH2[1] * ROH2[1] + ROH2[2] * ROH2[2]);
            double AxB[3];
            AxB[0] = ROH1[1] * ROH2[2] - ROH1[2] * ROH2[1];
            AxB[1] = -ROH1[0] * ROH2[2] + ROH1[2] * ROH2[0];
            AxB[2] = ROH1[0] * ROH2[1] - ROH1[1] * ROH2[0];
            double dAxB = std::sqrt(AxB[0] * AxB[0] + AxB[1] * AxB[1] + AxB[2] * AxB[2]);
            double costh = (ROH1[0] * ROH2[0] + ROH1[1] * ROH2[1] + ROH1[2] * ROH2[2]) / (dROH1 * dROH2);
            double sinth = dAxB / (dROH1 * dROH2);
            double ang = std::atan2(sinth, costh);
            double e1 = harmkb * ((dROH1 - roh0) * (dROH1 - roh0) + (dROH2 - roh0) * (dROH2 - roh0)) +
                        harmka * ((ang - th0) * (ang - th0));
            double tmp1 = 2.0 * harmkb * (dROH1 - roh0) / dROH1;
            double tmp2 = 2.0 * harmkb * (dROH2 - roh0) / dROH2;
            double tmp = 2.0 * harmka * (ang - th0);
            double A1[3], A2[3], dh1[3], dh2[3];
            for (int c = 0; c < 3; c++) {
                A1[c] = -(ROH2[c] / (dROH1 * dROH2) - costh * ROH1[c] / (dROH1 * dROH1)) / sinth;
                A2[c] = -(ROH1[c] / (dROH1 * dROH2) - costh * ROH2[c] / (dROH2 * dROH2)) / sinth;
                dh1[c] = tmp1 * ROH1[c] + tmp * A1[c];
                dh2[c] = tmp2 * ROH2[c] + tmp * A2[c];
            }
            Umon = Umon + e1;
            for (int c = 0; c < 3; c++) {
                dR[3 * sidx[1] + c] = dh1[c];
                dR[3 * sidx[2] + c] = dh2[c];
                dR[3 * sidx[0] + c] = -dh1[c] - dh2[c];
            }
            for (int iy = 0; iy < 3; iy++)
                for (int c = 0; c < 3; c++)
                    virt[c + 3 * iy] = virt[c + 3 * iy] + ROH1[c] * dh1[iy] + ROH2[c] * dh2[iy];
        }
    } else {
        // SPC/F (pot_spc.f90:107-137)
        const double Ap = 671.288262912, Bp = 164.376, Cp = -211.536, Dp = 111.744;
        double rhh0 = 2.0 * std::sin(0.5 * th0) * roh0;
        for (int iw = 0; iw < N; iw++) {
            int sidx[3] = {iw, iw + N, iw + 2 * N};
            double r1[3][3];
            for (int k = 0; k < 3; k++)
                for (int c = 0; c < 3; c++) r1[k][c] = R[3 * sidx[k] + c];
            double ROH1[3], ROH2[3], RHH[3];
            for (int c = 0; c < 3; c++) {
                ROH1[c] = r1[0][c] - r1[1][c];
                ROH1[c] = ROH1[c] - box[c] * anint(ROH1[c] / box[c]);
                ROH2[c] = r1[0][c] - r1[2][c];
                ROH2[c] = ROH2[c] - box[c] * anint(ROH2[c] / box[c]);
                RHH[c] = r1[1][c] - r1[2][c];
                RHH[c] = RHH[c] - box[c] * anint(RHH[c] / box[c]);
            }
            double dROH1 = std::sqrt(ROH1[0] * ROH1[0] + ROH1[1] * ROH1[1] + ROH1[2] * ROH1[2]);
            double dROH2 = std::sqrt(ROH2[0] * ROH2[0] + ROH2[1] * ROH2[1] + ROH2[2] * ROH2[2]);
            double dRHH = std::sqrt(RHH[0] * RHH[0] + RHH[1] * RHH[1] + RHH[2] * RHH[2]);
            double dd1 = dROH1 - roh0, dd2 = dROH2 - roh0, dd3 = dRHH - rhh0;
            double e1 = Ap * (dd1 * dd1 + dd2 * dd2) + Bp * dd3 * dd3 + Cp * (dd1 + dd2) * dd3 + Dp * dd1 * dd2;
            double dVdd1 = 2.0 * Ap * dd1 + Cp * dd3 + Dp * dd2;
            double dVdd2 = 2.0 * Ap * dd2 + Cp * dd3 + Dp * dd1;
            double dVdd3 = 2.0 * Bp * dd3 + Cp * (dd1 + dd2);
            double dr1[3][3];
            for (int c = 0; c < 3; c++) {
                dr1[0][c] = dVdd1 * ROH1[c] / dROH1 + dVdd2 * ROH2[c] / dROH2;
                dr1[1][c] = -dVdd1 * ROH1[c] / dROH1 + dVdd3 * RHH[c] / dRHH;
                dr1[2][c] = -dVdd2 * ROH2[c] / dROH2 - dVdd3 * RHH[c] / dRHH;
            }
            Umon = Umon + e1;
            for (int k = 0; k < 3; k++)
                for (int c = 0; c < 3; c++) dR[3 * sidx[k] + c] = dr1[k][c];
            for (int iy = 0; iy < 3; iy++)
                for (int c = 0; c < 3; c++)
                    virt[c + 3 * iy] = virt[c + 3 * iy] - ROH1[c] * dr1[1][iy] - ROH2[c] * dr1[2][iy];
        }
    }
    // 142-191 real-space vdW + electrostatics
    std::vector<int> nj;
    std::vector<double> nR, nR2;
    for (int i = 0; i < N; i++) {
        int iO = i;
        find_neigh(iO, nj, nR, nR2);
        for (size_t j = 0; j < nj.size(); j++) {
            int jO = nj[j];
            double Rij[3] = {nR[3 * j], nR[3 * j + 1], nR[3 * j + 2]};
            double dRsq = nR2[j];
            double R2i = 1.0 / dRsq, R6i = R2i * R2i * R2i, R8i = R6i * R2i;
            double uij = R6i * (m.vdwA * R6i + m.vdwC);
            double sc = R8i * (12.0 * m.vdwA * R6i + 6.0 * m.vdwC);
            double dij[3];
            for (int c = 0; c < 3; c++) dij[c] = -sc * Rij[c];
            Uvdw = Uvdw + uij;
            for (int c = 0; c < 3; c++) {
                dR[3 * iO + c] = dR[3 * iO + c] + dij[c];
                dR[3 * jO + c] = dR[3 * jO + c] - dij[c];
            }
            for (int col = 0; col < 3; col++)
                for (int c = 0; c < 3; c++) virt[c + 3 * col] = virt[c + 3 * col] + dij[col] * Rij[c];
            double Rij0[3];
            for (int c = 0; c < 3; c++) Rij0[c] = Rij[c] - R[3 * iO + c] + R[3 * jO + c];
            for (int isp = 1; isp <= 3; isp++) {
                int iat = iO + (isp - 1) * N;
                double Ri[3];
                for (int c = 0; c < 3; c++) Ri[c] = R[3 * iat + c] + Rij0[c];
                double qi = charge[iat];
                for (int jsp = 1; jsp <= 3; jsp++) {
                    int jat = jO + (jsp - 1) * N;
                    double qj = charge[jat];
                    double Rs[3];
                    for (int c = 0; c < 3; c++) {
                        Rs[c] = Ri[c] - R[3 * jat + c];
                        Rs[c] = Rs[c] - box[c] * anint(Rs[c] * boxi[c]);
                    }
                    double drsq = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                    double dd = std::sqrt(drsq);
                    double expon = std::exp(-(aewald * aewald * drsq));
                    double ts0 = erfc_as(aewald * dd) / dd;
                    double ts1 = (ts0 + const_ts1 * expon) / drsq;
                    phi[iat] = phi[iat] + ts0 * qj;
                    phi[jat] = phi[jat] + ts0 * qi;
                    double d[3];
                    for (int c = 0; c < 3; c++) {
                        Efq[3 * iat + c] = Efq[3 * iat + c] + ts1 * qj * Rs[c];
                        Efq[3 * jat + c] = Efq[3 * jat + c] - ts1 * qi * Rs[c];
                        d[c] = -ts1 * qi * qj * Rs[c];
                    }
                    for (int col = 0; col < 3; col++)
                        for (int c = 0; c < 3; c++) virt[c + 3 * col] = virt[c + 3 * col] + d[col] * Rs[c];
                }
            }
        }
    }
    // 201-233 self energy
    for (int iat = 0; iat < 3 * N; iat++) phi[iat] = phi[iat] - aewald * TSP * charge[iat];
    for (int iw = 0; iw < N; iw++)
        for (int isp = 1; isp <= 2; isp++) {
            int iat = iw + (isp - 1) * N;
            for (int jsp = isp + 1; jsp <= 3; jsp++) {
                int jat = iw + (jsp - 1) * N;
                double Rs[3];
                for (int c = 0; c < 3; c++) {
                    Rs[c] = (R[3 * iat + c] - R[3 * jat + c]);
                    Rs[c] = Rs[c] - box[c] * anint(Rs[c] / box[c]);
                }
                double drsq = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                double dd = std::sqrt(drsq);
                double expon = std::exp(-(aewald * aewald * drsq));
                double kr0 = (erfc_as(aewald * dd)) / dd;
                double kr1 = (kr0 + const_ts1 * expon) / drsq;
                double ch0 = -1.0 / dd;
                double ch1 = ch0 / drsq;
                double ts0 = ch0 + kr0;
                double ts1 = ch1 + kr1;
                phi[iat] = phi[iat] + ts0 * charge[jat];
                phi[jat] = phi[jat] + ts0 * charge[iat];
                double d[3];
                for (int c = 0; c < 3; c++) {
                    Efq[3 * iat + c] = Efq[3 * iat + c] + ts1 * charge[jat] * Rs[c];
                    Efq[3 * jat + c] = Efq[3 * jat + c] - ts1 * charge[iat] * Rs[c];
                    d[c] = -ts1 * charge[iat] * charge[jat] * Rs[c];
                }
                for (int col = 0; col < 3; col++)
                    for (int c = 0; c < 3; c++) virt[c + 3 * col] = virt[c + 3 * col] + d[col] * Rs[c];
            }
        }
    ewald_pw_std_qq();
    for (int i = 0; i < 9; i++) virt[i] = virt[i] + vir_rec[i];
    {
        double s = 0;
        for (int iat = 0; iat < 3 * N; iat++) s += charge[iat] * phi[iat];
        Uelec = 0.5 * s;
    }
    for (int iat = 0; iat < 3 * N; iat++)
        for (int c = 0; c < 3; c++) dR[3 * iat + c] = dR[3 * iat + c] - charge[iat] * Efq[3 * iat + c];
    virt[0] = virt[0] - Uvdw_lrc;
    virt[4] = virt[4] - Uvdw_lrc;
    virt[8] = virt[8] - Uvdw_lrc;
    for (int iw = 0; iw < N; iw++) {
        int iO = iw, iH1 = iw + N, iH2 = iw + 2 * N;
        double rh1O[3], rh2O[3];
        for (int c = 0; c < 3; c++) {
            rh1O[c] = R[3 * iH1 + c] - R[3 * iO + c];
            rh1O[c] = rh1O[c] - box[c] * anint(rh1O[c] / box[c]);
            rh2O[c] = R[3 * iH2 + c] - R[3 * iO + c];
            rh2O[c] = rh2O[c] - box[c] * anint(rh2O[c] / box[c]);
        }
        for (int c = 0; c < 3; c++) dip_momI[3 * iw + c] = charge[iH1] * rh1O[c] + charge[iH2] * rh2O[c];
    }
    *En = Umon + Uvdw + Uelec + Uvdw_lrc;
    for (int iw = 0; iw < N; iw++) {
        int is[3] = {iw, iw + N, iw + 2 * N};
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++) dRR[3 * (3 * iw + k) + c] = dR[3 * is[k] + c];
    }
}

}  // namespace

extern "C" {

void *orc_create(const orc_params *p) { return new Orc(p); }
void orc_destroy(void *h) { delete static_cast<Orc *>(h); }

void orc_ewald_info(void *h, double *alpha, int *nk, int *hkl_max) {
    Orc *o = static_cast<Orc *>(h);
    *alpha = o->aewald;
    *nk = o->nkvec;
    hkl_max[0] = o->hmax;
    hkl_max[1] = o->kmax;
    hkl_max[2] = o->lmax;
}

void orc_kvectors(void *h, int *k_hkl, double *kvec, double *Ak) {
    Orc *o = static_cast<Orc *>(h);
    std::copy(o->k_hkl.begin(), o->k_hkl.end(), k_hkl);
    std::copy(o->kvec.begin(), o->kvec.end(), kvec);
    std::copy(o->Ak.begin(), o->Ak.end(), Ak);
}

void orc_pot_ttm(void *h, int bead, const double *RR, const double *RRc, double *En, double *dRR,
                 double *virt, double *virialc, double *dip_momI, double *Edip_mom, double *chg, int t) {
    static_cast<Orc *>(h)->pot_ttm(bead, RR, RRc, En, dRR, virt, virialc, dip_momI, Edip_mom, chg, t);
}

void orc_pot_spc(void *h, const double *RR, double *En, double *dRR, double *virt, double *dip_momI,
                 double *chg) {
    static_cast<Orc *>(h)->pot_spc(RR, En, dRR, virt, dip_momI, chg);
}

// find_neigh.f90:14-120 for every molecule: (i, j) pairs in the reference's order
int orc_neighbors(void *h, const double *RR, int *ij, int cap) {
    Orc *o = static_cast<Orc *>(h);
    for (int iw = 0; iw < o->N; iw++)
        for (int c = 0; c < 3; c++) o->R[3 * iw + c] = RR[3 * (3 * iw) + c];
    std::vector<int> nj;
    std::vector<double> nR, nR2;
    int n = 0;
    for (int i = 0; i < o->N; i++) {
        o->find_neigh(i, nj, nR, nR2);
        for (int j : nj) {
            if (n < cap) {
                ij[2 * n] = i;
                ij[2 * n + 1] = j;
            }
            n++;
        }
    }
    return n;
}

void orc_energies(void *h, double *U4, int *niter, double *last_deltadip) {
    Orc *o = static_cast<Orc *>(h);
    U4[0] = o->Umon;
    U4[1] = o->Uvdw;
    U4[2] = o->Uelec;
    U4[3] = o->Uind;
    *niter = o->niter;
    *last_deltadip = o->deltadip_last;
}

// force_calc.f90:26-106: beads distributed over worker threads as MPI ranks would take them
void orc_full_bead_forces(const orc_params *p, int nthreads, const double *RRt, const double *RRc,
                          double *Upott, double *dRRt, double *virialt, double *virialct,
                          double *dip_momIt, double *dip_momEt, double *chg, int t) {
    int P = p->nbeads, na = p->natoms, nw = na / 3;
    nthreads = std::max(1, std::min(nthreads, P));
    std::vector<std::thread> th;
    std::vector<std::vector<double>> chgs(nthreads, std::vector<double>(na));
    for (int w = 0; w < nthreads; w++) {
        th.emplace_back([=, &chgs]() {
            Orc o(p);
            for (int k = w; k < P; k += nthreads) {
                double virt[9];
                double *dipI = dip_momIt + (size_t)3 * nw * k, *dipE = dip_momEt + (size_t)3 * nw * k;
                if (p->pot_model == 2 || p->pot_model == 3) {
                    o.pot_ttm(k, RRt + (size_t)3 * na * k, RRc, &Upott[k], dRRt + (size_t)3 * na * k, virt,
                              &virialct[k], dipI, dipE, chgs[w].data(), t);
                } else {
                    o.pot_spc(RRt + (size_t)3 * na * k, &Upott[k], dRRt + (size_t)3 * na * k, virt, dipI,
                              chgs[w].data());
                    virialct[k] = 0.0;  // pot_spc leaves virialc undefined (reference quirk)
                    for (int i = 0; i < 3 * nw; i++) dipE[i] = 0.0;
                }
                virialt[k] = virt[0] + virt[4] + virt[8];
                if (k == P - 1) std::copy(chgs[w].begin(), chgs[w].end(), chg);
            }
        });
    }
    for (auto &x : th) x.join();
}

// A persistent pool of oracle states, one per worker thread, bead k always on thread
// k % nthreads, so each bead's predictor history lives across calls like an MPI rank's.
struct OrcPool {
    orc_params p;
    int nthreads;
    std::vector<Orc *> w;
};

void *orc_pool_create(const orc_params *p, int nthreads) {
    OrcPool *pool = new OrcPool();
    pool->p = *p;
    pool->nthreads = std::max(1, std::min(nthreads, p->nbeads));
    for (int i = 0; i < pool->nthreads; i++) pool->w.push_back(new Orc(p));
    return pool;
}

void orc_pool_destroy(void *h) {
    OrcPool *pool = static_cast<OrcPool *>(h);
    for (Orc *o : pool->w) delete o;
    delete pool;
}

void orc_pool_forces(void *h, const double *RRt, const double *RRc, double *Upott, double *dRRt, double *virialt,
                     double *virialct, int t) {
    OrcPool *pool = static_cast<OrcPool *>(h);
    const int P = pool->p.nbeads, na = pool->p.natoms, nw = na / 3;
    std::vector<std::thread> th;
    for (int w = 0; w < pool->nthreads; w++) {
        th.emplace_back([=]() {
            Orc &o = *pool->w[w];
            std::vector<double> dI(3 * nw), dE(3 * nw), chg(na);
            for (int k = w; k < P; k += pool->nthreads) {
                double virt[9];
                if (o.polar)
                    o.pot_ttm(k, RRt + (size_t)3 * na * k, RRc, &Upott[k], dRRt + (size_t)3 * na * k, virt, &virialct[k],
                              dI.data(), dE.data(), chg.data(), t);
                else {
                    o.pot_spc(RRt + (size_t)3 * na * k, &Upott[k], dRRt + (size_t)3 * na * k, virt, dI.data(), chg.data());
                    virialct[k] = 0.0;
                }
                virialt[k] = virt[0] + virt[4] + virt[8];
            }
        });
    }
    for (auto &x : th) x.join();
}

// NormalModes.f90:68-218
void orc_nm_init(int P, double omegan, double delta, double setNMfreq, double *A11, double *A12,
                 double *A21, double *A22, double *omegalist, double *msf, double *C) {
    int l = (P % 2 == 0) ? (P - 2) / 2 : (P - 1) / 2;
    // C(row, col) -> C[(row-1) + P*(col-1)]
    for (int i = 1; i <= P; i++) {
        C[0 + P * (i - 1)] = std::sqrt(1.0 / P);
        for (int k = 1; k <= l; k++) {
            C[k + P * (i - 1)] = std::sqrt(2.0 / P) * std::cos((double)(k * i) * 2.0 * PI / P);
            C[k + l + P * (i - 1)] = std::sqrt(2.0 / P) * std::sin((double)(k * i) * 2.0 * PI / P);
        }
        if (P % 2 == 0) C[2 * l + 1 + P * (i - 1)] = std::sqrt(1.0 / P) * ((i % 2 == 0) ? 1.0 : -1.0);
    }
    omegalist[0] = 0.0;
    A11[0] = 1.0;
    A12[0] = delta;
    A21[0] = 0.0;
    A22[0] = 1.0;
    auto set_mode = [&](int idx, int k) {
        // NormalModes.f90:126: abs(k)/real(Nbeads) is evaluated in single precision
        float ratio = (float)std::abs(k) / (float)P;
        double omega = 2 * omegan * std::sin(PI * (double)ratio);
        omegalist[idx] = omega;
        A11[idx] = std::cos(omega * delta);
        A12[idx] = (1.0 / omega) * std::sin(omega * delta);
        A21[idx] = -omega * std::sin(omega * delta);
        A22[idx] = std::cos(omega * delta);
    };
    for (int k = 1; k <= l; k++) set_mode(k, k);
    for (int k = 1; k <= l; k++) set_mode(k + l, k);
    if (P % 2 == 0) set_mode(2 * l + 1, l + 1);
    for (int i = 0; i < P; i++) msf[i] = 1.0;
    if (setNMfreq != 0) {
        omegalist[0] = 0.0;
        A11[0] = 1.0;
        A12[0] = delta;
        A21[0] = 0.0;
        A22[0] = 1.0;
        double omega = (2 * PI) * setNMfreq / 33.33333;
        for (int i = 0; i < P; i++) msf[i] = (omegalist[i] == 0) ? 1.0 : (omegalist[i] / omega) * (omegalist[i] / omega);
        int hi = (P % 2 == 0) ? 2 * l + 1 : 2 * l;
        for (int i = 1; i <= hi; i++) {
            omegalist[i] = omega;
            A11[i] = std::cos(omega * delta);
            A12[i] = (1.0 / omega) * std::sin(omega * delta);
            A21[i] = -omega * std::sin(omega * delta);
            A22[i] = std::cos(omega * delta);
        }
    }
}

static void real2NM(int P, const double *C, const double *A, double *out) {
    for (int i = 0; i < 3 * P; i++) out[i] = 0.0;
    for (int j = 0; j < P; j++)
        for (int k = 0; k < P; k++)
            for (int c = 0; c < 3; c++) out[3 * j + c] = out[3 * j + c] + C[j + P * k] * A[3 * k + c];
}

static void NM2real(int P, const double *C, const double *A, double *out) {
    for (int i = 0; i < 3 * P; i++) out[i] = 0.0;
    for (int j = 0; j < P; j++)
        for (int k = 0; k < P; k++)
            for (int c = 0; c < 3; c++) out[3 * j + c] = out[3 * j + c] + C[k + P * j] * A[3 * k + c];
}

// NormalModes.f90:308-341 real2NM / NM2real for one atom
void orc_real2nm(int P, const double *C, const double *A, double *out) { real2NM(P, C, A, out); }
void orc_nm2real(int P, const double *C, const double *A, double *out) { NM2real(P, C, A, out); }

// NormalModes.f90:224-250 gen_rand_ring, rand_norm(std_dev) = std_dev * xi with xi(3,P) supplied
void orc_gen_rand_ring(int P, const double *C, const double *omegalist, const double *msf, double mass, double temp,
                       const double *xi, double *RR) {
    const double hbar = 6.35077993041;
    const double omegan = KB_AMU * temp * P / hbar;
    std::vector<double> tr(3 * P, 0.0);
    for (int j = 0; j < P; j++) {
        const double omega = omegalist[j];
        if (omega == 0.0) continue;
        const double sd = std::sqrt((omegan * hbar) / (mass * msf[j] * (omega * omega)));
        for (int c = 0; c < 3; c++) tr[3 * j + c] = sd * xi[3 * j + c];
    }
    NM2real(P, C, tr.data(), RR);
}

// NormalModes.f90:257-275 gen_rand_ring_momenta
void orc_gen_rand_ring_momenta(int P, const double *C, const double *msf, double mass, double temp, const double *xi,
                               double *PP) {
    std::vector<double> tr(3 * P);
    for (int j = 0; j < P; j++) {
        const double sd = std::sqrt(KB_AMU * mass * msf[j] * temp);
        for (int c = 0; c < 3; c++) tr[3 * j + c] = sd * xi[3 * j + c];
    }
    NM2real(P, C, tr.data(), PP);
}

// NormalModes.f90:34-63
void orc_evolve_ring(int P, const double *A11, const double *A12, const double *A21, const double *A22,
                     const double *msf, const double *C, double *RR, double *PP, double mass) {
    std::vector<double> RRtr(3 * P), PPtr(3 * P);
    real2NM(P, C, RR, RRtr.data());
    real2NM(P, C, PP, PPtr.data());
    for (int j = 0; j < P; j++) {
        double temp2[3];
        for (int c = 0; c < 3; c++) temp2[c] = A11[j] * RRtr[3 * j + c] + A12[j] * PPtr[3 * j + c] / (mass * msf[j]);
        for (int c = 0; c < 3; c++) PPtr[3 * j + c] = A21[j] * mass * msf[j] * RRtr[3 * j + c] + A22[j] * PPtr[3 * j + c];
        for (int c = 0; c < 3; c++) RRtr[3 * j + c] = temp2[c];
    }
    NM2real(P, C, RRtr.data(), RR);
    NM2real(P, C, PPtr.data(), PP);
}

// Langevin.f90:68-98
void orc_langevin_init(int P, const double *omegalist, double delt2, int centroid_thermostat,
                       double tau_centroid, double temp_P, double *c1, double *c2) {
    for (int i = 0; i < P; i++) {
        double gammak;
        if (i == 0)
            gammak = centroid_thermostat ? 1.0 / tau_centroid : 0.0;
        else
            gammak = 2 * omegalist[i];
        c1[i] = std::exp(-delt2 * gammak);
        c2[i] = std::sqrt(1 - c1[i] * c1[i]);
        c2[i] = std::sqrt(KB_AMU * temp_P) * c2[i];
    }
}

// Langevin.f90:30-64; rand_norm(sqrtmass) = sqrtmass * xi with xi(3,P,Natoms) supplied
void orc_langevin_nm(int P, int natoms, const double *C, const double *msf, const double *c1,
                     const double *c2, double massO, double massH, double *PPt, const double *xi) {
    std::vector<double> in(3 * P), tr(3 * P), out(3 * P);
    for (int i2 = 0; i2 < natoms; i2++) {
        for (int j = 0; j < P; j++)
            for (int c = 0; c < 3; c++) in[3 * j + c] = PPt[3 * i2 + c + (size_t)3 * natoms * j];
        real2NM(P, C, in.data(), tr.data());
        for (int j = 0; j < P; j++) {
            double sqrtmass = ((i2 + 1 + 2) % 3 == 0) ? std::sqrt(massO * msf[j]) : std::sqrt(massH * msf[j]);
            for (int k = 0; k < 3; k++)
                tr[3 * j + k] = c1[j] * tr[3 * j + k] + c2[j] * (sqrtmass * xi[k + 3 * j + (size_t)3 * P * i2]);
        }
        NM2real(P, C, tr.data(), out.data());
        for (int j = 0; j < P; j++)
            for (int c = 0; c < 3; c++) PPt[3 * i2 + c + (size_t)3 * natoms * j] = out[3 * j + c];
    }
}

// main_stuff.f90:349-388
double orc_calc_uk(int P, int natoms, double massO, double massH, const double *PPt, double setNMfreq,
                   const double *C, const double *msf) {
    double imassO = 1.0 / massO, imassH = 1.0 / massH;
    int nw = natoms / 3;
    double uk = 0;
    if (setNMfreq == 0 || P == 1) {
        for (int j = 0; j < P; j++)
            for (int i = 0; i < nw; i++)
                for (int a = 0; a < 3; a++) {
                    const double *p = &PPt[3 * (3 * i + a) + (size_t)3 * natoms * j];
                    double s = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
                    uk = uk + (a == 0 ? imassO : imassH) * s;
                }
    } else {
        std::vector<double> in(3 * P), tr(3 * P);
        for (int i = 0; i < nw; i++)
            for (int a = 0; a < 3; a++) {
                for (int j = 0; j < P; j++)
                    for (int c = 0; c < 3; c++) in[3 * j + c] = PPt[3 * (3 * i + a) + c + (size_t)3 * natoms * j];
                real2NM(P, C, in.data(), tr.data());
                for (int j = 0; j < P; j++) {
                    double s = tr[3 * j] * tr[3 * j] + tr[3 * j + 1] * tr[3 * j + 1] + tr[3 * j + 2] * tr[3 * j + 2];
                    uk = uk + (a == 0 ? imassO : imassH) * s / msf[j];
                }
            }
    }
    return 0.5 * uk;
}

// MD.f90:35-110 PIMD_VV (no global Nose-Hoover, no barostat)
void orc_pimd_vv_step(void *h, const orc_md_params *mp, int P, double *RRt, double *PPt, double *dRRt,
                      double *RRc, const double *xi1, const double *xi2, int t, double *Upot,
                      double *virial, double *virialc, double *uk) {
    orc_pimd_vv_step_pool(h, nullptr, mp, P, RRt, PPt, dRRt, RRc, xi1, xi2, t, Upot, virial, virialc, uk);
}

// Nose_Hoover.f90:33-112: one half step (delt2) of a chain-2 Nose-Hoover thermostat on uk, L
// degrees of freedom at temperature temp; returns s, updates vxi[2] and uk (= uk s^2)
void orc_nose_hoover(double *s, double *uk, double *vxi, double tau, double delt2, int L, double temp) {
    const double delt4 = delt2 / 2.0, delt8 = delt2 / 4.0;
    const double kT = KB_AMU * temp;
    const double M1 = (L * kT) * (tau * tau);
    const double M2 = M1;
    vxi[1] = vxi[1] + ((M1 * (vxi[0] * vxi[0]) - kT) * delt4) / M2;
    vxi[0] = vxi[0] * std::exp(-vxi[1] * delt8);
    vxi[0] = vxi[0] + ((2 * *uk - L * kT) * delt4) / M1;
    vxi[0] = vxi[0] * std::exp(-vxi[1] * delt8);
    *s = std::exp(-vxi[0] * delt2);
    *uk = (*uk * *s) * *s;
    vxi[0] = vxi[0] * std::exp(-vxi[1] * delt8);
    vxi[0] = vxi[0] + ((2 * *uk - L * kT) * delt4) / M1;
    vxi[0] = vxi[0] * std::exp(-vxi[1] * delt8);
    vxi[1] = vxi[1] + ((M1 * (vxi[0] * vxi[0]) - kT) * delt4) / M2;
}

// main_stuff.f90:145-171: bead_thermostat with bead_thermostat_type 'Nose-Hoover', one chain per
// (atom, normal mode, component) in normal-mode space; vxi_beads(2, natoms, P, 3)
void orc_bead_nose_hoover(int P, int natoms, const double *C, const double *omegalist, const double *msf,
                          double massO, double massH, double *PPt, double *vxi_beads, int centroid_thermostat,
                          double tau_centroid, double delt2, double temp) {
    std::vector<double> in(3 * P), tr(3 * P), out(3 * P);
    const double imassO = 1.0 / massO, imassH = 1.0 / massH;
    for (int i = 0; i < natoms; i++) {
        const double imass = (i % 3 == 0) ? imassO : imassH;
        for (int j = 0; j < P; j++)
            for (int c = 0; c < 3; c++) in[3 * j + c] = PPt[3 * i + c + (size_t)3 * natoms * j];
        real2NM(P, C, in.data(), tr.data());
        auto vxi = [&](int j, int k) { return vxi_beads + 2 * ((size_t)i + (size_t)natoms * ((size_t)j + (size_t)P * k)); };
        if (centroid_thermostat) {
            for (int k = 0; k < 3; k++) {
                double sbead, ukb = (0.5 * imass) * (tr[k] * tr[k]);
                orc_nose_hoover(&sbead, &ukb, vxi(0, k), tau_centroid, delt2, 1, P * temp);
                tr[k] = tr[k] * sbead;
            }
        }
        for (int j = 1; j < P; j++) {
            const double tau = 1.0 / omegalist[j];
            for (int k = 0; k < 3; k++) {
                double sbead, ukb = ((0.5 * imass) * (tr[3 * j + k] * tr[3 * j + k])) / msf[j];
                orc_nose_hoover(&sbead, &ukb, vxi(j, k), tau, delt2, 1, P * temp);
                tr[3 * j + k] = tr[3 * j + k] * sbead;
            }
        }
        NM2real(P, C, tr.data(), out.data());
        for (int j = 0; j < P; j++)
            for (int c = 0; c < 3; c++) PPt[3 * i + c + (size_t)3 * natoms * j] = out[3 * j + c];
    }
}

// estimators.f90:57-73: K0 = sum over beads k, atoms, components of m (r_k - r_(k-1))^2, ring closed
double orc_ring_k0(int P, int natoms, double massO, double massH, const double *RRt) {
    double K0 = 0;
    for (int k = 0; k < P; k++) {
        const int km = (k == 0) ? P - 1 : k - 1;
        for (int j = 0; j < natoms; j++) {
            const double mass = (j % 3 == 0) ? massO : massH;
            for (int i = 0; i < 3; i++) {
                const double d = RRt[i + 3 * (size_t)j + (size_t)3 * natoms * k] - RRt[i + 3 * (size_t)j + (size_t)3 * natoms * km];
                K0 = K0 + mass * (d * d);
            }
        }
    }
    return K0;
}

// write_out's per-step estimators (InputOutput.f90:566-571) from estimators.f90:30-96, with the
// reference's literal types: 1.5*Natoms(*Nbeads) is a default-real product
void orc_estimators(int natoms, int P, double volume, double omegan, double Upot, double virial, double virialc,
                    double uk, double K0raw, double *est5) {
    const double TEMPFACTOR = 0.80181484527, kb = 0.0019872041, PRESSCON2 = 69477.0, MASSCONi = 1.0 / 418.4;
    const int Nwaters = natoms / 3;
    const double sys_temp = TEMPFACTOR * uk / (double)(natoms * P * P);
    double KE = (double)(1.5f * (float)natoms) * kb * sys_temp;
    const double qE = (KE + 0.5 * (virial - virialc) / P + Upot / P) / Nwaters;
    const double qP = PRESSCON2 * (1 / (3 * volume)) * (2 * KE - virialc / P) / Nwaters;
    KE = (double)((1.5f * (float)natoms) * (float)P) * kb * sys_temp * P;
    const double K0 = 0.5 * K0raw * (omegan * omegan) * MASSCONi;
    const double sE = (KE - K0 + Upot) / (double)(Nwaters * P);
    const double sP = PRESSCON2 * (1 / (3 * volume)) * (2 * (KE - K0) - virial) / Nwaters;
    est5[0] = sys_temp;
    est5[1] = qE;
    est5[2] = qP;
    est5[3] = sE;
    est5[4] = sP;
}

// As orc_pimd_vv_step with the force call spread over a thread pool (orc_pool_create).
void orc_pimd_vv_step_pool(void *h, void *pool, const orc_md_params *mp, int P, double *RRt, double *PPt,
                           double *dRRt, double *RRc, const double *xi1, const double *xi2, int t, double *Upot,
                           double *virial, double *virialc, double *uk) {
    double out[ORC_MD_NOUT], vxg[2] = {1.0, 1.0}, ukst = 0.0;
    orc_pimd_vv_step_ex(h, pool, mp, (mp->langevin && xi1) ? 1 : 0, 0, 0.0, P, RRt, PPt, dRRt, RRc, xi1, xi2, vxg,
                        &ukst, nullptr, t, out);
    *Upot = out[0];
    *virial = out[1];
    *virialc = out[2];
    *uk = out[3];
}

// MD.f90:35-110 PIMD_VV with the reference's thermostats: bead_thermostat (main_stuff.f90:132-188,
// Langevin_NM or Nose-Hoover chains on the normal modes) and the global chain THERMOSTAT
// (Nose_Hoover on uk, L = 3 Natoms Nbeads, at temp Nbeads), each at the start and the end of the
// step; write_out's calc_uk after the force call feeds the estimators. out[ORC_MD_NOUT]: Upot,
// virial, virialc, uk (the reference's uk after the step), uk after the force call, K0, then
// sys_temp, virial-estimator energy and pressure, simple-estimator energy and pressure, and the
// step's last global scale factor s. uk_state is the reference's module variable uk across steps.
void orc_pimd_vv_step_ex(void *h, void *pool, const orc_md_params *mp, int bead_thermostat, int global_thermostat,
                         double tau, int P, double *RRt, double *PPt, double *dRRt, double *RRc, const double *xi1,
                         const double *xi2, double *vxi_global, double *uk_state, double *vxi_beads, int t,
                         double *out) {
    Orc *o = static_cast<Orc *>(h);
    int na = o->Natoms, nw = na / 3;
    double delt2 = mp->delt / 2.0;
    double omegan = KB_AMU * mp->temp * P / 6.35077993041;
    std::vector<double> A11(P), A12(P), A21(P), A22(P), om(P), msf(P), C(P * P), c1(P), c2(P);
    orc_nm_init(P, omegan, mp->delt, mp->setNMfreq, A11.data(), A12.data(), A21.data(), A22.data(), om.data(),
                msf.data(), C.data());
    orc_langevin_init(P, om.data(), delt2, mp->centroid_thermostat, mp->tau_centroid, P * mp->temp, c1.data(),
                      c2.data());
    size_t nall = (size_t)3 * na * P;
    auto bead_thermostat_step = [&](const double *xi) {
        if (bead_thermostat == 1 && xi)
            orc_langevin_nm(P, na, C.data(), msf.data(), c1.data(), c2.data(), mp->massO, mp->massH, PPt, xi);
        else if (bead_thermostat == 2)
            orc_bead_nose_hoover(P, na, C.data(), om.data(), msf.data(), mp->massO, mp->massH, PPt, vxi_beads,
                                 mp->centroid_thermostat, mp->tau_centroid, delt2, mp->temp);
    };
    double s = 1.0;
    bead_thermostat_step(xi1);
    if (global_thermostat) {
        orc_nose_hoover(&s, uk_state, vxi_global, tau, delt2, 3 * na * P, mp->temp * P);
        for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] * s;
    }
    for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] - MASSCON * dRRt[i] * delt2;
    if (P > 1) {
        std::vector<double> rr(3 * P), pp(3 * P);
        for (int a = 0; a < na; a++) {
            for (int j = 0; j < P; j++)
                for (int c = 0; c < 3; c++) {
                    rr[3 * j + c] = RRt[3 * a + c + (size_t)3 * na * j];
                    pp[3 * j + c] = PPt[3 * a + c + (size_t)3 * na * j];
                }
            double mass = (a % 3 == 0) ? mp->massO : mp->massH;
            orc_evolve_ring(P, A11.data(), A12.data(), A21.data(), A22.data(), msf.data(), C.data(), rr.data(),
                            pp.data(), mass);
            for (int j = 0; j < P; j++)
                for (int c = 0; c < 3; c++) {
                    RRt[3 * a + c + (size_t)3 * na * j] = rr[3 * j + c];
                    PPt[3 * a + c + (size_t)3 * na * j] = pp[3 * j + c];
                }
        }
    } else {
        double imassO = 1.0 / mp->massO, imassH = 1.0 / mp->massH;
        for (int a = 0; a < na; a++)
            for (int c = 0; c < 3; c++)
                RRt[3 * a + c] = RRt[3 * a + c] + (a % 3 == 0 ? imassO : imassH) * PPt[3 * a + c] * mp->delt;
    }
    // centroid and PBCs (main_stuff.f90:107-125, cubic box assumed by the reference)
    for (int i = 0; i < 3 * na; i++) {
        double sum = 0;
        for (int j = 0; j < P; j++) sum += RRt[i + (size_t)3 * na * j];
        RRc[i] = sum / P;
    }
    for (int i = 0; i < 3 * na; i++) {
        double shift = o->box[0] * anint(RRc[i] * o->boxi[0]);
        RRc[i] = RRc[i] - shift;
        for (int j = 0; j < P; j++) RRt[i + (size_t)3 * na * j] = RRt[i + (size_t)3 * na * j] - shift;
    }
    double U = 0, vir = 0, virc = 0;
    if (pool) {
        std::vector<double> Upott(P), virialt(P), virialct(P);
        orc_pool_forces(pool, RRt, RRc, Upott.data(), dRRt, virialt.data(), virialct.data(), t);
        for (int k = 0; k < P; k++) {
            U += Upott[k];
            vir += virialt[k];
            virc += virialct[k];
        }
    } else {
        std::vector<double> dipI(3 * nw), dipE(3 * nw), chg(na);
        for (int k = 0; k < P; k++) {
            double En, virt[9], vc;
            if (o->polar)
                o->pot_ttm(k, RRt + (size_t)3 * na * k, RRc, &En, dRRt + (size_t)3 * na * k, virt, &vc, dipI.data(),
                           dipE.data(), chg.data(), t);
            else {
                o->pot_spc(RRt + (size_t)3 * na * k, &En, dRRt + (size_t)3 * na * k, virt, dipI.data(), chg.data());
                vc = 0.0;
            }
            U += En;
            vir += virt[0] + virt[4] + virt[8];
            virc += vc;
        }
    }
    out[0] = U;
    out[1] = vir;
    out[2] = virc / P;
    // calc_uk and write_out (MD.f90:86-90)
    out[4] = orc_calc_uk(P, na, mp->massO, mp->massH, PPt, mp->setNMfreq, C.data(), msf.data());
    out[5] = orc_ring_k0(P, na, mp->massO, mp->massH, RRt);
    orc_estimators(na, P, o->box[0] * o->box[1] * o->box[2], omegan, out[0], out[1], out[2], out[4], out[5], out + 6);
    for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] - MASSCON * dRRt[i] * delt2;
    bead_thermostat_step(xi2);
    double ukv = orc_calc_uk(P, na, mp->massO, mp->massH, PPt, mp->setNMfreq, C.data(), msf.data());
    s = 1.0;
    if (global_thermostat) {
        *uk_state = ukv;
        orc_nose_hoover(&s, uk_state, vxi_global, tau, delt2, 3 * na * P, mp->temp * P);
        for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] * s;
        ukv = *uk_state;
    } else {
        *uk_state = ukv;
    }
    out[3] = ukv;
    out[11] = s;
}

// Ring-polymer contraction with multiple time steps (MD.f90:276-449, contracted_MD; mode 0) and
// monomer PIMD (MD.f90:117-265, monomer_PIMD; mode 1): the NASA monomer PES on every bead (fast,
// intra_timesteps inner steps with the normal modes made for deltfast = delt/intra_timesteps in
// mode 0), the intermolecular potential once on the centroid (h: an oracle of one bead with
// contraction set in mode 0 and unset in mode 1, so that monomer_PIMD's centroid call keeps the
// monomer PES as the reference's does). dRRfast (mode 0) persists across steps like the
// reference's saved array. Thermostats and out[12] as orc_pimd_vv_step_ex; dip_momIt/dip_momEt
// (3, Nw, P) from calc_monomer_dip_moments (force_calc.f90:205-264) plus the centroid's induced
// dipoles (may be null).
void orc_contracted_step(void *h, const orc_md_params *mp, int mode, int intra_timesteps, int bead_thermostat,
                         int global_thermostat, double tau, int P, double *RRt, double *PPt, double *dRRt,
                         double *dRRfast, double *RRc, const double *xi1, const double *xi2, double *vxi_global,
                         double *uk_state, double *vxi_beads, int t, double *out, double *dip_momIt,
                         double *dip_momEt) {
    Orc *o = static_cast<Orc *>(h);
    const int na = o->Natoms, nw = na / 3;
    const double delt2 = mp->delt / 2.0;
    const double deltfast = (mode == 0) ? mp->delt / intra_timesteps : mp->delt, delt2fast = deltfast / 2.0;
    const double omegan = KB_AMU * mp->temp * P / 6.35077993041;
    std::vector<double> A11(P), A12(P), A21(P), A22(P), om(P), msf(P), C(P * P), c1(P), c2(P);
    // InputOutput.f90:382-386: the normal-mode propagator of the contracted run is made for deltfast
    orc_nm_init(P, omegan, deltfast, mp->setNMfreq, A11.data(), A12.data(), A21.data(), A22.data(), om.data(),
                msf.data(), C.data());
    orc_langevin_init(P, om.data(), delt2, mp->centroid_thermostat, mp->tau_centroid, P * mp->temp, c1.data(),
                      c2.data());
    const size_t nall = (size_t)3 * na * P;
    auto bead_thermostat_step = [&](const double *xi) {
        if (bead_thermostat == 1 && xi)
            orc_langevin_nm(P, na, C.data(), msf.data(), c1.data(), c2.data(), mp->massO, mp->massH, PPt, xi);
        else if (bead_thermostat == 2)
            orc_bead_nose_hoover(P, na, C.data(), om.data(), msf.data(), mp->massO, mp->massH, PPt, vxi_beads,
                                 mp->centroid_thermostat, mp->tau_centroid, delt2, mp->temp);
    };
    auto centroid_pbc = [&]() {
        for (int i = 0; i < 3 * na; i++) {
            double sum = 0;
            for (int j = 0; j < P; j++) sum += RRt[i + (size_t)3 * na * j];
            RRc[i] = sum / P;
        }
        for (int i = 0; i < 3 * na; i++) {
            const double shift = o->box[0] * anint(RRc[i] * o->boxi[0]);
            RRc[i] = RRc[i] - shift;
            for (int j = 0; j < P; j++) RRt[i + (size_t)3 * na * j] = RRt[i + (size_t)3 * na * j] - shift;
        }
    };
    auto drift = [&](double dt) {
        if (P > 1) {
            std::vector<double> rr(3 * P), pp(3 * P);
            for (int a = 0; a < na; a++) {
                for (int j = 0; j < P; j++)
                    for (int c = 0; c < 3; c++) {
                        rr[3 * j + c] = RRt[3 * a + c + (size_t)3 * na * j];
                        pp[3 * j + c] = PPt[3 * a + c + (size_t)3 * na * j];
                    }
                const double mass = (a % 3 == 0) ? mp->massO : mp->massH;
                orc_evolve_ring(P, A11.data(), A12.data(), A21.data(), A22.data(), msf.data(), C.data(), rr.data(),
                                pp.data(), mass);
                for (int j = 0; j < P; j++)
                    for (int c = 0; c < 3; c++) {
                        RRt[3 * a + c + (size_t)3 * na * j] = rr[3 * j + c];
                        PPt[3 * a + c + (size_t)3 * na * j] = pp[3 * j + c];
                    }
            }
        } else {
            const double imassO = 1.0 / mp->massO, imassH = 1.0 / mp->massH;
            for (int a = 0; a < na; a++)
                for (int c = 0; c < 3; c++)
                    RRt[3 * a + c] = RRt[3 * a + c] + (a % 3 == 0 ? imassO : imassH) * PPt[3 * a + c] * dt;
        }
    };
    // the monomer PES on every bead; with acc, its energies into Upott and the monomer virials
    // (bead and centroid separations, min-imaged) into vir[0], vir[1]
    std::vector<double> Upott(P, 0.0);
    auto monomer = [&](double *g, bool acc, double *vir) {
        for (int j = 0; j < P; j++)
            for (int iw = 0; iw < nw; iw++) {
                const double *rb = RRt + (size_t)3 * na * j + 9 * (size_t)iw;
                double r1[3][3], dr1[3][3], e1;
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) r1[a][c] = rb[3 * a + c];
                o->pot_nasa(r1, dr1, &e1);
                double *gb = g + (size_t)3 * na * j + 9 * (size_t)iw;
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) gb[3 * a + c] = dr1[a][c];
                if (!acc) continue;
                Upott[j] = Upott[j] + e1;
                for (int w = 0; w < 2; w++) {  // w 1: the centroid's separations, w 0: the bead's
                    const double *rr = w ? RRc + 9 * (size_t)iw : rb;
                    double roh1[3], roh2[3];
                    for (int c = 0; c < 3; c++) {
                        roh1[c] = rr[3 + c] - rr[c];
                        roh1[c] = roh1[c] - o->box[c] * anint(roh1[c] * o->boxi[c]);
                        roh2[c] = rr[6 + c] - rr[c];
                        roh2[c] = roh2[c] - o->box[c] * anint(roh2[c] * o->boxi[c]);
                    }
                    vir[w] = vir[w] + (roh1[0] * dr1[1][0] + roh1[1] * dr1[1][1] + roh1[2] * dr1[1][2]);
                    vir[w] = vir[w] + (roh2[0] * dr1[2][0] + roh2[1] * dr1[2][1] + roh2[2] * dr1[2][2]);
                }
            }
    };
    double s = 1.0;
    bead_thermostat_step(xi1);
    if (global_thermostat) {
        orc_nose_hoover(&s, uk_state, vxi_global, tau, delt2, 3 * na * P, mp->temp * P);
        for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] * s;
    }
    for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] - MASSCON * dRRt[i] * delt2;
    double vir[2] = {0.0, 0.0};  // virialmon, virialcmon
    std::vector<double> dRRmon(nall);
    if (mode == 0) {
        centroid_pbc();
        for (int ti = 1; ti <= intra_timesteps; ti++) {
            for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] - MASSCON * dRRfast[i] * delt2fast;
            drift(deltfast);
            vir[0] = vir[1] = 0.0;
            monomer(dRRfast, ti == intra_timesteps, vir);
            for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] - MASSCON * dRRfast[i] * delt2fast;
        }
        centroid_pbc();
    } else {
        drift(mp->delt);
        centroid_pbc();
    }
    // the intermolecular (mode 0) or the full (mode 1) potential on the centroid
    double Uc, vt[9], vcc;
    std::vector<double> dRRc(3 * (size_t)na), dI(3 * (size_t)nw), dE(3 * (size_t)nw), chg(na);
    o->pot_ttm(0, RRc, RRc, &Uc, dRRc.data(), vt, &vcc, dI.data(), dE.data(), chg.data(), t);
    if (mode == 1) {  // Upott(:) = Upot, then the beads' monomer energies (MD.f90:179-198)
        for (int j = 0; j < P; j++) Upott[j] = Uc;
        monomer(dRRmon.data(), true, vir);
    }
    for (int j = 0; j < P; j++) {
        if (mode == 0) Upott[j] = Upott[j] + Uc;  // MD.f90:400
        for (int i = 0; i < 3 * na; i++)
            dRRt[i + (size_t)3 * na * j] = mode == 0 ? dRRc[i] : dRRc[i] + dRRmon[i + (size_t)3 * na * j];
    }
    if (dip_momIt || dip_momEt) {  // calc_monomer_dip_moments + the centroid's induced dipoles
        const double gammaM = o->m.gammaM, tmp = 0.5 * gammaM / (1.0 - gammaM);
        for (int j = 0; j < P; j++)
            for (int iw = 0; iw < nw; iw++) {
                const double *rb = RRt + (size_t)3 * na * j + 9 * (size_t)iw;
                double r1[3][3], q3[3], dq3[3][3][3];
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) r1[a][c] = rb[3 * a + c];
                o->dms_nasa(r1, q3, dq3);
                for (int a = 0; a < 3; a++) q3[a] = q3[a] * CHARGECON;
                const double cH1 = q3[1] + tmp * (q3[1] + q3[2]), cH2 = q3[2] + tmp * (q3[1] + q3[2]);
                double roh1[3], roh2[3], Rm[3], d[3];
                for (int c = 0; c < 3; c++) {
                    roh1[c] = rb[3 + c] - rb[c];
                    roh1[c] = roh1[c] - o->box[c] * anint(roh1[c] * o->boxi[c]);
                    roh2[c] = rb[6 + c] - rb[c];
                    roh2[c] = roh2[c] - o->box[c] * anint(roh2[c] * o->boxi[c]);
                }
                if (o->p.pot_model == 3 || o->p.pot_model == 4) {
                    for (int c = 0; c < 3; c++) Rm[c] = 0.5 * gammaM * (roh1[c] + roh2[c]) + rb[c];
                    for (int c = 0; c < 3; c++) {
                        double h1 = rb[3 + c] - Rm[c], h2 = rb[6 + c] - Rm[c];
                        h1 = h1 - o->box[c] * anint(h1 * o->boxi[c]);
                        h2 = h2 - o->box[c] * anint(h2 * o->boxi[c]);
                        d[c] = cH1 * h1 + cH2 * h2;
                    }
                } else {
                    for (int c = 0; c < 3; c++) d[c] = cH1 * roh1[c] + cH2 * roh2[c];
                }
                for (int c = 0; c < 3; c++) {
                    if (dip_momIt) dip_momIt[c + 3 * (size_t)iw + (size_t)3 * nw * j] = d[c] + dE[3 * iw + c];
                    if (dip_momEt) dip_momEt[c + 3 * (size_t)iw + (size_t)3 * nw * j] = dE[3 * iw + c];
                }
            }
    }
    double U = 0;
    for (int j = 0; j < P; j++) U += Upott[j];
    out[0] = U;
    out[1] = vir[0] + vt[0] + vt[4] + vt[8];
    out[2] = vir[1] / P + vcc;
    out[4] = orc_calc_uk(P, na, mp->massO, mp->massH, PPt, mp->setNMfreq, C.data(), msf.data());
    out[5] = orc_ring_k0(P, na, mp->massO, mp->massH, RRt);
    orc_estimators(na, P, o->box[0] * o->box[1] * o->box[2], omegan, out[0], out[1], out[2], out[4], out[5], out + 6);
    for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] - MASSCON * dRRt[i] * delt2;
    bead_thermostat_step(xi2);
    double ukv = orc_calc_uk(P, na, mp->massO, mp->massH, PPt, mp->setNMfreq, C.data(), msf.data());
    s = 1.0;
    *uk_state = ukv;
    if (global_thermostat) {
        orc_nose_hoover(&s, uk_state, vxi_global, tau, delt2, 3 * na * P, mp->temp * P);
        for (size_t i = 0; i < nall; i++) PPt[i] = PPt[i] * s;
        ukv = *uk_state;
    }
    out[3] = ukv;
    out[11] = s;
}

// ---------------------------------------------------------------------------------------------
// Analysis (geometry_calculator.f90, diffusion_calculator.f90, spectral_properties.f90, four1.f,
// math.f90:42-140). Geometry accumulator layout (ORC_GEOM_N doubles): [0..5] sum_HH, sum_OH,
// sum_HOH, sum_HH2, sum_OH2, sum_HOH2; [6..11] the bead sums in the same order; [12] max_OH,
// [13] bmax_OH, [14] num_total, [15] num_warn, [16..95] dOHhist, [96..175] bdOHhist.
static const double GEO_MIN = (double)0.6f, GEO_MAX = (double)1.6f;  // default-real literals .6 and 1.6
static const int GEO_NB = 80;

// geometry_calculator.f90:235-259 binit (normal binning)
static void geo_binit(double *hist, double x) {
    const double delta = (GEO_MAX - GEO_MIN) / GEO_NB;
    if (x > GEO_MIN && x < GEO_MAX) {
        int bin = (int)anint((x - GEO_MIN) / delta);
        if (bin == 0) bin = 1;
        if (bin > GEO_NB) bin = GEO_NB;
        hist[bin - 1] = hist[bin - 1] + 1;
    }
}

// geometry_calculator.f90:21-125 calc_geometry: centroid and bead O-H / H-H distances, H-O-H
// angles, running sums, maxima (the centroid maximum takes d_OH1 when d_OH2 exceeds it, as the
// reference's line does), dOH histograms; warnings counted, not printed
void orc_geometry_accumulate(double *acc, int natoms, int P, const double *box, const double *RR, const double *RRt) {
    const int nw = natoms / 3;
    const double dOHmax = 1.5;
    double boxi[3] = {1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
    auto dist = [&](const double *a, const double *b, double *v) {
        for (int c = 0; c < 3; c++) {
            v[c] = a[c] - b[c];
            v[c] = v[c] - box[c] * anint(v[c] * boxi[c]);
        }
    };
    for (int pass = 0; pass <= P; pass++) {  // pass 0: the centroid; 1..P: the beads
        const double *X = pass == 0 ? RR : RRt + (size_t)3 * natoms * (pass - 1);
        double *sm = acc + (pass == 0 ? 0 : 6);
        for (int i = 0; i < nw; i++) {
            const double *rO = X + 9 * (size_t)i, *rH2 = rO + 3, *rH1 = rO + 6;  // ih1 = 3i, ih2 = 3i-1
            double ROH1[3], ROH2[3], RHH[3];
            dist(rO, rH1, ROH1);
            dist(rO, rH2, ROH2);
            dist(rH2, rH1, RHH);
            const double dHH = std::sqrt(RHH[0] * RHH[0] + RHH[1] * RHH[1] + RHH[2] * RHH[2]);
            const double d1 = std::sqrt(ROH1[0] * ROH1[0] + ROH1[1] * ROH1[1] + ROH1[2] * ROH1[2]);
            const double d2 = std::sqrt(ROH2[0] * ROH2[0] + ROH2[1] * ROH2[1] + ROH2[2] * ROH2[2]);
            const double dHOH = std::acos((d1 * d1 + d2 * d2 - dHH * dHH) / (2.0 * d1 * d2));
            if (d1 > dOHmax) acc[15] += 1;
            if (d2 > dOHmax) acc[15] += 1;
            if (pass == 0) {
                if (d1 > acc[12]) acc[12] = d1;
                if (d2 > acc[12]) acc[12] = d1;
                geo_binit(acc + 16, d1);
                geo_binit(acc + 16, d2);
            } else {
                if (d1 > acc[13]) acc[13] = d1;
                if (d2 > acc[13]) acc[13] = d2;
                geo_binit(acc + 96, d1);
                geo_binit(acc + 96, d2);
            }
            sm[0] = sm[0] + dHH;
            sm[1] = sm[1] + d1 + d2;
            if (pass == 0 || std::fabs(dHOH) > 0) sm[2] = sm[2] + dHOH;
            sm[3] = sm[3] + dHH * dHH;
            sm[4] = sm[4] + d1 * d1 + d2 * d2;
            sm[5] = sm[5] + dHOH * dHOH;
        }
    }
    acc[14] += nw;
}

// geometry_calculator.f90:129-190 write_out_geometry: averages and RMS (degrees for angles)
// out[14]: avg_HH, RMS_HH, avg_OH, RMS_OH, avg_HOH, RMS_HOH, then the bead ones, max_OH, bmax_OH
void orc_geometry_report(const double *acc, int P, double *out) {
    const double nt = acc[14], bn = nt * P, deg = 180.0 / 3.141592;
    for (int b = 0; b < 2; b++) {
        const double *sm = acc + 6 * b;
        const double n = b ? bn : nt;
        const double aHH = sm[0] / n, aOH = sm[1] / (2.0 * n), aHOH = (sm[2] / n) * deg;
        const double aHH2 = sm[3] / n, aOH2 = sm[4] / (2.0 * n), aHOH2 = (sm[5] / n) * (deg * deg);
        out[6 * b + 0] = aHH;
        out[6 * b + 1] = std::sqrt(aHH2 - aHH * aHH);
        out[6 * b + 2] = aOH;
        out[6 * b + 3] = std::sqrt(aOH2 - aOH * aOH);
        out[6 * b + 4] = aHOH;
        out[6 * b + 5] = std::sqrt(aHOH2 - aHOH * aHOH);
    }
    out[12] = acc[12];
    out[13] = acc[13];
}

// diffusion_calculator.f90:14-58 calc_diff_RMSD: state = [t, initialised, aMS(ntimes + 1),
// netdisp(3 Nw), Oxy(3 Nw)]; the tracked atom of molecule ia is atom 3 ia (1-based), as the
// reference's Oxy2(:,ia) = RRc(:,3*ia) takes it
void orc_msd_step(double *st, int natoms, int ntimes, const double *box, const double *RRc) {
    const int nw = natoms / 3, t_out = 20;
    double *aMS = st + 2, *net = aMS + ntimes + 1, *Oxy = net + 3 * nw;
    const double boxi0 = 1.0 / box[0];
    st[0] += 1;
    if (st[1] == 0) {
        st[0] = 0;
        st[1] = 1;
        for (int i = 0; i < nw; i++)
            for (int c = 0; c < 3; c++) Oxy[3 * i + c] = RRc[3 * (3 * i + 2) + c];
    }
    const int t = (int)st[0];
    for (int i = 0; i < nw; i++)
        for (int c = 0; c < 3; c++) {
            const double o2 = RRc[3 * (3 * i + 2) + c];
            double d = o2 - Oxy[3 * i + c];
            d = d - box[0] * anint(d * boxi0);
            net[3 * i + c] = net[3 * i + c] + d;
            Oxy[3 * i + c] = o2;
        }
    if (t % t_out == 0) {
        const int ti = t / t_out + 1;
        if (ti <= ntimes + 1) {
            for (int i = 0; i < nw; i++)
                aMS[ti - 1] = aMS[ti - 1] + (net[3 * i] * net[3 * i] + net[3 * i + 1] * net[3 * i + 1] +
                                             net[3 * i + 2] * net[3 * i + 2]);
            aMS[ti - 1] = aMS[ti - 1] / nw;
        }
    }
}

// diffusion_calculator.f90:60-118 write_out_diffusion: least squares over the last half of
// aMS(t) with the reference's single-precision times and its (ntimesfit - 1) divisors; out[4] =
// D, errD (10^-5 cm^2/s), slope b, intercept a
void orc_msd_report(const double *aMS, int ntimes, double timestep, double *out) {
    const int t_out = 20;
    const float frac = 0.5f;
    std::vector<float> times(ntimes);
    for (int i = 1; i <= ntimes; i++) times[i - 1] = (float)(i * t_out * timestep);
    const int ft = (int)std::floor(frac * ntimes) + 1;
    const int nfit = ntimes - ft;
    double xbar = 0, ybar = 0, sx = 0, sy = 0, cr = 0;
    for (int i = ft; i <= ntimes; i++) xbar += (double)(times[i - 1] / (float)(nfit - 1));
    for (int i = ft; i <= ntimes; i++) ybar += aMS[i - 1] / (nfit - 1);
    for (int i = ft; i <= ntimes; i++) {
        sx += ((double)times[i - 1] - xbar) * ((double)times[i - 1] - xbar);
        sy += (aMS[i - 1] - ybar) * (aMS[i - 1] - ybar);
        cr += (aMS[i - 1] - ybar) * ((double)times[i - 1] - xbar);
    }
    const double b = cr / sx, a = ybar - b * xbar;
    double errb = (sy / sx - b * b) / (nfit - 2);
    errb = std::sqrt(errb);
    out[0] = 10 * b / 6;
    out[1] = errb / 6;
    out[2] = b;
    out[3] = a;
}

// four1.f (Numerical Recipes): in-place FFT of nn complex REAL values, twiddles by the DOUBLE
// recurrence; isign = 1: exp(+2 pi i jk / nn), -1: exp(-...)
void orc_four1(float *data, int nn, int isign) {
    const int n = 2 * nn;
    int j = 1;
    for (int i = 1; i <= n; i += 2) {
        if (j > i) {
            std::swap(data[j - 1], data[i - 1]);
            std::swap(data[j], data[i]);
        }
        int m = n / 2;
        while (m >= 2 && j > m) {
            j -= m;
            m /= 2;
        }
        j += m;
    }
    int mmax = 2;
    while (n > mmax) {
        const int istep = 2 * mmax;
        const double theta = 6.28318530717959 / (isign * mmax);
        const double st = std::sin(0.5 * theta);
        const double wpr = -2.0 * st * st, wpi = std::sin(theta);
        double wr = 1.0, wi = 0.0;
        for (int m = 1; m <= mmax; m += 2) {
            for (int i = m; i <= n; i += istep) {
                const int jj = i + mmax;
                const float tr = (float)wr * data[jj - 1] - (float)wi * data[jj];
                const float ti = (float)wr * data[jj] + (float)wi * data[jj - 1];
                data[jj - 1] = data[i - 1] - tr;
                data[jj] = data[i] - ti;
                data[i - 1] = data[i - 1] + tr;
                data[i] = data[i] + ti;
            }
            const double wt = wr;
            wr = wr * wpr - wi * wpi + wr;
            wi = wi * wpr + wt * wpi + wi;
        }
        mmax = istep;
    }
}

static int pow2_floor_log(int n, int add) { return 1 << ((int)std::floor(std::log((double)n) / std::log(2.0)) + add); }

// math.f90:45-81 calc_corr_function (zero-padded to 2 trun, trun = 2^(floor(log2 tread) + 1);
// lag i - 1 of output(i) divided by tread - i for i < tread)
void orc_corr_function(const float *in, int tread, double *out) {
    const int trun = pow2_floor_log(tread, 1);
    std::vector<float> tr(4 * (size_t)trun, 0.0f);
    for (int i = 0; i < tread; i++) tr[2 * i] = in[i];
    orc_four1(tr.data(), 2 * trun, 1);
    for (int i = 0; i < 2 * trun; i++) {
        const float re = tr[2 * i], im = tr[2 * i + 1];
        tr[2 * i] = re * re + im * im;  // z conj(z)
        tr[2 * i + 1] = 0.0f;
    }
    orc_four1(tr.data(), 2 * trun, -1);
    for (int i = 0; i < tread; i++) out[i] = (double)tr[2 * i];
    for (int i = 1; i <= tread - 1; i++) out[i - 1] = out[i - 1] / (tread - i);
}

// math.f90:88-116 calc_DFT
void orc_calc_dft(const double *in, int tread, double timestep, double *out, double *freqs) {
    const int trun = pow2_floor_log(tread, 1);
    std::vector<float> tr(4 * (size_t)trun, 0.0f);
    for (int i = 0; i < tread; i++) tr[2 * i] = (float)in[i];
    orc_four1(tr.data(), 2 * trun, 1);
    for (int i = 0; i < tread; i++) out[i] = (double)tr[2 * i] / (2.0 * trun);
    for (int i = 0; i < tread; i++) freqs[i] = (double)i / (timestep * 2.0 * trun);
}

// math.f90:123-140 block_average
static void block_average(const double *in, int n, int N, double *out) {
    const int bs = (int)std::floor((float)n / (float)N);
    if (bs == 0) {
        for (int i = 0; i < N && i < n; i++) out[i] = in[i];
        return;
    }
    for (int i = 0; i < N; i++) {
        double s = 0;
        for (int k = i * bs; k < (i + 1) * bs; k++) s += in[k];
        out[i] = s / bs;
    }
}

// spectral_properties.f90:10-123 calc_infrared_spectrum from the total dipole dip(3, tread)
// (REAL, Debye): the autocorrelation by FFT over 2 trun points (trun = 2^floor(log2 tread); the
// first trun samples, zero-padded -- the reference leaves the padding uninitialised), its FFT, and
// the omega^2-weighted, block-averaged line shape up to 7000 cm^-1. npoints inout (the module
// variable NumPointsOut, 350 at start); freq (cm^-1) and ir out, npoints of each.
void orc_ir_spectrum(const float *dip, int tread, const double *box, double timestep, double temp, int *npoints,
                     double *freq, double *ir) {
    const double ps2s = 1e-12, Cspeed = 3.00e10, Debye2SI = 3.33564e-30, eps0 = 8.854187e-12, kb = 0.0019872041;
    const double vol = (box[0] * box[1] * box[2]) * 1e-30;
    const int trun = pow2_floor_log(tread, 0), n = 2 * trun;
    std::vector<float> ACF(2 * (size_t)n, 0.0f), aux(2 * (size_t)n);
    for (int ix = 0; ix < 3; ix++) {
        std::fill(aux.begin(), aux.end(), 0.0f);
        for (int i = 0; i < trun; i++) aux[2 * i] = dip[ix + 3 * (size_t)i];
        orc_four1(aux.data(), n, -1);
        for (int i = 0; i < n; i++) {
            const float re = aux[2 * i], im = aux[2 * i + 1];
            aux[2 * i] = re * re + im * im;
            aux[2 * i + 1] = 0.0f;
        }
        orc_four1(aux.data(), n, 1);
        for (int i = 0; i < 2 * n; i++) ACF[i] = ACF[i] + aux[i];
    }
    aux = ACF;  // aux1 = cmplx(ACF): the complex ACF as it is
    orc_four1(aux.data(), n, -1);
    const double MinFreqOut = 1.0 / (timestep * ps2s * Cspeed * n);
    const double PointsAvailable = std::floor(7000.0 / MinFreqOut);
    int NumAvgOver;
    if (PointsAvailable < *npoints) {
        *npoints = (int)PointsAvailable;
        NumAvgOver = 1;
    } else {
        NumAvgOver = (int)std::floor(PointsAvailable / *npoints);
    }
    for (int t = 0; t < *npoints; t++) {
        double avg = 0;
        for (int i = 1; i <= NumAvgOver; i++) {
            const double omega = (t * NumAvgOver + i) / (timestep * n * ps2s);
            avg = avg + (omega * omega) * (double)aux[2 * (t * NumAvgOver + i)];
        }
        avg = avg / (double)(float)NumAvgOver;
        double IR = (2.0 * 3.14159 * (Debye2SI * Debye2SI) * avg) / (3.0 * vol * 2.99e8 * kb * temp * eps0);
        IR = IR * ps2s;
        IR = IR * .01;
        IR = IR * 2;
        double omega = std::floor((t + .5f) * NumAvgOver) / (timestep * n * ps2s);
        freq[t] = omega / Cspeed;
        ir[t] = IR;
    }
}

// spectral_properties.f90:128-187 calc_DOS from Hvel(3, tread, nhyd) (REAL): the velocity
// autocorrelations (calc_corr_function) summed, normalised by nhyd and lag 0, calc_DFT, and
// block averages of frequency (cm^-1) and spectrum up to 7000 cm^-1; npoints inout as above
void orc_dos(const float *Hvel, int tread, int nhyd, double timestep, int *npoints, double *freq, double *dos) {
    const double ps2s = 1e-12, Cspeed = 3.00e10;
    std::vector<double> ACF(tread, 0.0), out(tread), DFT(tread), fr(tread);
    std::vector<float> in(tread);
    for (int iH = 0; iH < nhyd; iH++)
        for (int ix = 0; ix < 3; ix++) {
            for (int i = 0; i < tread; i++) in[i] = Hvel[ix + 3 * ((size_t)i + (size_t)tread * iH)];
            orc_corr_function(in.data(), tread, out.data());
            for (int i = 0; i < tread; i++) ACF[i] = ACF[i] + out[i];
        }
    const double a0 = ACF[0];  // ACF = ACF/Nhyd/ACF(1): the right-hand side before the assignment
    for (int i = 0; i < tread; i++) ACF[i] = ACF[i] / nhyd / a0;
    orc_calc_dft(ACF.data(), tread, timestep, DFT.data(), fr.data());
    for (int i = 0; i < tread; i++) fr[i] = fr[i] / (ps2s * Cspeed);
    const double MinFreqOut = fr[1];
    const int PointsAvailable = std::min(tread, (int)std::floor(7000.0 / MinFreqOut));
    if (PointsAvailable < *npoints) *npoints = PointsAvailable;
    block_average(fr.data(), PointsAvailable, *npoints, freq);
    block_average(DFT.data(), PointsAvailable, *npoints, dos);
}

}  // extern "C"
