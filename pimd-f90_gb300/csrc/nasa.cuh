// nasa.cuh -- Partridge-Schwenke water monomer PES and dipole-moment surface on the device.
// Restates pot_ttm/nasa.f90:2-103 (pot_nasa) and :105-293 (dms_nasa) in FP64; one thread
// evaluates one molecule. Coefficient tables live in constant memory (all threads of a warp
// read the same term at the same time, so the reads are broadcasts).
#pragma once
#include "common.cuh"
#include "nasa_tables.h"

namespace pimd {

// Per translation unit (each .cu that includes this header has its own copy in its own device
// module): nasa_upload_constants() fills this unit's copy.
static __constant__ double c_c5z[245];
static __constant__ double c_coefD[84];
static __constant__ float c_c5zf[245];  // FP32 copies for the mixed engine's polynomial sums
static __constant__ float c_coefDf[84];
static __constant__ unsigned char c_idx[245][3];
static __constant__ unsigned char c_idxD[84][3];
// The sums of pot_nasa (terms 1..244) and dms_nasa (terms 1..83) regrouped by the powers (i, j)
// of x1, x2: per group, slots k = n .. 1 (descending, for Horner in x3) hold the term with
// power k of f3, or -1 where the table has none. Group: i, j, first slot, slots.
constexpr int NASA_PG = 32, NASA_PS = 256, NASA_DG = 32, NASA_DS = 128;
static __constant__ unsigned char c_pg[NASA_PG][4];
static __constant__ short c_ps[NASA_PS];
static __constant__ unsigned char c_dg[NASA_DG][4];
static __constant__ short c_ds[NASA_DS];
static __constant__ int c_ngrp[2];  // groups of the PES and of the DMS

// group terms j0 .. j1 - 1 of an (i, j, k) table by (i, j); returns the group count (-1: too many)
static inline int nasa_group(const int *I, const int *J, const int *K, int j0, int j1, unsigned char (*grp)[4], short *slot,
                             int maxg, int maxs) {
    int ng = 0, ns = 0;
    for (int a = 1; a <= 16; a++)
        for (int b = 1; b <= 16; b++) {
            int kmax = 0;
            for (int t = j0; t < j1; t++)
                if (I[t] == a && J[t] == b) kmax = K[t] > kmax ? K[t] : kmax;
            if (!kmax) continue;
            if (ng >= maxg || ns + kmax > maxs) return -1;
            grp[ng][0] = (unsigned char)a;
            grp[ng][1] = (unsigned char)b;
            grp[ng][2] = (unsigned char)ns;
            grp[ng][3] = (unsigned char)kmax;
            for (int k = kmax; k >= 1; k--) {
                short js = -1;
                for (int t = j0; t < j1; t++)
                    if (I[t] == a && J[t] == b && K[t] == k) js = (short)t;
                slot[ns++] = js;
            }
            ng++;
        }
    return ng;
}

// c5z = f5z C5ZA + fbasis CBASIS + fcore CCORE + frest CREST (nasa_mod.f90) and the index tables
static inline void nasa_upload_constants() {
    double c5z[245];
    for (int j = 0; j < 245; j++)
        c5z[j] = PIMD_NASA_F5Z * PIMD_NASA_C5ZA[j] + PIMD_NASA_FBASIS * PIMD_NASA_CBASIS[j] +
                 PIMD_NASA_FCORE * PIMD_NASA_CCORE[j] + PIMD_NASA_FREST * PIMD_NASA_CREST[j];
    unsigned char idx[245][3], idxD[84][3];
    for (int j = 0; j < 245; j++) {
        idx[j][0] = (unsigned char)PIMD_NASA_IDX1[j];
        idx[j][1] = (unsigned char)PIMD_NASA_IDX2[j];
        idx[j][2] = (unsigned char)PIMD_NASA_IDX3[j];
    }
    for (int j = 0; j < 84; j++) {
        idxD[j][0] = (unsigned char)PIMD_NASA_IDXD1[j];
        idxD[j][1] = (unsigned char)PIMD_NASA_IDXD2[j];
        idxD[j][2] = (unsigned char)PIMD_NASA_IDXD3[j];
    }
    cudaMemcpyToSymbol(c_c5z, c5z, sizeof(c5z));
    cudaMemcpyToSymbol(c_coefD, PIMD_NASA_COEFD, sizeof(double) * 84);
    float c5zf[245], coefDf[84];
    for (int j = 0; j < 245; j++) c5zf[j] = (float)c5z[j];
    for (int j = 0; j < 84; j++) coefDf[j] = (float)PIMD_NASA_COEFD[j];
    cudaMemcpyToSymbol(c_c5zf, c5zf, sizeof(c5zf));
    cudaMemcpyToSymbol(c_coefDf, coefDf, sizeof(coefDf));
    cudaMemcpyToSymbol(c_idx, idx, sizeof(idx));
    cudaMemcpyToSymbol(c_idxD, idxD, sizeof(idxD));
    unsigned char pg[NASA_PG][4] = {}, dg[NASA_DG][4] = {};
    short ps[NASA_PS], ds[NASA_DS];
    for (int i = 0; i < NASA_PS; i++) ps[i] = -1;
    for (int i = 0; i < NASA_DS; i++) ds[i] = -1;
    int ng[2];
    ng[0] = nasa_group(PIMD_NASA_IDX1, PIMD_NASA_IDX2, PIMD_NASA_IDX3, 1, 245, pg, ps, NASA_PG, NASA_PS);
    ng[1] = nasa_group(PIMD_NASA_IDXD1, PIMD_NASA_IDXD2, PIMD_NASA_IDXD3, 1, 84, dg, ds, NASA_DG, NASA_DS);
    cudaMemcpyToSymbol(c_pg, pg, sizeof(pg));
    cudaMemcpyToSymbol(c_ps, ps, sizeof(ps));
    cudaMemcpyToSymbol(c_dg, dg, sizeof(dg));
    cudaMemcpyToSymbol(c_ds, ds, sizeof(ds));
    cudaMemcpyToSymbol(c_ngrp, ng, sizeof(ng));
}

// The PES polynomial sums (nasa.f90:62-72) in the arithmetic type S: sum0 = sum_t c_t sym_t
// f3[k_t], sum3 its x3-derivative, sum1, sum2 the x1-, x2-derivatives. Per (i, j) group the
// k-sum is a polynomial in x3, evaluated by Horner together with its derivative (two FMAs per
// term). S = float (the mixed engine, published coefficients only) keeps the rest of the
// monomer in FP64: the sums carry about 1e-7 relative error into the gradient.
// a / d, or with fx (the mixed engine) a times the reciprocal id computed once: FP64 division
// costs this part a dozen FP64 instructions
PIMD_D double qdiv(double a, double d, double id, bool fx) { return fx ? a * id : a / d; }

template <typename S>
PIMD_D void nasa_pot_sums(double x1d, double x2d, double x3d, const double *c5zg, double &s0d, double &s1d, double &s2d,
                          double &s3d) {
    const S x1 = (S)x1d, x2 = (S)x2d, x3 = (S)x3d;
    S f1[16], f2[16];
    f1[0] = f2[0] = S(0);
    f1[1] = f2[1] = S(1);
#pragma unroll
    for (int j = 2; j <= 15; j++) {
        f1[j] = f1[j - 1] * x1;
        f2[j] = f2[j - 1] * x2;
    }
    S sum0 = 0, sum1 = 0, sum2 = 0, sum3 = 0;
    for (int g = 0; g < c_ngrp[0]; g++) {
        const int inI = c_pg[g][0], inJ = c_pg[g][1], s0 = c_pg[g][2], n = c_pg[g][3];
        S pk = S(0), dpk = S(0);
        for (int t = 0; t < n; t++) {
            const int j = c_ps[s0 + t];
            S c;
            if (sizeof(S) == sizeof(float))
                c = j < 0 ? S(0) : (S)c_c5zf[j];
            else
                c = j < 0 ? S(0) : (S)(c5zg ? c5zg[j] : c_c5z[j]);
            dpk = dpk * x3 + pk;
            pk = pk * x3 + c;
        }
        const S sym = f1[inI] * f2[inJ] + f1[inJ] * f2[inI];
        sum0 += sym * pk;
        sum1 += ((S)(inI - 1) * f1[inI - 1] * f2[inJ] + (S)(inJ - 1) * f1[inJ - 1] * f2[inI]) * pk;
        sum2 += ((S)(inJ - 1) * f1[inI] * f2[inJ - 1] + (S)(inI - 1) * f1[inJ] * f2[inI - 1]) * pk;
        sum3 += sym * dpk;
    }
    s0d = (double)sum0;
    s1d = (double)sum1;
    s2d = (double)sum2;
    s3d = (double)sum3;
}

// r1[atom][comp]: atoms O, H1, H2. Returns energy (kcal/mol) and gradient dr1[atom][comp].
// c5zg: the 245 combined coefficients when the four scale factors differ from the published
// ones (null: the constant-memory table), f5z: the CCSD(T)/5Z scale factor of deoh and phh1.
// fsum: polynomial sums in FP32 (ignored with c5zg).
PIMD_D void nasa_pot(const double r1[3][3], const double box[3], const double boxi[3], double dr1[3][3],
                     double *e1, const double *c5zg = nullptr, double f5z = PIMD_NASA_F5Z, bool fsum = false) {
    double ROH1[3], ROH2[3], RHH[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        ROH1[c] = min_image_rn(__dsub_rn(r1[1][c], r1[0][c]), box[c], boxi[c]);
        ROH2[c] = min_image_rn(__dsub_rn(r1[2][c], r1[0][c]), box[c], boxi[c]);
        RHH[c] = min_image_rn(__dsub_rn(r1[1][c], r1[2][c]), box[c], boxi[c]);
    }
    const double dROH1 = sqrt(ROH1[0] * ROH1[0] + ROH1[1] * ROH1[1] + ROH1[2] * ROH1[2]);
    const double dROH2 = sqrt(ROH2[0] * ROH2[0] + ROH2[1] * ROH2[1] + ROH2[2] * ROH2[2]);
    const double dRHH = sqrt(RHH[0] * RHH[0] + RHH[1] * RHH[1] + RHH[2] * RHH[2]);
    // fsum: the exponentials in FP32 as well (the FP64 ones dominate this part's FP64 work); the
    // Morse terms from em = e^x - 1 (expm1f), which keeps 1 - e^x at FP32 relative precision
    // where it cancels near the equilibrium bond length; divisions by reciprocals
    const bool fx = fsum && !c5zg;
    const double i1 = fx ? 1.0 / dROH1 : 0.0, i2 = fx ? 1.0 / dROH2 : 0.0, ihh = fx ? 1.0 / dRHH : 0.0;
    const double i12 = i1 * i2, ireoh = 1.0 / PIMD_NASA_REOH;
    const double costh = qdiv(ROH1[0] * ROH2[0] + ROH1[1] * ROH2[1] + ROH1[2] * ROH2[2], dROH1 * dROH2, i12, fx);
    const double reoh = PIMD_NASA_REOH, b1 = PIMD_NASA_B1, roh = PIMD_NASA_ROH, alphaoh = PIMD_NASA_ALPHAOH,
                 phh2 = PIMD_NASA_PHH2;
    const double deoh = f5z * PIMD_NASA_DEOHA;
    const double costhe = -.24780227221366464506;
    const double phh1 = (f5z * PIMD_NASA_PHH1A) * (fx ? (double)expf((float)phh2) : exp(phh2));
    double Va, dVa1, dVa2;
    if (fx) {
        const double em1 = (double)expm1f((float)(-alphaoh * (dROH1 - roh)));
        const double em2 = (double)expm1f((float)(-alphaoh * (dROH2 - roh)));
        Va = deoh * ((em1 * em1 - 1.0) + (em2 * em2 - 1.0));
        dVa1 = -2.0 * alphaoh * deoh * (1.0 + em1) * em1 * i1;
        dVa2 = -2.0 * alphaoh * deoh * (1.0 + em2) * em2 * i2;
    } else {
        const double exp1 = exp(-alphaoh * (dROH1 - roh));
        const double exp2 = exp(-alphaoh * (dROH2 - roh));
        Va = deoh * (exp1 * (exp1 - 2.0) + exp2 * (exp2 - 2.0));
        dVa1 = 2.0 * alphaoh * deoh * exp1 * (1.0 - exp1) / dROH1;
        dVa2 = 2.0 * alphaoh * deoh * exp2 * (1.0 - exp2) / dROH2;
    }
    const double Vb = phh1 * (fx ? (double)expf((float)(-phh2 * dRHH)) : exp(-phh2 * dRHH));
    const double dVb = qdiv(-phh2 * Vb, dRHH, ihh, fx);
    const double x1 = qdiv(dROH1 - reoh, reoh, ireoh, fx), x2 = qdiv(dROH2 - reoh, reoh, ireoh, fx), x3 = costh - costhe;
    const double earg = -b1 * ((dROH1 - reoh) * (dROH1 - reoh) + (dROH2 - reoh) * (dROH2 - reoh));
    const double efac = fx ? (double)expf((float)earg) : exp(earg);
    double sum0, sum1, sum2, sum3;
    if (fsum && !c5zg)
        nasa_pot_sums<float>(x1, x2, x3, nullptr, sum0, sum1, sum2, sum3);
    else
        nasa_pot_sums<double>(x1, x2, x3, c5zg, sum0, sum1, sum2, sum3);
    const double Vc = 2.0 * (c5zg ? c5zg[0] : c_c5z[0]) + efac * sum0;
    *e1 = ((Va + Vb + Vc) + 0.44739574026257) * 0.00285914375100642899;
    const double dVcdr1 = qdiv(-2.0 * b1 * efac * (dROH1 - reoh) * sum0 + qdiv(efac * sum1, reoh, ireoh, fx), dROH1, i1, fx);
    const double dVcdr2 = qdiv(-2.0 * b1 * efac * (dROH2 - reoh) * sum0 + qdiv(efac * sum2, reoh, ireoh, fx), dROH2, i2, fx);
    const double dVcdcth = efac * sum3;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double g1 = dVa1 * ROH1[c] + dVb * RHH[c] + dVcdr1 * ROH1[c] +
                    dVcdcth * (qdiv(ROH2[c], dROH1 * dROH2, i12, fx) - qdiv(costh * ROH1[c], dROH1 * dROH1, i1 * i1, fx));
        double g2 = dVa2 * ROH2[c] - dVb * RHH[c] + dVcdr2 * ROH2[c] +
                    dVcdcth * (qdiv(ROH1[c], dROH1 * dROH2, i12, fx) - qdiv(costh * ROH2[c], dROH2 * dROH2, i2 * i2, fx));
        dr1[1][c] = g1 * .00285914375100642899;
        dr1[2][c] = g2 * .00285914375100642899;
        dr1[0][c] = -(g1 + g2) * .00285914375100642899;
    }
}

// dms_nasa after the polynomial sums (nasa.f90:190-293): Legendre/power terms, the TTM3-F
// charge corrections and the charge derivatives
PIMD_D void nasa_dms_finish(const double ROH1[3], const double ROH2[3], double dROH1, double dROH2, double costh,
                            double efac, double P1, double P2, double dp1dr1, double dp1dr2, double dp1dcabc,
                            double dp2dr1, double dp2dr2, double dp2dcabc, double PL1, double PL2, double dms1,
                            double dms2, double dms3, double q3[3], double gradq[3][3][3], bool fx = false) {
    const double reoh = PIMD_NASA_REOH, b1D = PIMD_NASA_B1D, a = PIMD_NASA_A, b = PIMD_NASA_B,
                 c0 = PIMD_NASA_C0, c1 = PIMD_NASA_C1, c2 = PIMD_NASA_C2;
    const double ath0 = 1.82400520401572996557, B2A = 0.529177249;
    const double ireoh = 1.0 / PIMD_NASA_REOH;
    const double i1 = fx ? 1.0 / dROH1 : 0.0, i2 = fx ? 1.0 / dROH2 : 0.0, i12 = i1 * i2;
    dp1dr1 = qdiv(dp1dr1, reoh, ireoh, fx) * B2A;
    dp1dr2 = qdiv(dp1dr2, reoh, ireoh, fx) * B2A;
    dp2dr1 = qdiv(dp2dr1, reoh, ireoh, fx) * B2A;
    dp2dr2 = qdiv(dp2dr2, reoh, ireoh, fx) * B2A;
    // fx (the mixed engine): the powers and the angle in FP32 (FP64 pow is this part's largest
    // FP64 cost); 1e-7 relative in the charges
    const double pw1 = fx ? (double)powf((float)dROH1, (float)b) : pow(dROH1, b);
    const double pw2 = fx ? (double)powf((float)dROH2, (float)b) : pow(dROH2, b);
    const double pm1 = fx ? (double)powf((float)dROH1, (float)(b - 1)) : pow(dROH1, b - 1);
    const double pm2 = fx ? (double)powf((float)dROH2, (float)(b - 1)) : pow(dROH2, b - 1);
    const double leg = c0 + PL1 * c1 + PL2 * c2;
    const double PC0 = a * (pw1 + pw2) * leg;
    const double dpc0dr1 = a * (b * pm1) * leg * B2A * B2A;
    const double dpc0dr2 = a * (b * pm2) * leg * B2A * B2A;
    const double dpc0dcabc = a * (pw1 + pw2) * (c1 + 0.5 * (6.0 * PL1) * c2) * B2A;
    const double defacdr1 = -2.0 * b1D * (dROH1 - reoh) * efac * B2A;
    const double defacdr2 = -2.0 * b1D * (dROH2 - reoh) * efac * B2A;
    dp1dr1 = dp1dr1 * efac + P1 * defacdr1 + dpc0dr1;
    dp1dr2 = dp1dr2 * efac + P1 * defacdr2 + dpc0dr2;
    dp1dcabc = dp1dcabc * efac + dpc0dcabc;
    dp2dr1 = dp2dr1 * efac + P2 * defacdr1 + dpc0dr1;
    dp2dr2 = dp2dr2 * efac + P2 * defacdr2 + dpc0dr2;
    dp2dcabc = dp2dcabc * efac + dpc0dcabc;
    P1 = c_coefD[0] + P1 * efac + PC0 * B2A;
    P2 = c_coefD[0] + P2 * efac + PC0 * B2A;
    // nasa.f90:218: bfac = 1.d0/0.529177249 divides by a single-precision literal
    const double bfac = 1.0 / (double)0.529177249f;
    q3[0] = -(P1 + P2);
    q3[1] = P1;
    q3[2] = P2;
    dp1dr1 *= bfac;
    dp1dr2 *= bfac;
    dp2dr1 *= bfac;
    dp2dr2 *= bfac;
    double AxB0 = ROH1[1] * ROH2[2] - ROH1[2] * ROH2[1];
    double AxB1 = -ROH1[0] * ROH2[2] + ROH1[2] * ROH2[0];
    double AxB2 = ROH1[0] * ROH2[1] - ROH1[1] * ROH2[0];
    const double dAxB = sqrt(AxB0 * AxB0 + AxB1 * AxB1 + AxB2 * AxB2);
    const double sinth = qdiv(dAxB, dROH1 * dROH2, i12, fx);
    const double ang = fx ? (double)atan2f((float)sinth, (float)costh) : atan2(sinth, costh);
    const double Q1 = dms1 * (dROH1 - dms2) + dms3 * (ang - ath0);
    const double Q2 = dms1 * (dROH2 - dms2) + dms3 * (ang - ath0);
    q3[0] = q3[0] - (Q1 + Q2);
    q3[1] = q3[1] + Q1;
    q3[2] = q3[2] + Q2;
    dp1dr1 += dms1;
    dp2dr2 += dms1;
    const double ds = fx ? dms3 / sinth : 0.0;
    dp1dcabc -= fx ? ds : dms3 / sinth;
    dp2dcabc -= fx ? ds : dms3 / sinth;
    const double f1q1r13 = qdiv(dp1dr1 - qdiv(dp1dcabc * costh, dROH1, i1, fx), dROH1, i1, fx);
    const double f1q1r23 = qdiv(dp1dcabc, dROH1 * dROH2, i12, fx);
    const double f2q1r23 = qdiv(dp1dr2 - qdiv(dp1dcabc * costh, dROH2, i2, fx), dROH2, i2, fx);
    const double f2q1r13 = qdiv(dp1dcabc, dROH2 * dROH1, i12, fx);
    const double f1q2r13 = qdiv(dp2dr1 - qdiv(dp2dcabc * costh, dROH1, i1, fx), dROH1, i1, fx);
    const double f1q2r23 = qdiv(dp2dcabc, dROH1 * dROH2, i12, fx);
    const double f2q2r23 = qdiv(dp2dr2 - qdiv(dp2dcabc * costh, dROH2, i2, fx), dROH2, i2, fx);
    const double f2q2r13 = qdiv(dp2dcabc, dROH2 * dROH1, i12, fx);
#pragma unroll
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

// The DMS polynomial sums (nasa.f90:229-241) regrouped by (i, j) with Horner in x3, as in
// nasa_pot_sums, in the arithmetic type S: P1, P2 and their x1-, x2- and x3-derivatives.
template <typename S>
PIMD_D void nasa_dms_sums(double x1d, double x2d, double x3d, double (&out)[8]) {
    const S x1 = (S)x1d, x2 = (S)x2d, x3 = (S)x3d;
    S f1[16], f2[16];
    f1[0] = f2[0] = S(0);
    f1[1] = f2[1] = S(1);
#pragma unroll
    for (int j = 2; j <= 15; j++) {
        f1[j] = f1[j - 1] * x1;
        f2[j] = f2[j - 1] * x2;
    }
    S P1 = 0, P2 = 0, dp1dr1 = 0, dp1dr2 = 0, dp1dcabc = 0, dp2dr1 = 0, dp2dr2 = 0, dp2dcabc = 0;
    for (int g = 0; g < c_ngrp[1]; g++) {
        const int inI = c_dg[g][0], inJ = c_dg[g][1], s0 = c_dg[g][2], n = c_dg[g][3];
        S qk = S(0), dqk = S(0);
        for (int t = 0; t < n; t++) {
            const int j = c_ds[s0 + t];
            S c;
            if (sizeof(S) == sizeof(float))
                c = j < 0 ? S(0) : (S)c_coefDf[j];
            else
                c = j < 0 ? S(0) : (S)c_coefD[j];
            dqk = dqk * x3 + qk;
            qk = qk * x3 + c;
        }
        const S a = f1[inI] * f2[inJ], bb = f1[inJ] * f2[inI];
        P1 += a * qk;
        P2 += bb * qk;
        dp1dr1 += (S)(inI - 1) * f1[inI - 1] * f2[inJ] * qk;
        dp1dr2 += (S)(inJ - 1) * f1[inI] * f2[inJ - 1] * qk;
        dp1dcabc += a * dqk;
        dp2dr1 += (S)(inJ - 1) * f1[inJ - 1] * f2[inI] * qk;
        dp2dr2 += (S)(inI - 1) * f1[inJ] * f2[inI - 1] * qk;
        dp2dcabc += bb * dqk;
    }
    const S r[8] = {P1, P2, dp1dr1, dp1dr2, dp1dcabc, dp2dr1, dp2dr2, dp2dcabc};
#pragma unroll
    for (int i = 0; i < 8; i++) out[i] = (double)r[i];
}

// dms_nasa: site charges q3 (O, H1, H2) in e and gradq[a][b][c] = d q_b / d x_{a,c}
// with a = H1, H2, O (the reference's gradq(a, b, c) ordering).
PIMD_D void nasa_dms(const double r1[3][3], const double box[3], const double boxi[3], double dms1, double dms2,
                     double dms3, double q3[3], double gradq[3][3][3], bool fsum = false) {
    const double reoh = PIMD_NASA_REOH, b1D = PIMD_NASA_B1D, costhe = -.24780227221366464506;
    double ROH1[3], ROH2[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        ROH1[c] = min_image_rn(__dsub_rn(r1[1][c], r1[0][c]), box[c], boxi[c]);
        ROH2[c] = min_image_rn(__dsub_rn(r1[2][c], r1[0][c]), box[c], boxi[c]);
    }
    const double dROH1 = sqrt(ROH1[0] * ROH1[0] + ROH1[1] * ROH1[1] + ROH1[2] * ROH1[2]);
    const double dROH2 = sqrt(ROH2[0] * ROH2[0] + ROH2[1] * ROH2[1] + ROH2[2] * ROH2[2]);
    const double costh = (ROH1[0] * ROH2[0] + ROH1[1] * ROH2[1] + ROH1[2] * ROH2[2]) / (dROH1 * dROH2);
    const double earg = -b1D * ((dROH1 - reoh) * (dROH1 - reoh) + (dROH2 - reoh) * (dROH2 - reoh));
    const double efac = fsum ? (double)expf((float)earg) : exp(earg);
    const double ireoh = 1.0 / PIMD_NASA_REOH;
    const double x1 = qdiv(dROH1 - reoh, reoh, ireoh, fsum), x2 = qdiv(dROH2 - reoh, reoh, ireoh, fsum), x3 = costh - costhe;
    const double PL1 = costh, PL2 = 0.5 * (3.0 * PL1 * PL1 - 1.0);
    double sums[8];
    if (fsum)
        nasa_dms_sums<float>(x1, x2, x3, sums);
    else
        nasa_dms_sums<double>(x1, x2, x3, sums);
    const double P1 = sums[0], P2 = sums[1], dp1dr1 = sums[2], dp1dr2 = sums[3], dp1dcabc = sums[4], dp2dr1 = sums[5],
                 dp2dr2 = sums[6], dp2dcabc = sums[7];
    nasa_dms_finish(ROH1, ROH2, dROH1, dROH2, costh, efac, P1, P2, dp1dr1, dp1dr2, dp1dcabc, dp2dr1, dp2dr2, dp2dcabc,
                    PL1, PL2, dms1, dms2, dms3, q3, gradq, fsum);
}

}  // namespace pimd
