// pot.cu -- real-space, monomer and bookkeeping kernels of the TTM2.1-F / TTM3-F force call
// for all beads at once (FP64). Restates pot_ttm/pot_ttm.f90:3-630 and find_neigh.f90.
//
// Work decomposition: the bead is blockIdx.y (or .z) everywhere. Monomer and intramolecular
// work is one thread per molecule; intermolecular work is one thread per O-O pair of the
// half neighbour list, accumulating the pair's 4+4 site contributions in registers and
// issuing one atomic per site component. Energies and virials are reduced per block and
// added once per block to the per-bead accumulators.
#include <cstdio>

#include "engine.h"
#include "nasa.cuh"

namespace pimd {

// site kinds (1-based like the reference): 1 O, 2 H1, 3 H2, 4 M
template <int MODEL>
struct TT {
    static constexpr int FDI = MODEL == 2 ? 1 : 4;
    static constexpr int LDI = MODEL == 2 ? 3 : 4;
    PIMD_HD static constexpr bool dip(int k) { return k >= FDI && k <= LDI; }
    PIMD_HD static constexpr bool chg(int k) { return k != 1; }
    // charge-phase site pairs that change an output (O carries no charge; its field is
    // only needed when O carries a dipole, TTM2.1-F)
    PIMD_HD static constexpr bool qq_active(int i, int j) {
        return !(i == 1 && j == 1) && (MODEL == 2 || (i != 1 && j != 1));
    }
    // force-phase site pairs with a dipole-dipole or charge-dipole term
    PIMD_HD static constexpr bool f_active(int i, int j) {
        return (dip(i) && dip(j)) || (dip(i) && chg(j)) || (chg(i) && dip(j));
    }
};

void pot_init_constants(Engine &E) {
    (void)E;
    nasa_upload_constants();
}

PIMD_D double3 ld3(const double *p) { return make_double3(p[0], p[1], p[2]); }

// ---------------------------------------------------------------------------------------
// pot_ttm.f90:56-151 and 232-261: site layout, M sites, NASA PES + DMS charges, monomer
// virials, self energy and intramolecular Ewald exclusions. Two threads per (molecule, bead),
// in two warps of a 64-thread block (32 molecules): the first warp evaluates the PES
// (nasa_pot), the monomer virial and the gradient rows; the second the DMS charges (nasa_dms),
// their gradients, the site rows, the self energy and the intramolecular exclusions. The two
// halves share no data, so the FP64-latency-bound chain of a molecule is split in two; about 7
// warps per SM at 512 x 32, spread over every SM.
constexpr int SITES_NT = 64;

// FSUM: the NASA polynomial sums in FP32 (the mixed engine)
template <int MODEL, bool FSUM>
__global__ void __launch_bounds__(SITES_NT) k_sites(KP kp) {
    const int w = blockIdx.x * (SITES_NT / 2) + (threadIdx.x & 31);
    const bool pes = threadIdx.x < 32;  // warp-uniform roles
    const int b = blockIdx.y;
    const int N = kp.N, S = kp.S;
    double av[14];
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.0;
    if (w < N) {
        const double *RR = kp.RRt + (size_t)b * kp.natoms * 3 + 9 * w;
        const int rep = rep_of(kp, b);
        const double *RC = kp.RRc + (size_t)rep * kp.natoms * 3 + 9 * w;
        const bool first_bead = (b == 0) || (kp.brep && kp.brep[b - 1] != rep);
        double R[4][3], Rc[4][3];
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                R[k][c] = RR[3 * k + c];
                Rc[k][c] = RC[3 * k + c];
            }
        const double hg = 0.5 * kp.gammaM;
        // the O-H minimum images of the bead and the centroid (the M sites, and in the mixed
        // engine the FP32 site offsets of the exclusion pairs)
        double oh[2][3], ohc[2][3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            oh[0][c] = min_image_rn(__dsub_rn(R[1][c], R[0][c]), kp.box[c], kp.boxi[c]);
            oh[1][c] = min_image_rn(__dsub_rn(R[2][c], R[0][c]), kp.box[c], kp.boxi[c]);
            R[3][c] = __dadd_rn(__dmul_rn(hg, __dadd_rn(oh[0][c], oh[1][c])), R[0][c]);
            ohc[0][c] = min_image_rn(__dsub_rn(Rc[1][c], Rc[0][c]), kp.box[c], kp.boxi[c]);
            ohc[1][c] = min_image_rn(__dsub_rn(Rc[2][c], Rc[0][c]), kp.box[c], kp.boxi[c]);
            Rc[3][c] = __dadd_rn(__dmul_rn(hg, __dadd_rn(ohc[0][c], ohc[1][c])), Rc[0][c]);
        }
        if (pes) {
            double dr1[3][3], e1 = 0.0;
            if (!kp.contraction) {
                nasa_pot(R, kp.box, kp.boxi, dr1, &e1, kp.c5z, kp.nasa_f5z, FSUM);
            } else {
#pragma unroll
                for (int k = 0; k < 3; k++)
#pragma unroll
                    for (int c = 0; c < 3; c++) dr1[k][c] = 0.0;
            }
            av[ACC_UMON] = e1;
            if (!kp.contraction) {
                double roh1[3], roh2[3], rc1[3], rc2[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    roh1[c] = min_image_rn(__dsub_rn(R[1][c], R[0][c]), kp.box[c], kp.boxi[c]);
                    roh2[c] = min_image_rn(__dsub_rn(R[2][c], R[0][c]), kp.box[c], kp.boxi[c]);
                    rc1[c] = min_image_rn(__dsub_rn(Rc[1][c], Rc[0][c]), kp.box[c], kp.boxi[c]);
                    rc2[c] = min_image_rn(__dsub_rn(Rc[2][c], Rc[0][c]), kp.box[c], kp.boxi[c]);
                }
#pragma unroll
                for (int col = 0; col < 3; col++)
#pragma unroll
                    for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += roh1[c] * dr1[1][col] + roh2[c] * dr1[2][col];
                av[ACC_VIRIALC] += (rc1[0] * dr1[1][0] + rc1[1] * dr1[1][1] + rc1[2] * dr1[1][2]) +
                                   (rc2[0] * dr1[2][0] + rc2[1] * dr1[2][1] + rc2[2] * dr1[2][2]);
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const size_t s = (size_t)b * S + k * N + w;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    kp.dR[3 * s + c] = (k < 3) ? dr1[k][c] : 0.0;
                    kp.dip[3 * s + c] = 0.0;
                    kp.Efdr[3 * s + c] = 0.0;
                }
            }
        } else {
            double q3[3], dq3[3][3][3];
            nasa_dms(R, kp.box, kp.boxi, kp.dms1, kp.dms2, kp.dms3, q3, dq3, FSUM);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                q3[k] *= CHARGECON;
                kp.chg[(size_t)b * kp.natoms + 3 * w + k] = q3[k];
            }
            const double tmp = 0.5 * kp.gammaM / (1.0 - kp.gammaM);
            double q[4];
            q[0] = 0.0;
            q[1] = q3[1] + tmp * (q3[1] + q3[2]);
            q[2] = q3[2] + tmp * (q3[1] + q3[2]);
            q[3] = q3[0] / (1.0 - kp.gammaM);
            double *g = kp.grdq + ((size_t)b * N + w) * 27;
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const double s01 = dq3[a][0][c] * CHARGECON + dq3[a][1][c] * CHARGECON;
                    g[9 * a + 0 + c] = dq3[a][0][c] * CHARGECON + tmp * s01;
                    g[9 * a + 3 + c] = dq3[a][1][c] * CHARGECON + tmp * s01;
                    g[9 * a + 6 + c] = dq3[a][2][c] * CHARGECON - 2.0 * tmp * s01;
                }
            // self energy and intramolecular exclusions (pot_ttm.f90:232-261)
            double Ef[4][3], ph[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                ph[k] = (k == 0) ? 0.0 : -kp.ew.aewald * TSP * q[k];
                Ef[k][0] = Ef[k][1] = Ef[k][2] = 0.0;
            }
            if (FSUM && MODEL == 3) {
                // the mixed engine, TTM3-F: the six exclusion pairs in FP32 from the sites' offsets
                // to their O site (a molecule spans far less than half a box, so a pair's minimum
                // image is the difference of the two offsets); sums converted once
                float rel[4][3], relc[4][3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    rel[0][c] = relc[0][c] = 0.f;
                    rel[1][c] = (float)oh[0][c];
                    rel[2][c] = (float)oh[1][c];
                    rel[3][c] = (float)__dsub_rn(R[3][c], R[0][c]);
                    relc[1][c] = (float)ohc[0][c];
                    relc[2][c] = (float)ohc[1][c];
                    relc[3][c] = (float)__dsub_rn(Rc[3][c], Rc[0][c]);
                }
                const float qf[4] = {(float)q[0], (float)q[1], (float)q[2], (float)q[3]};
                float phf[4] = {0.f, 0.f, 0.f, 0.f}, Eff[4][3], vcf = 0.f, vtf[9];
#pragma unroll
                for (int k = 0; k < 4; k++) Eff[k][0] = Eff[k][1] = Eff[k][2] = 0.f;
#pragma unroll
                for (int k = 0; k < 9; k++) vtf[k] = 0.f;
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = i + 1; j < 4; j++) {
                        const float Rs[3] = {rel[i][0] - rel[j][0], rel[i][1] - rel[j][1], rel[i][2] - rel[j][2]};
                        const float Rcs[3] = {relc[i][0] - relc[j][0], relc[i][1] - relc[j][1], relc[i][2] - relc[j][2]};
                        float ts0, ts1;
                        self1f(Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2], kp.ewf, &ts0, &ts1);
                        phf[i] += ts0 * qf[j];
                        phf[j] += ts0 * qf[i];
                        float d[3];
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            Eff[i][c] += ts1 * qf[j] * Rs[c];
                            Eff[j][c] -= ts1 * qf[i] * Rs[c];
                            d[c] = -ts1 * qf[i] * qf[j] * Rs[c];
                        }
                        vcf += Rcs[0] * d[0] + Rcs[1] * d[1] + Rcs[2] * d[2];
#pragma unroll
                        for (int col = 0; col < 3; col++)
#pragma unroll
                            for (int c = 0; c < 3; c++) vtf[c + 3 * col] += d[col] * Rs[c];
                    }
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    ph[k] += (double)phf[k];
#pragma unroll
                    for (int c = 0; c < 3; c++) Ef[k][c] = (double)Eff[k][c];
                }
                av[ACC_VIRIALC] += (double)vcf;
#pragma unroll
                for (int k = 0; k < 9; k++) av[ACC_VIRT + k] += (double)vtf[k];
            } else
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = i + 1; j < 4; j++) {
                    double Rs[3], Rcs[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        Rs[c] = min_image_rn(__dsub_rn(R[i][c], R[j][c]), kp.box[c], kp.boxi[c]);
                        Rcs[c] = min_image_rn(__dsub_rn(Rc[i][c], Rc[j][c]), kp.box[c], kp.boxi[c]);
                    }
                    // FP64 (TTM2.1-F's polarisable H sites take the exclusion field into the
                    // dipoles, so its mixed engine keeps these in FP64 as well)
                    double ts0, ts1;
                    self1(dot3_rn(Rs[0], Rs[1], Rs[2]), kp.ew, &ts0, &ts1);
                    ph[i] += ts0 * q[j];
                    ph[j] += ts0 * q[i];
                    double d[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        Ef[i][c] += ts1 * q[j] * Rs[c];
                        Ef[j][c] -= ts1 * q[i] * Rs[c];
                        d[c] = -ts1 * q[i] * q[j] * Rs[c];
                    }
                    av[ACC_VIRIALC] += Rcs[0] * d[0] + Rcs[1] * d[1] + Rcs[2] * d[2];
#pragma unroll
                    for (int col = 0; col < 3; col++)
#pragma unroll
                        for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += d[col] * Rs[c];
                }
            // TTM2.1-F intramolecular dipole tensors (pot_ttm.f90:344-365), cached per molecule
            if (MODEL == 2) {
                int t = 0;
#pragma unroll
                for (int i = 0; i < 2; i++)
#pragma unroll
                    for (int j = i + 1; j < 3; j++, t++) {
                        double Rs[3];
#pragma unroll
                        for (int c = 0; c < 3; c++) Rs[c] = min_image_rn(__dsub_rn(R[i][c], R[j][c]), kp.box[c], kp.boxi[c]);
                        double t1, t2;
                        smear2<double>(dot3_rn(Rs[0], Rs[1], Rs[2]), kp.pt.apol_dd[i + 1][j + 1], kp.ew, &t1, &t2);
                        double *T = kp.Tself + (((size_t)b * N + w) * 3 + t) * 6;
                        T[0] = 3.0 * t2 * Rs[0] * Rs[0] - t1;
                        T[1] = 3.0 * t2 * Rs[1] * Rs[1] - t1;
                        T[2] = 3.0 * t2 * Rs[2] * Rs[2] - t1;
                        T[3] = 3.0 * t2 * Rs[0] * Rs[1];
                        T[4] = 3.0 * t2 * Rs[0] * Rs[2];
                        T[5] = 3.0 * t2 * Rs[1] * Rs[2];
                    }
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const size_t s = (size_t)b * S + k * N + w;
                kp.pos[s] = make_double4_32a(R[k][0], R[k][1], R[k][2], q[k]);
                if (first_bead) kp.posc[(size_t)rep * S + k * N + w] = make_double4_32a(Rc[k][0], Rc[k][1], Rc[k][2], 0.0);
                kp.F[s] = make_double4_32a(Ef[k][0], Ef[k][1], Ef[k][2], ph[k]);
            }
        }
    }
    block_reduce_add<14, SITES_NT>(av, kp.acc + (size_t)b * NACC);
}

// ---------------------------------------------------------------------------------------
// ---------------------------------------------------------------------------------------
// pot_ttm.f90:159-228: O-O van der Waals and the charge-charge real-space sum (screened
// Coulomb with Thole smearing below 5 A) over all site pairs of each neighbour pair. Also
// caches the dipole-dipole tensors of the induced-dipole iterations (pot_ttm.f90:311-342).
template <int MODEL>
__global__ void __launch_bounds__(128) k_pair_qq(KP kp) {
    using T = TT<MODEL>;
    const int b = blockIdx.y, N = kp.N;
    const int np = kp.npair[b];
    const double4_32a *pos = kp.pos + (size_t)b * kp.S;
    double av[14];
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int2 ij = kp.pairs[(size_t)b * kp.cap + p];
        const int i = ij.x, j = ij.y;
        double4_32a si[5], sj[5], ci[5], cj[5];
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            si[k] = pos[(k - 1) * N + i];
            sj[k] = pos[(k - 1) * N + j];
            ci[k] = posc_of(kp, b)[(k - 1) * N + i];
            cj[k] = posc_of(kp, b)[(k - 1) * N + j];
        }
        double Rij[3];
        Rij[0] = min_image_rn(__dsub_rn(si[1].x, sj[1].x), kp.box[0], kp.boxi[0]);
        Rij[1] = min_image_rn(__dsub_rn(si[1].y, sj[1].y), kp.box[1], kp.boxi[1]);
        Rij[2] = min_image_rn(__dsub_rn(si[1].z, sj[1].z), kp.box[2], kp.boxi[2]);
        const double dRsq = dot3_rn(Rij[0], Rij[1], Rij[2]);
        {  // van der Waals (pot_ttm.f90:168-190)
            const double dRij = sqrt(dRsq);
            const double R2i = 1.0 / dRsq, R4i = R2i * R2i, R6i = R2i * R2i * R2i, R8i = R6i * R2i;
            const double tv = kp.vdwD * exp(-kp.vdwE * dRij);
            av[ACC_UVDW] += R6i * ((kp.vdwA * R6i + kp.vdwB * R4i) + kp.vdwC) + tv;
            const double xr = dRij - kp.rc1;
            const double sc = R8i * 6.0 * kp.vdwC + tv * kp.vdwE / dRij + kp.shiftA * (xr * xr) + kp.shiftB * (xr * xr * xr);
            double d[3], Rc[3];
            const double xyz_i[3] = {ci[1].x, ci[1].y, ci[1].z}, xyz_j[3] = {cj[1].x, cj[1].y, cj[1].z};
#pragma unroll
            for (int c = 0; c < 3; c++) {
                d[c] = -(sc * Rij[c]);
                Rc[c] = min_image_rn(__dsub_rn(xyz_i[c], xyz_j[c]), kp.box[c], kp.boxi[c]);
            }
            double *dRi = kp.dR + 3 * ((size_t)b * kp.S + i), *dRj = kp.dR + 3 * ((size_t)b * kp.S + j);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                atomicAdd(dRi + c, d[c]);
                atomicAdd(dRj + c, -d[c]);
            }
            av[ACC_VIRIALC] += Rc[0] * d[0] + Rc[1] * d[1] + Rc[2] * d[2];
#pragma unroll
            for (int col = 0; col < 3; col++)
#pragma unroll
                for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += d[col] * Rij[c];
        }
        const double Rij0[3] = {__dadd_rn(__dsub_rn(Rij[0], si[1].x), sj[1].x),
                                __dadd_rn(__dsub_rn(Rij[1], si[1].y), sj[1].y),
                                __dadd_rn(__dsub_rn(Rij[2], si[1].z), sj[1].z)};
        double Fi[5][4], Fj[5][4];
#pragma unroll
        for (int k = 0; k < 5; k++)
#pragma unroll
            for (int c = 0; c < 4; c++) Fi[k][c] = Fj[k][c] = 0.0;
        unsigned err = 0;
#pragma unroll
        for (int isp = 1; isp <= 4; isp++) {
#pragma unroll
            for (int jsp = 1; jsp <= 4; jsp++) {
                if (!T::qq_active(isp, jsp)) continue;
                const double Rs[3] = {
                    min_image_rn(__dsub_rn(__dadd_rn(si[isp].x, Rij0[0]), sj[jsp].x), kp.box[0], kp.boxi[0]),
                    min_image_rn(__dsub_rn(__dadd_rn(si[isp].y, Rij0[1]), sj[jsp].y), kp.box[1], kp.boxi[1]),
                    min_image_rn(__dsub_rn(__dadd_rn(si[isp].z, Rij0[2]), sj[jsp].z), kp.box[2], kp.boxi[2])};
                const double d2 = dot3_rn(Rs[0], Rs[1], Rs[2]);
                double ts0, ts1;
                smear01<double>(d2, kp.pt.apol_qq[isp][jsp], kp.pt.ra_qq[isp][jsp], kp.ew, &ts0, &ts1, &err);
                const double qi = si[isp].w, qj = sj[jsp].w;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    Fi[isp][c] += ts1 * qj * Rs[c];
                    Fj[jsp][c] -= ts1 * qi * Rs[c];
                }
                Fi[isp][3] += ts0 * qj;
                Fj[jsp][3] += ts0 * qi;
                if (T::chg(isp) && T::chg(jsp)) {
                    double d[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) d[c] = -ts1 * qi * qj * Rs[c];
                    const double Rc[3] = {ci[isp].x - cj[jsp].x + Rij0[0], ci[isp].y - cj[jsp].y + Rij0[1],
                                          ci[isp].z - cj[jsp].z + Rij0[2]};
                    av[ACC_VIRIALC] += Rc[0] * d[0] + Rc[1] * d[1] + Rc[2] * d[2];
#pragma unroll
                    for (int col = 0; col < 3; col++)
#pragma unroll
                        for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += d[col] * Rs[c];
                }
            }
        }
        // dipole tensors with the wrapped Rij0 of the iteration loop (pot_ttm.f90:318-319)
        const double Rw[3] = {min_image_rn(Rij0[0], kp.box[0], kp.boxi[0]), min_image_rn(Rij0[1], kp.box[1], kp.boxi[1]),
                              min_image_rn(Rij0[2], kp.box[2], kp.boxi[2])};
        double *Tp = kp.Tdd + ((size_t)b * kp.cap + p) * kp.ndd * 6;
        int t = 0;
#pragma unroll
        for (int isp = T::FDI; isp <= T::LDI; isp++)
#pragma unroll
            for (int jsp = T::FDI; jsp <= T::LDI; jsp++, t++) {
                const double Rs[3] = {
                    min_image_rn(__dsub_rn(__dadd_rn(si[isp].x, Rw[0]), sj[jsp].x), kp.box[0], kp.boxi[0]),
                    min_image_rn(__dsub_rn(__dadd_rn(si[isp].y, Rw[1]), sj[jsp].y), kp.box[1], kp.boxi[1]),
                    min_image_rn(__dsub_rn(__dadd_rn(si[isp].z, Rw[2]), sj[jsp].z), kp.box[2], kp.boxi[2])};
                double t1, t2;
                smear2<double>(dot3_rn(Rs[0], Rs[1], Rs[2]), kp.pt.apol_dd[isp][jsp], kp.ew, &t1, &t2);
                const double t3 = 3.0 * t2;
                Tp[6 * t + 0] = t3 * Rs[0] * Rs[0] - t1;
                Tp[6 * t + 1] = t3 * Rs[1] * Rs[1] - t1;
                Tp[6 * t + 2] = t3 * Rs[2] * Rs[2] - t1;
                Tp[6 * t + 3] = t3 * Rs[0] * Rs[1];
                Tp[6 * t + 4] = t3 * Rs[0] * Rs[2];
                Tp[6 * t + 5] = t3 * Rs[1] * Rs[2];
            }
        if (err) atomicOr(kp.err, err);
        double4_32a *Fb = kp.F + (size_t)b * kp.S;
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            const bool need_i = (MODEL == 2) ? true : (k != 1);
            if (!need_i) continue;
            double *fi = reinterpret_cast<double *>(Fb + (k - 1) * N + i);
            double *fj = reinterpret_cast<double *>(Fb + (k - 1) * N + j);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                atomicAdd(fi + c, Fi[k][c]);
                atomicAdd(fj + c, Fj[k][c]);
            }
            if (k != 1) {
                atomicAdd(fi + 3, Fi[k][3]);
                atomicAdd(fj + 3, Fj[k][3]);
            }
        }
    }
    block_reduce_add<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// ---------------------------------------------------------------------------------------
// pot_ttm.f90:273-297: charge forces -q Efq, Uelec, and the initial induced dipoles
// (polarisability times the charge field, or the 4-step predictor from the history).
// pot_ttm.f90:649-675 calc_dpcf: the 4-step predictor coefficients for MD step t, from the
// history slots mod(t,4) (oldest first in the reference's rotation)
PIMD_D double4_32a predictor_coefficients(int t) {
    switch (t % 4) {
        case 0: return make_double4_32a(-1, 4, -6, 4);
        case 1: return make_double4_32a(4, -1, 4, -6);
        case 2: return make_double4_32a(-6, 4, -1, 4);
        default: return make_double4_32a(4, -6, 4, -1);
    }
}

template <int MODEL>
__global__ void __launch_bounds__(128) k_after_qq(KP kp) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    const int t = kp.dstep[0];
    const bool use_pred = (t > 4) && kp.guess;
    const double4_32a dpcf = predictor_coefficients(t);
    double av[3] = {0.0, 0.0, 0.0};
    if (s < kp.S) {
        const size_t gs = (size_t)b * kp.S + s;
        double4_32a F = kp.F[gs];
        if ((kp.fx_mode & 1) && s >= kp.fx_s0) {  // the reciprocal charge field from its scratch
            const double4_32a x = kp.Fx[gs];
            F.x += x.x;
            F.y += x.y;
            F.z += x.z;
            F.w += x.w;
            kp.F[gs] = F;
        }
        const double q = kp.pos[gs].w;
        if (s >= kp.N) {
            kp.dR[3 * gs + 0] -= q * F.x;
            kp.dR[3 * gs + 1] -= q * F.y;
            kp.dR[3 * gs + 2] -= q * F.z;
            av[2] = q * F.w;
        }
        if (s >= kp.fd && s < kp.ld) {
            const int kind = s / kp.N + 1;
            double mu[3];
            if (use_pred) {
                const double *h = kp.txdip + (size_t)b * 4 * kp.S * 3;
                const size_t st = (size_t)kp.S * 3;
#pragma unroll
                for (int c = 0; c < 3; c++)
                    mu[c] = dpcf.x * h[3 * s + c] + dpcf.y * h[st + 3 * s + c] + dpcf.z * h[2 * st + 3 * s + c] +
                            dpcf.w * h[3 * st + 3 * s + c];
            } else {
                mu[0] = kp.polar[kind] * F.x;
                mu[1] = kp.polar[kind] * F.y;
                mu[2] = kp.polar[kind] * F.z;
            }
            kp.dip[3 * gs + 0] = mu[0];
            kp.dip[3 * gs + 1] = mu[1];
            kp.dip[3 * gs + 2] = mu[2];
            const float4 mf = make_float4((float)mu[0], (float)mu[1], (float)mu[2], 0.f);
            if (kp.dipf) kp.dipf[gs] = mf;
            mrec_dipole(kp, b, s, mf);
        }
    }
    block_reduce_add<3, 128>(av, kp.acc + (size_t)b * NACC);  // slot 2 = ACC_UELEC2
}

// ---------------------------------------------------------------------------------------
// pot_ttm.f90:311-365: real-space dipole field of one iteration from the cached tensors.
template <int MODEL>
__global__ void __launch_bounds__(128) k_dd_real(KP kp) {
    using T = TT<MODEL>;
    const int b = blockIdx.y, N = kp.N;
    if (kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    const int np = kp.npair[b];
    const double *dip = kp.dip + (size_t)b * kp.S * 3;
    double *Ef = kp.Efdr + (size_t)b * kp.S * 3;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int2 ij = kp.pairs[(size_t)b * kp.cap + p];
        const double *Tp = kp.Tdd + ((size_t)b * kp.cap + p) * kp.ndd * 6;
        double ei[5][3], ej[5][3];
#pragma unroll
        for (int k = 0; k < 5; k++) ei[k][0] = ei[k][1] = ei[k][2] = ej[k][0] = ej[k][1] = ej[k][2] = 0.0;
        int t = 0;
#pragma unroll
        for (int isp = T::FDI; isp <= T::LDI; isp++) {
            const double3 mi = ld3(dip + 3 * ((isp - 1) * N + ij.x));
#pragma unroll
            for (int jsp = T::FDI; jsp <= T::LDI; jsp++, t++) {
                const double3 mj = ld3(dip + 3 * ((jsp - 1) * N + ij.y));
                const double *Tt = Tp + 6 * t;
                const double xx = Tt[0], yy = Tt[1], zz = Tt[2], xy = Tt[3], xz = Tt[4], yz = Tt[5];
                ei[isp][0] += xx * mj.x + xy * mj.y + xz * mj.z;
                ei[isp][1] += xy * mj.x + yy * mj.y + yz * mj.z;
                ei[isp][2] += xz * mj.x + yz * mj.y + zz * mj.z;
                ej[jsp][0] += xx * mi.x + xy * mi.y + xz * mi.z;
                ej[jsp][1] += xy * mi.x + yy * mi.y + yz * mi.z;
                ej[jsp][2] += xz * mi.x + yz * mi.y + zz * mi.z;
            }
        }
#pragma unroll
        for (int k = T::FDI; k <= T::LDI; k++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                atomicAdd(Ef + 3 * ((k - 1) * N + ij.x) + c, ei[k][c]);
                atomicAdd(Ef + 3 * ((k - 1) * N + ij.y) + c, ej[k][c]);
            }
    }
    if (MODEL == 2) {  // intramolecular O-H1, O-H2, H1-H2 (pot_ttm.f90:344-365)
        for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < N; w += gridDim.x * blockDim.x) {
            const double *Tw = kp.Tself + ((size_t)b * N + w) * 18;
            double e[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            double3 m[3];
#pragma unroll
            for (int k = 0; k < 3; k++) m[k] = ld3(dip + 3 * (k * N + w));
            int t = 0;
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = i + 1; j < 3; j++, t++) {
                    const double *Tt = Tw + 6 * t;
                    const double xx = Tt[0], yy = Tt[1], zz = Tt[2], xy = Tt[3], xz = Tt[4], yz = Tt[5];
                    e[i][0] += xx * m[j].x + xy * m[j].y + xz * m[j].z;
                    e[i][1] += xy * m[j].x + yy * m[j].y + yz * m[j].z;
                    e[i][2] += xz * m[j].x + yz * m[j].y + zz * m[j].z;
                    e[j][0] += xx * m[i].x + xy * m[i].y + xz * m[i].z;
                    e[j][1] += xy * m[i].x + yy * m[i].y + yz * m[i].z;
                    e[j][2] += xz * m[i].x + yz * m[i].y + zz * m[i].z;
                }
#pragma unroll
            for (int k = 0; k < 3; k++)
#pragma unroll
                for (int c = 0; c < 3; c++) atomicAdd(Ef + 3 * (k * N + w) + c, e[k][c]);
        }
    }
}

__global__ void k_set_step(int *dstep, int t) {
    if (threadIdx.x == 0) {
        dstep[0] = t;
        dstep[1] = 0;
    }
}

// ---------------------------------------------------------------------------------------

// pot_ttm.f90:399-542: real-space forces on charges and dipoles (charge-dipole and
// dipole-dipole), the dipole part of phi, and the intramolecular terms.
template <int MODEL>
__global__ void __launch_bounds__(128) k_pair_force(KP kp) {
    using T = TT<MODEL>;
    const int b = blockIdx.y, N = kp.N;
    const int np = kp.npair[b];
    const double4_32a *pos = kp.pos + (size_t)b * kp.S;
    const double *dip = kp.dip + (size_t)b * kp.S * 3;
    double *dR = kp.dR + (size_t)b * kp.S * 3;
    double4_32a *Fb = kp.F + (size_t)b * kp.S;
    const bool same_a = kp.same_acd != 0;  // |aCCaCD - aDD| < 1e-12 (pot_ttm.f90:443)
    double av[14];
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int2 ij = kp.pairs[(size_t)b * kp.cap + p];
        const int i = ij.x, j = ij.y;
        double4_32a si[5], sj[5];
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            si[k] = pos[(k - 1) * N + i];
            sj[k] = pos[(k - 1) * N + j];
        }
        const double Rij[3] = {min_image_rn(__dsub_rn(si[1].x, sj[1].x), kp.box[0], kp.boxi[0]),
                               min_image_rn(__dsub_rn(si[1].y, sj[1].y), kp.box[1], kp.boxi[1]),
                               min_image_rn(__dsub_rn(si[1].z, sj[1].z), kp.box[2], kp.boxi[2])};
        double Rw[3];
        Rw[0] = min_image_rn(__dadd_rn(__dsub_rn(Rij[0], si[1].x), sj[1].x), kp.box[0], kp.boxi[0]);
        Rw[1] = min_image_rn(__dadd_rn(__dsub_rn(Rij[1], si[1].y), sj[1].y), kp.box[1], kp.boxi[1]);
        Rw[2] = min_image_rn(__dadd_rn(__dsub_rn(Rij[2], si[1].z), sj[1].z), kp.box[2], kp.boxi[2]);
        double gi[5][3], gj[5][3], pi[5], pj[5];
#pragma unroll
        for (int k = 0; k < 5; k++) {
            gi[k][0] = gi[k][1] = gi[k][2] = gj[k][0] = gj[k][1] = gj[k][2] = 0.0;
            pi[k] = pj[k] = 0.0;
        }
#pragma unroll
        for (int isp = 1; isp <= 4; isp++) {
#pragma unroll
            for (int jsp = 1; jsp <= 4; jsp++) {
                if (!T::f_active(isp, jsp)) continue;
                const double Rs[3] = {
                    min_image_rn(__dsub_rn(__dadd_rn(si[isp].x, Rw[0]), sj[jsp].x), kp.box[0], kp.boxi[0]),
                    min_image_rn(__dsub_rn(__dadd_rn(si[isp].y, Rw[1]), sj[jsp].y), kp.box[1], kp.boxi[1]),
                    min_image_rn(__dsub_rn(__dadd_rn(si[isp].z, Rw[2]), sj[jsp].z), kp.box[2], kp.boxi[2])};
                const double d2 = dot3_rn(Rs[0], Rs[1], Rs[2]);
                const double qi = si[isp].w, qj = sj[jsp].w;
                double di[3] = {0, 0, 0}, dj[3] = {0, 0, 0};
                if (T::dip(isp)) {
                    const double3 m = ld3(dip + 3 * ((isp - 1) * N + i));
                    di[0] = m.x, di[1] = m.y, di[2] = m.z;
                }
                if (T::dip(jsp)) {
                    const double3 m = ld3(dip + 3 * ((jsp - 1) * N + j));
                    dj[0] = m.x, dj[1] = m.y, dj[2] = m.z;
                }
                double qd[3];
#pragma unroll
                for (int c = 0; c < 3; c++) qd[c] = qj * di[c] - qi * dj[c];
                const double qd2 = qd[0] * qd[0] + qd[1] * qd[1] + qd[2] * qd[2];
                double dij[3] = {0, 0, 0};
                double ts1 = 0.0, ts2 = 0.0;
                bool have = false;
                if (T::dip(isp) && T::dip(jsp)) {
                    double t1, t2, t3;
                    smear3<double>(d2, kp.pt.apol_dd[isp][jsp], kp.ew, &t1, &t2, &t3);
                    dd_force(Rs, di, dj, t2, t3, dij);
                    if (same_a) {
                        ts1 = t1, ts2 = t2;
                        have = true;
                    }
                }
                if (qd2 > 1.e-9) {
                    if (!have) smear2<double>(d2, kp.pt.apol_cd[isp][jsp], kp.ew, &ts1, &ts2);
                    const double rq = Rs[0] * qd[0] + Rs[1] * qd[1] + Rs[2] * qd[2];
#pragma unroll
                    for (int c = 0; c < 3; c++) dij[c] += 3.0 * ts2 * rq * Rs[c] - ts1 * qd[c];
                    if (isp != 1) pi[isp] += ts1 * (Rs[0] * dj[0] + Rs[1] * dj[1] + Rs[2] * dj[2]);
                    if (jsp != 1) pj[jsp] -= ts1 * (Rs[0] * di[0] + Rs[1] * di[1] + Rs[2] * di[2]);
                }
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    gi[isp][c] += dij[c];
                    gj[jsp][c] -= dij[c];
                }
                const double4_32a ca = posc_of(kp, b)[(isp - 1) * N + i], cb = posc_of(kp, b)[(jsp - 1) * N + j];
                const double Rc[3] = {ca.x - cb.x + Rw[0], ca.y - cb.y + Rw[1], ca.z - cb.z + Rw[2]};
                av[ACC_VIRIALC] += Rc[0] * dij[0] + Rc[1] * dij[1] + Rc[2] * dij[2];
#pragma unroll
                for (int col = 0; col < 3; col++)
#pragma unroll
                    for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += dij[c] * Rs[col];
            }
        }
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            const bool any = (MODEL == 2) || k != 1;
            if (!any) continue;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                atomicAdd(dR + 3 * ((k - 1) * N + i) + c, gi[k][c]);
                atomicAdd(dR + 3 * ((k - 1) * N + j) + c, gj[k][c]);
            }
            if (k != 1) {
                atomicAdd(&Fb[(k - 1) * N + i].w, pi[k]);
                atomicAdd(&Fb[(k - 1) * N + j].w, pj[k]);
            }
        }
    }
    // intramolecular (pot_ttm.f90:482-542), one molecule per thread
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < N; w += gridDim.x * blockDim.x) {
        double4_32a s[5], c4[5];
        double mu[5][3];
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            s[k] = pos[(k - 1) * N + w];
            c4[k] = posc_of(kp, b)[(k - 1) * N + w];
            const double3 m = ld3(dip + 3 * ((k - 1) * N + w));
            mu[k][0] = T::dip(k) ? m.x : 0.0;
            mu[k][1] = T::dip(k) ? m.y : 0.0;
            mu[k][2] = T::dip(k) ? m.z : 0.0;
        }
        double g[5][3], ph[5];
#pragma unroll
        for (int k = 0; k < 5; k++) g[k][0] = g[k][1] = g[k][2] = ph[k] = 0.0;
#pragma unroll
        for (int isp = 1; isp <= 3; isp++)
#pragma unroll
            for (int jsp = isp + 1; jsp <= 4; jsp++) {
                const double Rs[3] = {min_image_rn(__dsub_rn(s[isp].x, s[jsp].x), kp.box[0], kp.boxi[0]),
                                      min_image_rn(__dsub_rn(s[isp].y, s[jsp].y), kp.box[1], kp.boxi[1]),
                                      min_image_rn(__dsub_rn(s[isp].z, s[jsp].z), kp.box[2], kp.boxi[2])};
                const double Rc[3] = {min_image_rn(__dsub_rn(c4[isp].x, c4[jsp].x), kp.box[0], kp.boxi[0]),
                                      min_image_rn(__dsub_rn(c4[isp].y, c4[jsp].y), kp.box[1], kp.boxi[1]),
                                      min_image_rn(__dsub_rn(c4[isp].z, c4[jsp].z), kp.box[2], kp.boxi[2])};
                const double d2 = dot3_rn(Rs[0], Rs[1], Rs[2]);
                double dij[3] = {0, 0, 0};
                if (T::dip(isp) && T::dip(jsp)) {
                    double t1, t2, t3;
                    smear3<double>(d2, kp.pt.apol_dd[isp][jsp], kp.ew, &t1, &t2, &t3);
                    dd_force(Rs, mu[isp], mu[jsp], t2, t3, dij);
                }
                const double qi = s[isp].w, qj = s[jsp].w;
                double qd[3];
#pragma unroll
                for (int c = 0; c < 3; c++) qd[c] = qj * mu[isp][c] - qi * mu[jsp][c];
                double ts1, ts2;
                self2(d2, kp.ew, &ts1, &ts2);
                const double rq = Rs[0] * qd[0] + Rs[1] * qd[1] + Rs[2] * qd[2];
#pragma unroll
                for (int c = 0; c < 3; c++) dij[c] += 3.0 * ts2 * rq * Rs[c] - ts1 * qd[c];
                ph[isp] += ts1 * (Rs[0] * mu[jsp][0] + Rs[1] * mu[jsp][1] + Rs[2] * mu[jsp][2]);
                ph[jsp] -= ts1 * (Rs[0] * mu[isp][0] + Rs[1] * mu[isp][1] + Rs[2] * mu[isp][2]);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    g[isp][c] += dij[c];
                    g[jsp][c] -= dij[c];
                }
                av[ACC_VIRIALC] += Rc[0] * dij[0] + Rc[1] * dij[1] + Rc[2] * dij[2];
#pragma unroll
                for (int col = 0; col < 3; col++)
#pragma unroll
                    for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += dij[c] * Rs[col];
            }
#pragma unroll
        for (int k = 1; k <= 4; k++) {
#pragma unroll
            for (int c = 0; c < 3; c++) atomicAdd(dR + 3 * ((k - 1) * N + w) + c, g[k][c]);
            if (k != 1) atomicAdd(&Fb[(k - 1) * N + w].w, ph[k]);
        }
    }
    block_reduce_add<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// ---------------------------------------------------------------------------------------
// pot_ttm.f90:556-627: charge-derivative forces grdq*phi, their virials, M-site force
// redistribution onto O/H, dipole outputs, and the predictor history (391-392).
template <int MODEL>
__global__ void __launch_bounds__(128) k_finish(KP kp) {
    using T = TT<MODEL>;
    const int w = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    const int N = kp.N;
    double av[14];
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.0;
    if (w < N) {
        const size_t base = (size_t)b * kp.S;
        const double4_32a *pos = kp.pos + base;
        const double4_32a *Fb = kp.F + base;
        double *dR = kp.dR + 3 * base;
        double phH1 = Fb[N + w].w, phH2 = Fb[2 * N + w].w, phM = Fb[3 * N + w].w;
        if (kp.fx_mode & 2) {  // the force pass's sums from its scratch (sites from fx_s0 on)
            const double4_32a *X = kp.Fx + base;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int s = k * N + w;
                if (s < kp.fx_s0) continue;
                const double4_32a x = X[s];
                dR[3 * s + 0] += x.x;
                dR[3 * s + 1] += x.y;
                dR[3 * s + 2] += x.z;
                if (k == 1) phH1 += x.w;
                if (k == 2) phH2 += x.w;
                if (k == 3) phM += x.w;
            }
        }
        const double *g = kp.grdq + ((size_t)b * N + w) * 27;
        double dg[3][3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            dg[1][c] = g[0 + 0 + c] * phH1 + g[0 + 3 + c] * phH2 + g[0 + 6 + c] * phM;
            dg[2][c] = g[9 + 0 + c] * phH1 + g[9 + 3 + c] * phH2 + g[9 + 6 + c] * phM;
            dg[0][c] = g[18 + 0 + c] * phH1 + g[18 + 3 + c] * phH2 + g[18 + 6 + c] * phM;
        }
        const double4_32a O = pos[w], H1 = pos[N + w], H2 = pos[2 * N + w], M = pos[3 * N + w];
        const double4_32a *pc = posc_of(kp, b);
        const double4_32a Oc = pc[w], H1c = pc[N + w], H2c = pc[2 * N + w];
        const double o[3] = {O.x, O.y, O.z}, h1[3] = {H1.x, H1.y, H1.z}, h2[3] = {H2.x, H2.y, H2.z};
        const double m[3] = {M.x, M.y, M.z};
        const double oc[3] = {Oc.x, Oc.y, Oc.z}, h1c[3] = {H1c.x, H1c.y, H1c.z}, h2c[3] = {H2c.x, H2c.y, H2c.z};
        double r1[3], r2[3], rc1[3], rc2[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            r1[c] = min_image_rn(__dsub_rn(h1[c], o[c]), kp.box[c], kp.boxi[c]);
            r2[c] = min_image_rn(__dsub_rn(h2[c], o[c]), kp.box[c], kp.boxi[c]);
            rc1[c] = min_image_rn(__dsub_rn(h1c[c], oc[c]), kp.box[c], kp.boxi[c]);
            rc2[c] = min_image_rn(__dsub_rn(h2c[c], oc[c]), kp.box[c], kp.boxi[c]);
        }
#pragma unroll
        for (int ix = 0; ix < 3; ix++)
#pragma unroll
            for (int iy = 0; iy < 3; iy++) av[ACC_VIRT + ix + 3 * iy] += r1[ix] * dg[1][iy] + r2[ix] * dg[2][iy];
#pragma unroll
        for (int c = 0; c < 3; c++) av[ACC_VIRIALC] += rc1[c] * dg[1][c] + rc2[c] * dg[2][c];
        double gO[3], gH1[3], gH2[3], gM[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            gO[c] = dR[3 * w + c] + dg[0][c];
            gH1[c] = dR[3 * (N + w) + c] + dg[1][c];
            gH2[c] = dR[3 * (2 * N + w) + c] + dg[2][c];
            gM[c] = dR[3 * (3 * N + w) + c];
        }
        double *out = kp.dRRt + ((size_t)b * kp.natoms + 3 * w) * 3;
        const double hg = 0.5 * kp.gammaM;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            out[3 + c] = gH1[c] + hg * gM[c];
            out[6 + c] = gH2[c] + hg * gM[c];
            out[c] = gO[c] + (1.0 - kp.gammaM) * gM[c];
        }
        // dipole outputs (pot_ttm.f90:605-627)
        double dI[3], dE[3] = {0, 0, 0};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const double a = min_image_rn(__dsub_rn(h1[c], m[c]), kp.box[c], kp.boxi[c]);
            const double bb = min_image_rn(__dsub_rn(h2[c], m[c]), kp.box[c], kp.boxi[c]);
            dI[c] = H1.w * a + H2.w * bb;
        }
        const double *dip = kp.dip + 3 * base;
        const int slot = kp.dstep[0] % 4;
        double *hist = kp.txdip + ((size_t)b * 4 + slot) * kp.S * 3;
#pragma unroll
        for (int k = T::FDI; k <= T::LDI; k++) {
            const int s = (k - 1) * N + w;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double mu = dip[3 * s + c];
                dI[c] = mu + dI[c];
                dE[c] = mu;
                if (kp.guess) hist[3 * s + c] = mu;
            }
        }
        double *pI = kp.dipI + ((size_t)b * N + w) * 3, *pE = kp.dipE + ((size_t)b * N + w) * 3;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            pI[c] = dI[c];
            pE[c] = dE[c];
        }
    }
    block_reduce_add<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// pot_ttm.f90:588-591, 628 and force_calc.f90:49: per-bead totals
__global__ void k_totals(KP kp, double *Upott, double *virialt, double *virialct, double *virt9) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= kp.P) return;
    const double *a = kp.acc + (size_t)b * NACC;
    const double En = a[ACC_UMON] + a[ACC_UVDW] + 0.5 * a[ACC_UELEC2] + a[ACC_UIND] + kp.Uvdw_lrc;
    double v[9];
#pragma unroll
    for (int i = 0; i < 9; i++) v[i] = a[ACC_VIRT + i];
    v[0] -= kp.Uvdw_lrc;
    v[4] -= kp.Uvdw_lrc;
    v[8] -= kp.Uvdw_lrc;
    if (Upott) Upott[b] = En;
    if (virialt) virialt[b] = v[0] + v[4] + v[8];
    // pot_spc never sets virialc (its value in the reference is whatever the caller held); 0 here
    if (virialct) virialct[b] = (kp.model >= 4) ? 0.0 : a[ACC_VIRIALC] - 3 * kp.Uvdw_lrc;
    if (virt9)
        for (int i = 0; i < 9; i++) virt9[9 * b + i] = v[i];
}

// ---------------------------------------------------------------------------------------
#define DISPATCH_TTM(E, KERN, GRID, BLOCK, ...)                                              \
    do {                                                                                     \
        if ((E).kp.model == 2)                                                               \
            KERN<2><<<GRID, BLOCK, 0, (E).stream>>>((E).kp, ##__VA_ARGS__);                  \
        else                                                                                 \
            KERN<3><<<GRID, BLOCK, 0, (E).stream>>>((E).kp, ##__VA_ARGS__);                  \
        ++(E).nlaunch;                                                                       \
    } while (0)

static int pair_blocks(const Engine &E) {
    // enough blocks to cover the expected pairs of one bead; the kernels grid-stride
    const long est = (long)E.kp.N * 64;
    long nb = (est + 127) / 128;
    if (nb < 8) nb = 8;
    if (nb > 4096) nb = 4096;
    return (int)nb;
}

void launch_sites(Engine &E) {
    dim3 g((2 * E.kp.N + SITES_NT - 1) / SITES_NT, E.kp.P);
    const bool f = E.precision == PIMD_PREC_MIXED;
    if (E.kp.model == 2) {
        if (f)
            k_sites<2, true><<<g, SITES_NT, 0, E.stream>>>(E.kp);
        else
            k_sites<2, false><<<g, SITES_NT, 0, E.stream>>>(E.kp);
    } else {
        if (f)
            k_sites<3, true><<<g, SITES_NT, 0, E.stream>>>(E.kp);
        else
            k_sites<3, false><<<g, SITES_NT, 0, E.stream>>>(E.kp);
    }
    ++E.nlaunch;
}

void launch_pair_qq(Engine &E) {
    dim3 g(pair_blocks(E), E.kp.P);
    DISPATCH_TTM(E, k_pair_qq, g, 128);
}

void launch_after_qq(Engine &E) {
    dim3 g((E.kp.S + 127) / 128, E.kp.P);
    DISPATCH_TTM(E, k_after_qq, g, 128);
}

void launch_set_step(Engine &E, int t) {
    k_set_step<<<1, 32, 0, E.stream>>>(E.kp.dstep, t);
    ++E.nlaunch;
}

void launch_dd_real(Engine &E) {
    dim3 g(pair_blocks(E), E.kp.P);
    DISPATCH_TTM(E, k_dd_real, g, 128);
}


void launch_pair_force(Engine &E) {
    dim3 g(pair_blocks(E), E.kp.P);
    DISPATCH_TTM(E, k_pair_force, g, 128);
}

void launch_finish(Engine &E) {
    dim3 g((E.kp.N + 127) / 128, E.kp.P);
    DISPATCH_TTM(E, k_finish, g, 128);
}

void launch_totals(Engine &E, double *Upott, double *virialt, double *virialct, double *virt9) {
    k_totals<<<(E.kp.P + 63) / 64, 64, 0, E.stream>>>(E.kp, Upott, virialt, virialct, virt9); ++E.nlaunch;
}

}  // namespace pimd
