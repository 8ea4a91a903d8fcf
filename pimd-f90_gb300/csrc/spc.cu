// spc.cu -- q-SPC/Fw (pot_model 4) and SPC/F (pot_model 5) force call for all beads (FP64).
// Restates pot_ttm/pot_spc.f90:1-277: harmonic (q-SPC/Fw) or Toukan-Rahman (SPC/F)
// monomers, O-O Lennard-Jones, the 3x3 screened-Coulomb site sums of every neighbour
// pair, self and intramolecular exclusion terms, and the Ewald reciprocal sum with its
// virial (ewald.f90:230-291, ewald_pw_std_qq). No induced dipoles, no M site.
//
// Sites per bead are O(0..N-1) H1(N..2N-1) H2(2N..3N-1) with fixed charges. The neighbour
// list and Ewald kernels are the TTM engine's (the Ewald charge sums cover all 3N sites).
// Decomposition: one thread per (molecule, bead) for monomer/self work and the epilogue,
// one thread per O-O pair for the real-space sums (registers, then FP64 atomics per site).
#include "engine.h"

namespace pimd {

// r - box*anint(r/box): pot_spc.f90 divides by the box in its intramolecular, self and
// dipole terms (pot_spc.f90:74-75, 211, 261, 264) where pot_ttm multiplies by 1/box.
PIMD_D double min_image_div_rn(double r, double box) {
    return __dsub_rn(r, __dmul_rn(box, round(__ddiv_rn(r, box))));
}

// pot_spc.f90:54-137, 201-233 and 258-267: site layout, monomer energy/gradient and virial,
// self energy, intramolecular Ewald exclusions, charges and molecular dipoles.
template <int MODEL>
__global__ void __launch_bounds__(128) k_sites_spc(KP kp) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    const int N = kp.N;
    double av[14];
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.0;
    if (w < N) {
        const double *RR = kp.RRt + (size_t)b * kp.natoms * 3 + 9 * w;
        double R[3][3];
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int c = 0; c < 3; c++) R[k][c] = RR[3 * k + c];
        const double q[3] = {kp.qO * CHARGECON, kp.qH * CHARGECON, kp.qH * CHARGECON};
        double dr1[3][3];
        double e1;
        if (MODEL == 4) {
            // pot_spc.f90:73-104 harmonic O-H stretches and H-O-H bend
            double roh1[3], roh2[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                roh1[c] = min_image_div_rn(R[1][c] - R[0][c], kp.box[c]);
                roh2[c] = min_image_div_rn(R[2][c] - R[0][c], kp.box[c]);
            }
            const double d1 = sqrt(roh1[0] * roh1[0] + roh1[1] * roh1[1] + roh1[2] * roh1[2]);
            const double d2 = sqrt(roh2[0] * roh2[0] + roh2[1] * roh2[1] + roh2[2] * roh2[2]);
            const double ax = roh1[1] * roh2[2] - roh1[2] * roh2[1];
            const double ay = -roh1[0] * roh2[2] + roh1[2] * roh2[0];
            const double az = roh1[0] * roh2[1] - roh1[1] * roh2[0];
            const double dAxB = sqrt(ax * ax + ay * ay + az * az);
            const double costh = (roh1[0] * roh2[0] + roh1[1] * roh2[1] + roh1[2] * roh2[2]) / (d1 * d2);
            const double sinth = dAxB / (d1 * d2);
            const double ang = atan2(sinth, costh);
            e1 = kp.harmkb * ((d1 - kp.roh0) * (d1 - kp.roh0) + (d2 - kp.roh0) * (d2 - kp.roh0)) +
                 kp.harmka * ((ang - kp.th0) * (ang - kp.th0));
            const double t1 = 2.0 * kp.harmkb * (d1 - kp.roh0) / d1;
            const double t2 = 2.0 * kp.harmkb * (d2 - kp.roh0) / d2;
            const double ta = 2.0 * kp.harmka * (ang - kp.th0);
            double dh1[3], dh2[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double A1 = -(roh2[c] / (d1 * d2) - costh * roh1[c] / (d1 * d1)) / sinth;
                const double A2 = -(roh1[c] / (d1 * d2) - costh * roh2[c] / (d2 * d2)) / sinth;
                dh1[c] = t1 * roh1[c] + ta * A1;
                dh2[c] = t2 * roh2[c] + ta * A2;
                dr1[1][c] = dh1[c];
                dr1[2][c] = dh2[c];
                dr1[0][c] = -dh1[c] - dh2[c];
            }
#pragma unroll
            for (int iy = 0; iy < 3; iy++)
#pragma unroll
                for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * iy] += roh1[c] * dh1[iy] + roh2[c] * dh2[iy];
        } else {
            // pot_spc.f90:107-137 SPC/F (Toukan-Rahman) stretch-bend polynomial
            const double Ap = 671.288262912, Bp = 164.376, Cp = -211.536, Dp = 111.744;
            const double rhh0 = 2.0 * sin(0.5 * kp.th0) * kp.roh0;
            double roh1[3], roh2[3], rhh[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                roh1[c] = min_image_div_rn(R[0][c] - R[1][c], kp.box[c]);
                roh2[c] = min_image_div_rn(R[0][c] - R[2][c], kp.box[c]);
                rhh[c] = min_image_div_rn(R[1][c] - R[2][c], kp.box[c]);
            }
            const double d1 = sqrt(roh1[0] * roh1[0] + roh1[1] * roh1[1] + roh1[2] * roh1[2]);
            const double d2 = sqrt(roh2[0] * roh2[0] + roh2[1] * roh2[1] + roh2[2] * roh2[2]);
            const double d3 = sqrt(rhh[0] * rhh[0] + rhh[1] * rhh[1] + rhh[2] * rhh[2]);
            const double x1 = d1 - kp.roh0, x2 = d2 - kp.roh0, x3 = d3 - rhh0;
            e1 = Ap * (x1 * x1 + x2 * x2) + Bp * x3 * x3 + Cp * (x1 + x2) * x3 + Dp * x1 * x2;
            const double g1 = 2.0 * Ap * x1 + Cp * x3 + Dp * x2;
            const double g2 = 2.0 * Ap * x2 + Cp * x3 + Dp * x1;
            const double g3 = 2.0 * Bp * x3 + Cp * (x1 + x2);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                dr1[0][c] = g1 * roh1[c] / d1 + g2 * roh2[c] / d2;
                dr1[1][c] = -g1 * roh1[c] / d1 + g3 * rhh[c] / d3;
                dr1[2][c] = -g2 * roh2[c] / d2 - g3 * rhh[c] / d3;
            }
#pragma unroll
            for (int iy = 0; iy < 3; iy++)
#pragma unroll
                for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * iy] -= roh1[c] * dr1[1][iy] + roh2[c] * dr1[2][iy];
        }
        av[ACC_UMON] = e1;
        // pot_spc.f90:201-233 self energy and the three intramolecular exclusions
        double Ef[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, ph[3];
#pragma unroll
        for (int k = 0; k < 3; k++) ph[k] = -kp.ew.aewald * TSP * q[k];
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = i + 1; j < 3; j++) {
                double Rs[3];
#pragma unroll
                for (int c = 0; c < 3; c++) Rs[c] = min_image_div_rn(R[i][c] - R[j][c], kp.box[c]);
                const double drsq = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                const double dd = sqrt(drsq);
                const double expon = exp(-(kp.ew.a2 * drsq));
                const double kr0 = erfc_as<double>(kp.ew.aewald * dd) / dd;
                const double kr1 = (kr0 + kp.ew.cts1 * expon) / drsq;
                const double ch0 = -1.0 / dd;
                const double ch1 = ch0 / drsq;
                const double ts0 = ch0 + kr0, ts1 = ch1 + kr1;
                ph[i] += ts0 * q[j];
                ph[j] += ts0 * q[i];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    Ef[i][c] += ts1 * q[j] * Rs[c];
                    Ef[j][c] -= ts1 * q[i] * Rs[c];
                }
#pragma unroll
                for (int col = 0; col < 3; col++)
#pragma unroll
                    for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += (-ts1 * q[i] * q[j] * Rs[col]) * Rs[c];
            }
        // pot_spc.f90:258-267 molecular dipoles from the O-H vectors
        double dI[3];
#pragma unroll
        for (int c = 0; c < 3; c++)
            dI[c] = q[1] * min_image_div_rn(R[1][c] - R[0][c], kp.box[c]) + q[2] * min_image_div_rn(R[2][c] - R[0][c], kp.box[c]);
        double *pI = kp.dipI + ((size_t)b * N + w) * 3, *pE = kp.dipE + ((size_t)b * N + w) * 3;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            pI[c] = dI[c];
            pE[c] = 0.0;  // pot_spc has no induced dipoles (Edip_mom is not written)
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const size_t s = (size_t)b * kp.S + k * N + w;
            kp.pos[s] = make_double4_32a(R[k][0], R[k][1], R[k][2], q[k]);
            kp.F[s] = make_double4_32a(Ef[k][0], Ef[k][1], Ef[k][2], ph[k]);
            kp.chg[(size_t)b * kp.natoms + 3 * w + k] = q[k];
#pragma unroll
            for (int c = 0; c < 3; c++) kp.dR[3 * s + c] = dr1[k][c];
        }
    }
    block_reduce_add<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// pot_spc.f90:142-191: O-O Lennard-Jones and the 9 screened charge-charge site pairs of
// every neighbour pair (molecule-based cutoff).
__global__ void __launch_bounds__(128) k_pair_spc(KP kp) {
    const int b = blockIdx.y, N = kp.N;
    const int np = kp.npair[b];
    const double4_32a *pos = kp.pos + (size_t)b * kp.S;
    double4_32a *Fb = kp.F + (size_t)b * kp.S;
    double *dRb = kp.dR + (size_t)b * kp.S * 3;
    double av[14];
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int2 ij = kp.pairs[(size_t)b * kp.cap + p];
        const int i = ij.x, j = ij.y;
        double4_32a si[3], sj[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            si[k] = pos[k * N + i];
            sj[k] = pos[k * N + j];
        }
        // find_neigh.f90:76-109: the O-O separation and its square as stored in the list
        double Rij[3];
        Rij[0] = min_image_rn(__dsub_rn(si[0].x, sj[0].x), kp.box[0], kp.boxi[0]);
        Rij[1] = min_image_rn(__dsub_rn(si[0].y, sj[0].y), kp.box[1], kp.boxi[1]);
        Rij[2] = min_image_rn(__dsub_rn(si[0].z, sj[0].z), kp.box[2], kp.boxi[2]);
        const double dRsq = dot3_rn(Rij[0], Rij[1], Rij[2]);
        {
            const double R2i = 1.0 / dRsq, R6i = R2i * R2i * R2i, R8i = R6i * R2i;
            av[ACC_UVDW] += R6i * (kp.vdwA * R6i + kp.vdwC);
            const double sc = R8i * (12.0 * kp.vdwA * R6i + 6.0 * kp.vdwC);
            double d[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                d[c] = -sc * Rij[c];
                atomicAdd(dRb + 3 * i + c, d[c]);
                atomicAdd(dRb + 3 * j + c, -d[c]);
            }
#pragma unroll
            for (int col = 0; col < 3; col++)
#pragma unroll
                for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += d[col] * Rij[c];
        }
        const double Rij0[3] = {Rij[0] - si[0].x + sj[0].x, Rij[1] - si[0].y + sj[0].y, Rij[2] - si[0].z + sj[0].z};
        double Fi[3][4], Fj[3][4];
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int c = 0; c < 4; c++) Fi[k][c] = Fj[k][c] = 0.0;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double Ri[3] = {si[a].x + Rij0[0], si[a].y + Rij0[1], si[a].z + Rij0[2]};
            const double qi = si[a].w;
#pragma unroll
            for (int bb = 0; bb < 3; bb++) {
                const double qj = sj[bb].w;
                const double Rs[3] = {min_image_rn(Ri[0] - sj[bb].x, kp.box[0], kp.boxi[0]),
                                      min_image_rn(Ri[1] - sj[bb].y, kp.box[1], kp.boxi[1]),
                                      min_image_rn(Ri[2] - sj[bb].z, kp.box[2], kp.boxi[2])};
                const double drsq = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                const double dd = sqrt(drsq);
                const double expon = exp(-(kp.ew.a2 * drsq));
                const double ts0 = erfc_as<double>(kp.ew.aewald * dd) / dd;
                const double ts1 = (ts0 + kp.ew.cts1 * expon) / drsq;
                Fi[a][3] += ts0 * qj;
                Fj[bb][3] += ts0 * qi;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    Fi[a][c] += ts1 * qj * Rs[c];
                    Fj[bb][c] -= ts1 * qi * Rs[c];
                }
#pragma unroll
                for (int col = 0; col < 3; col++)
#pragma unroll
                    for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += (-ts1 * qi * qj * Rs[col]) * Rs[c];
            }
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            double *fi = reinterpret_cast<double *>(Fb + k * N + i);
            double *fj = reinterpret_cast<double *>(Fb + k * N + j);
#pragma unroll
            for (int c = 0; c < 4; c++) {
                atomicAdd(fi + c, Fi[k][c]);
                atomicAdd(fj + c, Fj[k][c]);
            }
        }
    }
    block_reduce_add<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// pot_spc.f90:245-249, 270-275: Uelec = 1/2 sum q phi, charge forces -q Efq, and the
// gradient in the caller's O H H atom order.
__global__ void __launch_bounds__(128) k_finish_spc(KP kp) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    const int N = kp.N;
    double av[3] = {0.0, 0.0, 0.0};
    if (w < N) {
        double *out = kp.dRRt + ((size_t)b * kp.natoms + 3 * w) * 3;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const size_t s = (size_t)b * kp.S + k * N + w;
            const double4_32a f = kp.F[s];
            const double q = kp.pos[s].w;
            av[2] += q * f.w;
            out[3 * k + 0] = kp.dR[3 * s + 0] - q * f.x;
            out[3 * k + 1] = kp.dR[3 * s + 1] - q * f.y;
            out[3 * k + 2] = kp.dR[3 * s + 2] - q * f.z;
        }
    }
    block_reduce_add<3, 128>(av, kp.acc + (size_t)b * NACC);  // slot 2 = ACC_UELEC2
}

void launch_sites_spc(Engine &E) {
    dim3 g((E.kp.N + 127) / 128, E.kp.P);
    if (E.kp.model == 4)
        k_sites_spc<4><<<g, 128, 0, E.stream>>>(E.kp);
    else
        k_sites_spc<5><<<g, 128, 0, E.stream>>>(E.kp);
    ++E.nlaunch;
}

void launch_pair_spc(Engine &E) {
    long nb = ((long)E.kp.N * 32 + 127) / 128;
    nb = nb < 8 ? 8 : (nb > 4096 ? 4096 : nb);
    dim3 g((unsigned)nb, E.kp.P);
    k_pair_spc<<<g, 128, 0, E.stream>>>(E.kp);
    ++E.nlaunch;
}

void launch_finish_spc(Engine &E) {
    dim3 g((E.kp.N + 127) / 128, E.kp.P);
    k_finish_spc<<<g, 128, 0, E.stream>>>(E.kp);
    ++E.nlaunch;
}

}  // namespace pimd
