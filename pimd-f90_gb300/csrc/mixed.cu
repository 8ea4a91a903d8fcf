// mixed.cu -- mixed-precision real-space kernels of the TTM force call (pot_ttm.f90:159-542).
//
// Site-pair arithmetic (screened/Thole-smeared tensors, vdW, charge-dipole and dipole-dipole
// terms) runs in FP32; energies, virials, fields and gradients are accumulated in FP64.
// Site-pair separations are never formed from absolute FP32 coordinates: each site keeps
// its offset from its own molecule's O (min-imaged in FP64, stored FP32) and each molecule
// pair its O-O minimum-image vector (FP64, the same bits as the neighbour list), so
//   R_s(i) - R_s'(j) = R_OO(ij) + delta_s(i) - delta_s'(j)        (then wrapped in FP32).
// The centroid-virial separations of the reference (raw centroid differences, see
// pot_ttm.f90:217 and :468) are rebuilt the same way from rho_s = Rc_s - R_O (FP64 difference
// stored FP32).
//
// The real-space dipole field of the iterations is a gather over a full neighbour list with
// cached FP32 tensors: deterministic, so the FP64 SOR residual converges below 1e-8 without
// atomic-order noise.
#include "engine.h"

namespace pimd {

template <int MODEL>
struct TM {
    static constexpr int FDI = MODEL == 2 ? 1 : 4;
    static constexpr int LDI = MODEL == 2 ? 3 : 4;
    PIMD_HD static constexpr bool dip(int k) { return k >= FDI && k <= LDI; }
    PIMD_HD static constexpr bool chg(int k) { return k != 1; }
    PIMD_HD static constexpr bool qq_active(int i, int j) {
        return !(i == 1 && j == 1) && (MODEL == 2 || (i != 1 && j != 1));
    }
    PIMD_HD static constexpr bool f_active(int i, int j) {
        return (dip(i) && dip(j)) || (dip(i) && chg(j)) || (chg(i) && dip(j));
    }
};

PIMD_D float wrapf(float v, float L, float Li) { return v - L * rintf(v * Li); }

// ---------------------------------------------------------------------------------------
// per-site offsets: delta = site - own O (min image), rho = centroid site - own bead O (raw)
__global__ void __launch_bounds__(128) k_site_offsets(KP kp) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (s >= kp.S) return;
    const int mol = s % kp.N;
    const size_t gs = (size_t)b * kp.S + s;
    const double4_32a O = kp.pos[(size_t)b * kp.S + mol], R = kp.pos[gs], C = posc_of(kp, b)[s];
    float4 d;
    if (s < kp.N) {
        d = make_float4(0.f, 0.f, 0.f, (float)R.w);
    } else {
        d = make_float4((float)min_image_rn(__dsub_rn(R.x, O.x), kp.box[0], kp.boxi[0]),
                        (float)min_image_rn(__dsub_rn(R.y, O.y), kp.box[1], kp.boxi[1]),
                        (float)min_image_rn(__dsub_rn(R.z, O.z), kp.box[2], kp.boxi[2]), (float)R.w);
    }
    kp.posf[gs] = d;
    kp.rhof[gs] = make_float4((float)(C.x - O.x), (float)(C.y - O.y), (float)(C.z - O.z), 0.f);
}

// ---------------------------------------------------------------------------------------
// pot_ttm.f90:159-228 in FP32 pair arithmetic (vdW + screened/Thole charge-charge)
template <int MODEL>
__global__ void __launch_bounds__(128) k_pair_qq_m(KP kp) {
    using T = TM<MODEL>;
    const int b = blockIdx.y, N = kp.N;
    const int np = kp.npair[b];
    const double4_32a *pos = kp.pos + (size_t)b * kp.S;
    const float4 *pf = kp.posf + (size_t)b * kp.S;
    const float4 *rh = kp.rhof + (size_t)b * kp.S;
    const float L[3] = {(float)kp.box[0], (float)kp.box[1], (float)kp.box[2]};
    const float Li[3] = {(float)kp.boxi[0], (float)kp.boxi[1], (float)kp.boxi[2]};
    const float vA = kp.vdwA, vB = kp.vdwB, vC = kp.vdwC, vD = kp.vdwD, vE = kp.vdwE;
    const float sA = kp.shiftA, sB = kp.shiftB, r1 = kp.rc1;
    float av[14];  // per-thread FP32 partials, reduced in FP64 per warp (block_reduce_add_f)
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.f;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int2 ij = kp.pairs[(size_t)b * kp.cap + p];
        const int i = ij.x, j = ij.y;
        const double4_32a Oi = pos[i], Oj = pos[j];
        float Rf[3];
        Rf[0] = (float)min_image_rn(__dsub_rn(Oi.x, Oj.x), kp.box[0], kp.boxi[0]);
        Rf[1] = (float)min_image_rn(__dsub_rn(Oi.y, Oj.y), kp.box[1], kp.boxi[1]);
        Rf[2] = (float)min_image_rn(__dsub_rn(Oi.z, Oj.z), kp.box[2], kp.boxi[2]);
        float4 di[5], dj[5], ri[5], rj[5];
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            di[k] = pf[(k - 1) * N + i];
            dj[k] = pf[(k - 1) * N + j];
            ri[k] = rh[(k - 1) * N + i];
            rj[k] = rh[(k - 1) * N + j];
        }
        {  // van der Waals, O-O (pot_ttm.f90:168-190)
            const float dRsq = Rf[0] * Rf[0] + Rf[1] * Rf[1] + Rf[2] * Rf[2];
            const float dRij = sqrtf(dRsq);
            const float R2i = 1.f / dRsq, R4i = R2i * R2i, R6i = R4i * R2i, R8i = R6i * R2i;
            const float tv = vD * __expf(-vE * dRij);
            av[ACC_UVDW] += R6i * ((vA * R6i + vB * R4i) + vC) + tv;
            const float xr = dRij - r1;
            const float sc = R8i * 6.f * vC + tv * vE / dRij + sA * (xr * xr) + sB * (xr * xr * xr);
            float d[3];
#pragma unroll
            for (int c = 0; c < 3; c++) d[c] = -sc * Rf[c];
            const double4_32a ci = posc_of(kp, b)[i], cj = posc_of(kp, b)[j];
            const float Rc[3] = {(float)min_image_rn(__dsub_rn(ci.x, cj.x), kp.box[0], kp.boxi[0]),
                                 (float)min_image_rn(__dsub_rn(ci.y, cj.y), kp.box[1], kp.boxi[1]),
                                 (float)min_image_rn(__dsub_rn(ci.z, cj.z), kp.box[2], kp.boxi[2])};
            double *dRi = kp.dR + 3 * ((size_t)b * kp.S + i), *dRj = kp.dR + 3 * ((size_t)b * kp.S + j);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                atomicAdd(dRi + c, (double)d[c]);
                atomicAdd(dRj + c, -(double)d[c]);
            }
            av[ACC_VIRIALC] += Rc[0] * d[0] + Rc[1] * d[1] + Rc[2] * d[2];
#pragma unroll
            for (int col = 0; col < 3; col++)
#pragma unroll
                for (int c = 0; c < 3; c++) av[ACC_VIRT + c + 3 * col] += d[col] * Rf[c];
        }
        float Fi[5][4], Fj[5][4];
#pragma unroll
        for (int k = 0; k < 5; k++)
#pragma unroll
            for (int c = 0; c < 4; c++) Fi[k][c] = Fj[k][c] = 0.f;
        float vt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vc = 0.f;
        unsigned err = 0;
#pragma unroll
        for (int isp = 1; isp <= 4; isp++) {
#pragma unroll
            for (int jsp = 1; jsp <= 4; jsp++) {
                if (!T::qq_active(isp, jsp)) continue;
                const float Rs[3] = {wrapf(Rf[0] + di[isp].x - dj[jsp].x, L[0], Li[0]),
                                     wrapf(Rf[1] + di[isp].y - dj[jsp].y, L[1], Li[1]),
                                     wrapf(Rf[2] + di[isp].z - dj[jsp].z, L[2], Li[2])};
                const float d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                float ts0, ts1;
                smear01<float>(d2, (float)kp.pt.apol_qq[isp][jsp], (float)kp.pt.ra_qq[isp][jsp], kp.ewf, &ts0, &ts1, &err);
                const float qi = di[isp].w, qj = dj[jsp].w;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    Fi[isp][c] += ts1 * qj * Rs[c];
                    Fj[jsp][c] -= ts1 * qi * Rs[c];
                }
                Fi[isp][3] += ts0 * qj;
                Fj[jsp][3] += ts0 * qi;
                if (T::chg(isp) && T::chg(jsp)) {
                    float d[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) d[c] = -ts1 * qi * qj * Rs[c];
                    const float Rc[3] = {Rf[0] + ri[isp].x - rj[jsp].x, Rf[1] + ri[isp].y - rj[jsp].y,
                                         Rf[2] + ri[isp].z - rj[jsp].z};
                    vc += Rc[0] * d[0] + Rc[1] * d[1] + Rc[2] * d[2];
#pragma unroll
                    for (int col = 0; col < 3; col++)
#pragma unroll
                        for (int c = 0; c < 3; c++) vt[c + 3 * col] += d[col] * Rs[c];
                }
            }
        }
        av[ACC_VIRIALC] += vc;
#pragma unroll
        for (int q = 0; q < 9; q++) av[ACC_VIRT + q] += vt[q];
        if (err) atomicOr(kp.err, err);
        double4_32a *Fb = kp.F + (size_t)b * kp.S;
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            if (MODEL != 2 && k == 1) continue;
            double *fi = reinterpret_cast<double *>(Fb + (k - 1) * N + i);
            double *fj = reinterpret_cast<double *>(Fb + (k - 1) * N + j);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                atomicAdd(fi + c, (double)Fi[k][c]);
                atomicAdd(fj + c, (double)Fj[k][c]);
            }
            if (k != 1) {
                atomicAdd(fi + 3, (double)Fi[k][3]);
                atomicAdd(fj + 3, (double)Fj[k][3]);
            }
        }
    }
    block_reduce_add_f<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// FP32 Thole-smeared dipole tensors for every entry (i, j) of the full neighbour list,
// T[t] for the dipole site-kind pairs t = (isp, jsp) (pot_ttm.f90:320-338)
template <int MODEL>
__global__ void __launch_bounds__(128) k_dd_tensors_m(KP kp) {
    using T = TM<MODEL>;
    const int b = blockIdx.y, N = kp.N;
    const int ne = kp.fntot[b];
    const double4_32a *pos = kp.pos + (size_t)b * kp.S;
    const float4 *pf = kp.posf + (size_t)b * kp.S;
    const int2 *fl = reinterpret_cast<const int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    const float L[3] = {(float)kp.box[0], (float)kp.box[1], (float)kp.box[2]};
    const float Li[3] = {(float)kp.boxi[0], (float)kp.boxi[1], (float)kp.boxi[2]};
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const int2 ij = fl[e];
        const double4_32a Oi = pos[ij.x], Oj = pos[ij.y];
        const float Rf[3] = {(float)min_image_rn(__dsub_rn(Oi.x, Oj.x), kp.box[0], kp.boxi[0]),
                             (float)min_image_rn(__dsub_rn(Oi.y, Oj.y), kp.box[1], kp.boxi[1]),
                             (float)min_image_rn(__dsub_rn(Oi.z, Oj.z), kp.box[2], kp.boxi[2])};
        float *Te = kp.Tf + ((size_t)b * kp.fcap + e) * kp.ndd * 6;
        int t = 0;
#pragma unroll
        for (int isp = T::FDI; isp <= T::LDI; isp++) {
            const float4 a = pf[(isp - 1) * N + ij.x];
#pragma unroll
            for (int jsp = T::FDI; jsp <= T::LDI; jsp++, t++) {
                const float4 c = pf[(jsp - 1) * N + ij.y];
                const float Rs[3] = {wrapf(Rf[0] + a.x - c.x, L[0], Li[0]), wrapf(Rf[1] + a.y - c.y, L[1], Li[1]),
                                     wrapf(Rf[2] + a.z - c.z, L[2], Li[2])};
                float t1, t2;
                smear2<float>(Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2], (float)kp.pt.apol_dd[isp][jsp], kp.ewf, &t1, &t2);
                const float t3 = 3.f * t2;
                Te[6 * t + 0] = t3 * Rs[0] * Rs[0] - t1;
                Te[6 * t + 1] = t3 * Rs[1] * Rs[1] - t1;
                Te[6 * t + 2] = t3 * Rs[2] * Rs[2] - t1;
                Te[6 * t + 3] = t3 * Rs[0] * Rs[1];
                Te[6 * t + 4] = t3 * Rs[0] * Rs[2];
                Te[6 * t + 5] = t3 * Rs[1] * Rs[2];
            }
        }
    }
}

// real-space dipole field of one iteration: gather over the full list, one warp per
// molecule, lanes striding over its entries, butterfly reduction in a fixed order
// (deterministic); writes Efdr (pot_ttm.f90:311-365)
template <int MODEL>
__global__ void __launch_bounds__(128) k_dd_real_m(KP kp) {
    using T = TM<MODEL>;
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, b = blockIdx.y, N = kp.N;
    if (i >= N) return;
    if (kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    const double *dip = kp.dip + (size_t)b * kp.S * 3;
    const float4 *dipf = kp.dipf + (size_t)b * kp.S;
    const int2 *fl = reinterpret_cast<const int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    const int e0 = kp.foff[(size_t)b * N + i];
    const int e1 = (i + 1 < N) ? kp.foff[(size_t)b * N + i + 1] : kp.fntot[b];
    float ei[5][3];
#pragma unroll
    for (int k = 0; k < 5; k++) ei[k][0] = ei[k][1] = ei[k][2] = 0.f;
    for (int e = e0 + lane; e < e1; e += 32) {
        const int j = fl[e].y;
        const float *Te = kp.Tf + ((size_t)b * kp.fcap + e) * kp.ndd * 6;
        int t = 0;
#pragma unroll
        for (int isp = T::FDI; isp <= T::LDI; isp++)
#pragma unroll
            for (int jsp = T::FDI; jsp <= T::LDI; jsp++, t++) {
                const float4 m = dipf[(jsp - 1) * N + j];
                const float mx = m.x, my = m.y, mz = m.z;
                const float *Tt = Te + 6 * t;
                ei[isp][0] += Tt[0] * mx + Tt[3] * my + Tt[4] * mz;
                ei[isp][1] += Tt[3] * mx + Tt[1] * my + Tt[5] * mz;
                ei[isp][2] += Tt[4] * mx + Tt[5] * my + Tt[2] * mz;
            }
    }
#pragma unroll
    for (int k = T::FDI; k <= T::LDI; k++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float v = ei[k][c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            ei[k][c] = v;
        }
    if (lane != 0) return;
    if (MODEL == 2) {  // intramolecular O-H1, O-H2, H1-H2 from the FP64 per-molecule cache
        const double *Tw = kp.Tself + ((size_t)b * N + i) * 18;
        int t = 0;
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
            for (int c = a + 1; c < 3; c++, t++) {
                const double *Tt = Tw + 6 * t;
                const double *ma = dip + 3 * (a * N + i), *mc = dip + 3 * (c * N + i);
                ei[a + 1][0] += (float)(Tt[0] * mc[0] + Tt[3] * mc[1] + Tt[4] * mc[2]);
                ei[a + 1][1] += (float)(Tt[3] * mc[0] + Tt[1] * mc[1] + Tt[5] * mc[2]);
                ei[a + 1][2] += (float)(Tt[4] * mc[0] + Tt[5] * mc[1] + Tt[2] * mc[2]);
                ei[c + 1][0] += (float)(Tt[0] * ma[0] + Tt[3] * ma[1] + Tt[4] * ma[2]);
                ei[c + 1][1] += (float)(Tt[3] * ma[0] + Tt[1] * ma[1] + Tt[5] * ma[2]);
                ei[c + 1][2] += (float)(Tt[4] * ma[0] + Tt[5] * ma[1] + Tt[2] * ma[2]);
            }
    }
    double *Ef = kp.Efdr + (size_t)b * kp.S * 3;
#pragma unroll
    for (int k = T::FDI; k <= T::LDI; k++)
#pragma unroll
        for (int c = 0; c < 3; c++) Ef[3 * ((k - 1) * N + i) + c] = (double)ei[k][c];
}

PIMD_D void dd_force_f(const float R[3], const float di[3], const float dj[3], float t2, float t3, float dij[3]) {
    const float rdi = R[0] * di[0] + R[1] * di[1] + R[2] * di[2];
    const float rdj = R[0] * dj[0] + R[1] * dj[1] + R[2] * dj[2];
    const float didj = di[0] * dj[0] + di[1] * dj[1] + di[2] * dj[2];
    const float a = 15.f * t3 * rdi * rdj - 3.f * t2 * didj;
#pragma unroll
    for (int c = 0; c < 3; c++) dij[c] += a * R[c] - 3.f * t2 * (rdi * dj[c] + rdj * di[c]);
}

// pot_ttm.f90:399-542 in FP32 pair arithmetic, FP64 accumulation
template <int MODEL>
__global__ void __launch_bounds__(128) k_pair_force_m(KP kp) {
    using T = TM<MODEL>;
    const int b = blockIdx.y, N = kp.N;
    const int np = kp.npair[b];
    const double4_32a *pos = kp.pos + (size_t)b * kp.S;
    const float4 *pf = kp.posf + (size_t)b * kp.S;
    const float4 *rh = kp.rhof + (size_t)b * kp.S;
    const double *dip = kp.dip + (size_t)b * kp.S * 3;
    double *dR = kp.dR + (size_t)b * kp.S * 3;
    double4_32a *Fb = kp.F + (size_t)b * kp.S;
    const bool same_a = kp.same_acd != 0;
    const float L[3] = {(float)kp.box[0], (float)kp.box[1], (float)kp.box[2]};
    const float Li[3] = {(float)kp.boxi[0], (float)kp.boxi[1], (float)kp.boxi[2]};
    float av[14];  // per-thread FP32 partials, reduced in FP64 per warp (block_reduce_add_f)
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.f;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int2 ij = kp.pairs[(size_t)b * kp.cap + p];
        const int i = ij.x, j = ij.y;
        const double4_32a Oi = pos[i], Oj = pos[j];
        double Rd[3], Cd[3];
        Rd[0] = min_image_rn(__dsub_rn(Oi.x, Oj.x), kp.box[0], kp.boxi[0]);
        Rd[1] = min_image_rn(__dsub_rn(Oi.y, Oj.y), kp.box[1], kp.boxi[1]);
        Rd[2] = min_image_rn(__dsub_rn(Oi.z, Oj.z), kp.box[2], kp.boxi[2]);
        // raw O-O difference plus the wrapped Rij0 of pot_ttm.f90:406-407 (centroid virial)
        const double Raw[3] = {Oi.x - Oj.x, Oi.y - Oj.y, Oi.z - Oj.z};
#pragma unroll
        for (int c = 0; c < 3; c++) Cd[c] = Raw[c] + min_image_rn(Rd[c] - Raw[c], kp.box[c], kp.boxi[c]);
        const float Rf[3] = {(float)Rd[0], (float)Rd[1], (float)Rd[2]};
        const float Cf[3] = {(float)Cd[0], (float)Cd[1], (float)Cd[2]};
        float gi[5][3], gj[5][3], pi[5], pj[5];
#pragma unroll
        for (int k = 0; k < 5; k++) {
            gi[k][0] = gi[k][1] = gi[k][2] = gj[k][0] = gj[k][1] = gj[k][2] = 0.f;
            pi[k] = pj[k] = 0.f;
        }
        float vt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vc = 0.f;
#pragma unroll
        for (int isp = 1; isp <= 4; isp++) {
#pragma unroll
            for (int jsp = 1; jsp <= 4; jsp++) {
                if (!T::f_active(isp, jsp)) continue;
                const float4 a = pf[(isp - 1) * N + i], c4 = pf[(jsp - 1) * N + j];
                const float Rs[3] = {wrapf(Rf[0] + a.x - c4.x, L[0], Li[0]), wrapf(Rf[1] + a.y - c4.y, L[1], Li[1]),
                                     wrapf(Rf[2] + a.z - c4.z, L[2], Li[2])};
                const float d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                const float qi = a.w, qj = c4.w;
                float di[3] = {0, 0, 0}, dj[3] = {0, 0, 0};
                if (T::dip(isp)) {
                    const double *m = dip + 3 * ((isp - 1) * N + i);
                    di[0] = (float)m[0], di[1] = (float)m[1], di[2] = (float)m[2];
                }
                if (T::dip(jsp)) {
                    const double *m = dip + 3 * ((jsp - 1) * N + j);
                    dj[0] = (float)m[0], dj[1] = (float)m[1], dj[2] = (float)m[2];
                }
                float qd[3];
#pragma unroll
                for (int c = 0; c < 3; c++) qd[c] = qj * di[c] - qi * dj[c];
                const float qd2 = qd[0] * qd[0] + qd[1] * qd[1] + qd[2] * qd[2];
                float dij[3] = {0, 0, 0};
                float ts1 = 0.f, ts2 = 0.f;
                bool have = false;
                if (T::dip(isp) && T::dip(jsp)) {
                    float t1, t2, t3;
                    smear3<float>(d2, (float)kp.pt.apol_dd[isp][jsp], kp.ewf, &t1, &t2, &t3);
                    dd_force_f(Rs, di, dj, t2, t3, dij);
                    if (same_a) {
                        ts1 = t1, ts2 = t2;
                        have = true;
                    }
                }
                if (qd2 > 1.e-9f) {
                    if (!have) smear2<float>(d2, (float)kp.pt.apol_cd[isp][jsp], kp.ewf, &ts1, &ts2);
                    const float rq = Rs[0] * qd[0] + Rs[1] * qd[1] + Rs[2] * qd[2];
#pragma unroll
                    for (int c = 0; c < 3; c++) dij[c] += 3.f * ts2 * rq * Rs[c] - ts1 * qd[c];
                    if (isp != 1) pi[isp] += ts1 * (Rs[0] * dj[0] + Rs[1] * dj[1] + Rs[2] * dj[2]);
                    if (jsp != 1) pj[jsp] -= ts1 * (Rs[0] * di[0] + Rs[1] * di[1] + Rs[2] * di[2]);
                }
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    gi[isp][c] += dij[c];
                    gj[jsp][c] -= dij[c];
                }
                const float4 ra = rh[(isp - 1) * N + i], rb = rh[(jsp - 1) * N + j];
                const float Rc[3] = {Cf[0] + ra.x - rb.x, Cf[1] + ra.y - rb.y, Cf[2] + ra.z - rb.z};
                vc += Rc[0] * dij[0] + Rc[1] * dij[1] + Rc[2] * dij[2];
#pragma unroll
                for (int col = 0; col < 3; col++)
#pragma unroll
                    for (int c = 0; c < 3; c++) vt[c + 3 * col] += dij[c] * Rs[col];
            }
        }
        av[ACC_VIRIALC] += vc;
#pragma unroll
        for (int q = 0; q < 9; q++) av[ACC_VIRT + q] += vt[q];
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            if (MODEL != 2 && k == 1) continue;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                atomicAdd(dR + 3 * ((k - 1) * N + i) + c, (double)gi[k][c]);
                atomicAdd(dR + 3 * ((k - 1) * N + j) + c, (double)gj[k][c]);
            }
            if (k != 1) {
                atomicAdd(&Fb[(k - 1) * N + i].w, (double)pi[k]);
                atomicAdd(&Fb[(k - 1) * N + j].w, (double)pj[k]);
            }
        }
    }
    // intramolecular (pot_ttm.f90:482-542), one molecule per thread
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < N; w += gridDim.x * blockDim.x) {
        float4 s[5], r4[5];
        float mu[5][3];
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            s[k] = pf[(k - 1) * N + w];
            r4[k] = rh[(k - 1) * N + w];
            const double *m = dip + 3 * ((k - 1) * N + w);
            mu[k][0] = T::dip(k) ? (float)m[0] : 0.f;
            mu[k][1] = T::dip(k) ? (float)m[1] : 0.f;
            mu[k][2] = T::dip(k) ? (float)m[2] : 0.f;
        }
        float g[5][3], ph[5];
#pragma unroll
        for (int k = 0; k < 5; k++) g[k][0] = g[k][1] = g[k][2] = ph[k] = 0.f;
        float vt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vc = 0.f;
#pragma unroll
        for (int isp = 1; isp <= 3; isp++)
#pragma unroll
            for (int jsp = isp + 1; jsp <= 4; jsp++) {
                const float Rs[3] = {s[isp].x - s[jsp].x, s[isp].y - s[jsp].y, s[isp].z - s[jsp].z};
                const float Rc[3] = {wrapf(r4[isp].x - r4[jsp].x, L[0], Li[0]), wrapf(r4[isp].y - r4[jsp].y, L[1], Li[1]),
                                     wrapf(r4[isp].z - r4[jsp].z, L[2], Li[2])};
                const float d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                float dij[3] = {0, 0, 0};
                if (T::dip(isp) && T::dip(jsp)) {
                    float t1, t2, t3;
                    smear3<float>(d2, (float)kp.pt.apol_dd[isp][jsp], kp.ewf, &t1, &t2, &t3);
                    dd_force_f(Rs, mu[isp], mu[jsp], t2, t3, dij);
                }
                const float qi = s[isp].w, qj = s[jsp].w;
                float qd[3];
#pragma unroll
                for (int c = 0; c < 3; c++) qd[c] = qj * mu[isp][c] - qi * mu[jsp][c];
                // self2 (smear.f90:133-156) in FP32
                const float dd = sqrtf(d2), drsqi = 1.f / d2, dri = sqrtf(drsqi);
                const float expon = __expf(-(kp.ewf.a2 * d2));
                const float kr0 = erfc_as<float>(kp.ewf.aewald * dd) * dri;
                const float kr1 = (kr0 + kp.ewf.cts1 * expon) * drsqi;
                const float kr2 = (kr1 + kp.ewf.cts2 * expon) * drsqi;
                const float ch1 = -dri * drsqi, ch2 = ch1 * drsqi;
                const float ts1 = kr1 + ch1, ts2 = kr2 + ch2;
                const float rq = Rs[0] * qd[0] + Rs[1] * qd[1] + Rs[2] * qd[2];
#pragma unroll
                for (int c = 0; c < 3; c++) dij[c] += 3.f * ts2 * rq * Rs[c] - ts1 * qd[c];
                ph[isp] += ts1 * (Rs[0] * mu[jsp][0] + Rs[1] * mu[jsp][1] + Rs[2] * mu[jsp][2]);
                ph[jsp] -= ts1 * (Rs[0] * mu[isp][0] + Rs[1] * mu[isp][1] + Rs[2] * mu[isp][2]);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    g[isp][c] += dij[c];
                    g[jsp][c] -= dij[c];
                }
                vc += Rc[0] * dij[0] + Rc[1] * dij[1] + Rc[2] * dij[2];
#pragma unroll
                for (int col = 0; col < 3; col++)
#pragma unroll
                    for (int c = 0; c < 3; c++) vt[c + 3 * col] += dij[c] * Rs[col];
            }
        av[ACC_VIRIALC] += vc;
#pragma unroll
        for (int q = 0; q < 9; q++) av[ACC_VIRT + q] += vt[q];
#pragma unroll
        for (int k = 1; k <= 4; k++) {
#pragma unroll
            for (int c = 0; c < 3; c++) atomicAdd(dR + 3 * ((k - 1) * N + w) + c, (double)g[k][c]);
            if (k != 1) atomicAdd(&Fb[(k - 1) * N + w].w, (double)ph[k]);
        }
    }
    block_reduce_add_f<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// ---------------------------------------------------------------------------------------
#define DISPATCH_M(E, KERN, GRID, BLOCK)                                  \
    do {                                                                  \
        if ((E).kp.model == 2)                                            \
            KERN<2><<<GRID, BLOCK, 0, (E).stream>>>((E).kp);              \
        else                                                              \
            KERN<3><<<GRID, BLOCK, 0, (E).stream>>>((E).kp);              \
        ++(E).nlaunch;                                                    \
    } while (0)

static int pair_blocks_m(const Engine &E, int per_mol) {
    long nb = ((long)E.kp.N * per_mol + 127) / 128;
    if (nb < 8) nb = 8;
    if (nb > 4096) nb = 4096;
    return (int)nb;
}

void launch_site_offsets(Engine &E) {
    dim3 g((E.kp.S + 127) / 128, E.kp.P);
    k_site_offsets<<<g, 128, 0, E.stream>>>(E.kp);
    ++E.nlaunch;
}

void launch_pair_qq_m(Engine &E) {
    dim3 g(pair_blocks_m(E, 64), E.kp.P);
    DISPATCH_M(E, k_pair_qq_m, g, 128);
    dim3 g2(pair_blocks_m(E, 128), E.kp.P);
    DISPATCH_M(E, k_dd_tensors_m, g2, 128);
}

void launch_dd_real_m(Engine &E) {
    dim3 g((E.kp.N * 32 + 127) / 128, E.kp.P);
    DISPATCH_M(E, k_dd_real_m, g, 128);
}

void launch_pair_force_m(Engine &E) {
    dim3 g(pair_blocks_m(E, 64), E.kp.P);
    DISPATCH_M(E, k_pair_force_m, g, 128);
}

}  // namespace pimd
