// mixed.cu -- mixed-precision real-space kernels of the TTM force call (pot_ttm.f90:159-542).
//
// Site-pair arithmetic (screened/Thole-smeared tensors, vdW, charge-dipole and dipole-dipole
// terms) runs in FP32; energies, virials, fields and gradients are accumulated in FP64 per
// molecule or per block. Site-pair separations are never formed from absolute FP32 coordinates:
// each site keeps its offset from its own molecule's O (min-imaged in FP64, stored FP32) and
// each O site its position as 32-bit fractions of the box edges, so that the O-O minimum image
// is one wrapping integer difference per component (exact) and one rounding to FP32:
//   R_s(i) - R_s'(j) = R_OO(ij) + delta_s(i) - delta_s'(j)        (then wrapped in FP32).
// The centroid-virial separations of the reference (raw centroid differences, see
// pot_ttm.f90:217 and :468) are rebuilt the same way from rho_s = Rc_s - R_O (FP64 difference
// stored FP32).
//
// Every pair kernel is a gather over the full neighbour list (a group of lanes per molecule,
// fixed order, one plain FP64 add per output row): deterministic, no FP64 atomics, no FP64
// arithmetic per pair, so the FP64 SOR residual of the dipole iterations converges below 1e-8
// without atomic-order noise. Each unordered pair is evaluated from both ends.
#include <cmath>

#include "engine.h"
#include "dipole_check.cuh"

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

PIMD_D float wrapf(float v, float L, float Li) { return v - L * rint_small(__fmul_rn(v, Li)); }

// ---------------------------------------------------------------------------------------
// Q(2/3, x) of the Thole-smeared charge pairs (smear.f90:2-34 calls math.f90:188-285 with
// x = a r^3) without the iterative series / continued fraction. With u = a^(1/3) r,
//   G(u) = Gamma(2/3) Q(2/3, u^3) = 3 int_u^inf s exp(-s^3) ds,
// and h(u) = G(u) exp(u^3) is smooth on [0, inf) with h(0) = Gamma(2/3), h ~ 1/u for large u,
// and h'(u) = 3u^2 h(u) - 3u. The table holds h as cubic Hermite pieces on a grid of 1/32
// (interpolation error below 1e-8 relative, under FP32 rounding); the kernel forms
// ra g23 Q = ra exp(-a r^3) h(ra r) from the exp(-a r^3) it already has. Beyond u = 4.5
// exp(-u^3) is below the FP32 range and the term vanishes. Values of h come from the same
// series / continued fraction evaluated in FP64 to 1e-16 at engine creation.
constexpr int GQ_PER_UNIT = 32;
constexpr int GQ_N = 144;  // u in [0, 4.5)

static double gq_h_host(double u) {
    const double a = 2.0 / 3.0;
    if (u <= 0.0) return std::tgamma(a);
    const double x = u * u * u;
    if (x < a + 1.0) {  // P(a, x) by its series
        double ap = a, sum = 1.0 / a, del = sum;
        for (int n = 0; n < 2000 && std::fabs(del) > std::fabs(sum) * 1e-17; n++) {
            ap += 1.0;
            del *= x / ap;
            sum += del;
        }
        const double P = sum * std::exp(-x + a * std::log(x) - std::lgamma(a));
        return std::tgamma(a) * (1.0 - P) * std::exp(x);
    }
    // Q(a, x) = exp(-x) x^a cf / Gamma(a) by the modified Lentz continued fraction, so h = x^a cf
    const double tiny = 1e-300;
    double b = x + 1.0 - a, c = 1.0 / tiny, d = 1.0 / b, h = d;
    for (int i = 1; i < 2000; i++) {
        const double an = -i * (i - a);
        b += 2.0;
        d = an * d + b;
        if (std::fabs(d) < tiny) d = tiny;
        c = b + an / c;
        if (std::fabs(c) < tiny) c = tiny;
        d = 1.0 / d;
        const double del = d * c;
        h *= del;
        if (std::fabs(del - 1.0) < 1e-16) break;
    }
    return std::pow(x, a) * h;
}

// FP32 tables and the second stream of the mixed engine
cudaError_t mixed_init(Engine &E) {
    float4 tab[GQ_N];
    const double du = 1.0 / GQ_PER_UNIT;
    for (int k = 0; k < GQ_N; k++) {
        const double u0 = k * du, u1 = (k + 1) * du;
        const double h0 = gq_h_host(u0), h1 = gq_h_host(u1);
        const double d0 = (3.0 * u0 * u0 * h0 - 3.0 * u0) * du, d1 = (3.0 * u1 * u1 * h1 - 3.0 * u1) * du;
        tab[k] = make_float4((float)h0, (float)d0, (float)(3.0 * (h1 - h0) - 2.0 * d0 - d1),
                             (float)(2.0 * (h0 - h1) + d0 + d1));
    }
    cudaError_t e = cudaStreamCreateWithFlags(&E.aux_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E.ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E.ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E.ev_nbr, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&E.loop_aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E.loop_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E.loop_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E.loop_pev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E.loop_jpev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void **)&E.kp.gq23, sizeof(tab));
    if (e == cudaSuccess) E.allocs.push_back(E.kp.gq23);
    if (e == cudaSuccess) e = cudaMemcpy(E.kp.gq23, tab, sizeof(tab), cudaMemcpyHostToDevice);
    return e;
}

// ra g23 Q(2/3, a r^3) = ra exp1 h(ra r), exp1 = exp(-a r^3)
PIMD_D float gq_h(const float4 *tab, float u) {
    const float x = u * (float)GQ_PER_UNIT;
    const int k = min((int)x, GQ_N - 1);
    const float t = fminf(x - (float)k, 1.f);
    const float4 c = __ldg(tab + k);
    return c.x + t * (c.y + t * (c.z + t * c.w));
}

// smear01<float> (smear.f90:2-34) with the tabulated Q(2/3, x)
PIMD_D void smear01_m(float drsq, float a_pol12, float ra, const EwCf &e, const float4 *gq, float *ts0, float *ts1) {
    float dd, dri;
    rinv<float>(drsq, dd, dri);
    const float drsqi = dri * dri;
    const float expon = __expf(-(e.a2 * drsq));
    const float er = erfc_as<float>(e.aewald * dd);
    float t0 = er * dri;
    float t1 = (t0 + e.cts1 * expon) * drsqi;
    if (drsq < 25.f) {
        const float rA3 = dd * drsq * a_pol12;
        const float exp1 = __expf(-rA3);
        const float ch1 = -dri * drsqi;
        const float sr1 = (1.f - exp1) * dri * drsqi;
        t1 = t1 + ch1 + sr1;
        t0 = t0 - exp1 * dri + ra * exp1 * gq_h(gq, ra * dd);
    }
    *ts0 = t0;
    *ts1 = t1;
}

// ---------------------------------------------------------------------------------------
// per-site offsets: delta = site - own O (min image), rho = centroid site - own bead O (raw);
// per molecule the O site as fractions of the box edges in 32-bit fixed point (ofix) and in
// FP32 (orawf, unwrapped)
__global__ void __launch_bounds__(128) k_site_offsets(KP kp) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (s >= kp.S) return;
    const int mol = s % kp.N;
    const size_t gs = (size_t)b * kp.S + s;
    const double4_32a O = kp.pos[(size_t)b * kp.S + mol], R = kp.pos[gs], C = posc_of(kp, b)[s];
    float4 d;
    if (s < kp.N) {
        d = make_float4(0.f, 0.f, 0.f, (float)R.w);
        const double o[3] = {O.x, O.y, O.z};
        unsigned u[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const double t = o[c] * kp.boxi[c];
            // fraction in [0, 1) times 2^32; a round-up to 2^32 wraps to 0, the same point
            u[c] = (unsigned)(unsigned long long)__double2ll_rn((t - floor(t)) * 0x1p32);
        }
        kp.ofix[(size_t)b * kp.N + s] = make_uint4(u[0], u[1], u[2], 0u);
        kp.orawf[(size_t)b * kp.N + s] = make_float4((float)O.x, (float)O.y, (float)O.z, 0.f);
    } else {
        d = make_float4((float)min_image_rn(__dsub_rn(R.x, O.x), kp.box[0], kp.boxi[0]),
                        (float)min_image_rn(__dsub_rn(R.y, O.y), kp.box[1], kp.boxi[1]),
                        (float)min_image_rn(__dsub_rn(R.z, O.z), kp.box[2], kp.boxi[2]), (float)R.w);
        if (kp.mrec && s >= kp.fd && s < kp.ld) {  // the M site in the same fixed point as ofix
            const double r[3] = {R.x, R.y, R.z};
            unsigned u[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double t = r[c] * kp.boxi[c];
                u[c] = (unsigned)(unsigned long long)__double2ll_rn((t - floor(t)) * 0x1p32);
            }
            kp.mrec[2 * ((size_t)b * kp.N + (s - kp.fd))] =
                make_float4(__uint_as_float(u[0]), __uint_as_float(u[1]), __uint_as_float(u[2]), 0.f);
        }
    }
    kp.posf[gs] = d;
    kp.rhof[gs] = make_float4((float)(C.x - O.x), (float)(C.y - O.y), (float)(C.z - O.z), 0.f);
}

// O_i - O_j, minimum image, from the fixed-point sites: the unsigned difference wraps modulo the
// box, read as signed it is the nearest image; one rounding to FP32 (relative 2^-24) and the scale
PIMD_D void oo_min_image(const KP &kp, uint4 oi, uint4 oj, float R[3]) {
    R[0] = (float)(int)(oi.x - oj.x) * kp.boxq[0];
    R[1] = (float)(int)(oi.y - oj.y) * kp.boxq[1];
    R[2] = (float)(int)(oi.z - oj.z) * kp.boxq[2];
}

// sum over the QL lanes of one molecule's group (QL divides 32; every lane of the warp calls it)
template <int QL>
PIMD_D float group_sum(float v) {
#pragma unroll
    for (int o = QL / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// lanes per molecule of the gather kernels (two molecules per warp)
constexpr int QL = 16;

// ---------------------------------------------------------------------------------------
// pot_ttm.f90:159-228 in FP32 pair arithmetic (vdW + screened/Thole charge-charge), as a
// gather over the full neighbour list: QL lanes per molecule i stride over its entries (i, j)
// and accumulate only i's side -- the fields and potentials at i's sites from j's charges and
// i's share of the vdW gradient; j's side is accumulated when j gathers i. Every unordered pair
// is visited twice, so energies and virials are added with weight 1/2. No atomics per entry: the
// group's sums are added once to the F and dR rows k_sites initialised (deterministic).
template <int MODEL>
__global__ void __launch_bounds__(128) k_pair_qq_m(KP kp) {
    using T = TM<MODEL>;
    const int b = blockIdx.y, N = kp.N;
    const int sub = threadIdx.x & (QL - 1);
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) / QL;
    const float4 *pf = kp.posf + (size_t)b * kp.S;
    const float4 *rh = kp.rhof + (size_t)b * kp.S;
    const uint4 *of = kp.ofix + (size_t)b * N;
    const int2 *fl = reinterpret_cast<const int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    const float L[3] = {kp.ptf.box[0], kp.ptf.box[1], kp.ptf.box[2]};
    const float Li[3] = {kp.ptf.boxi[0], kp.ptf.boxi[1], kp.ptf.boxi[2]};
    const float vA = kp.ptf.vdw[0], vB = kp.ptf.vdw[1], vC = kp.ptf.vdw[2], vD = kp.ptf.vdw[3], vE = kp.ptf.vdw[4];
    const float sA = kp.ptf.shiftA, sB = kp.ptf.shiftB, r1 = kp.ptf.rc1;
    float av[14];  // per-lane FP32 partials, reduced in FP64 per warp (block_reduce_add_f)
#pragma unroll
    for (int q = 0; q < 14; q++) av[q] = 0.f;
    float Fi[5][4], gR[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 5; k++)
#pragma unroll
        for (int c = 0; c < 4; c++) Fi[k][c] = 0.f;
    if (i < N) {
        // row bounds clamped to the stored length (offsets run past it when the list overflowed)
        const int ne = kp.fntot[b];
        const int e0 = min(kp.foff[(size_t)b * N + i], ne);
        const int e1 = (i + 1 < N) ? min(kp.foff[(size_t)b * N + i + 1], ne) : ne;
        const uint4 oi = of[i];
        float4 di[5], ri[5];
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            di[k] = pf[(k - 1) * N + i];
            ri[k] = rh[(k - 1) * N + i];
        }
        float vt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vc = 0.f;
        for (int e = e0 + sub; e < e1; e += QL) {
            const int j = fl[e].y;
            float Rf[3];
            oo_min_image(kp, oi, of[j], Rf);
            float4 dj[5], rj[5];
#pragma unroll
            for (int k = 1; k <= 4; k++) {
                dj[k] = pf[(k - 1) * N + j];
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
                for (int c = 0; c < 3; c++) {
                    d[c] = -sc * Rf[c];
                    gR[c] += d[c];
                }
                // centroid O-O minimum image: Rc_i - Rc_j = (O_i - O_j) + rho_i - rho_j
                const float Rc[3] = {wrapf(Rf[0] + ri[1].x - rj[1].x, L[0], Li[0]),
                                     wrapf(Rf[1] + ri[1].y - rj[1].y, L[1], Li[1]),
                                     wrapf(Rf[2] + ri[1].z - rj[1].z, L[2], Li[2])};
                vc += Rc[0] * d[0] + Rc[1] * d[1] + Rc[2] * d[2];
#pragma unroll
                for (int col = 0; col < 3; col++)
#pragma unroll
                    for (int c = 0; c < 3; c++) vt[c + 3 * col] += d[col] * Rf[c];
            }
#pragma unroll
            for (int isp = 1; isp <= 4; isp++) {
#pragma unroll
                for (int jsp = 2; jsp <= 4; jsp++) {  // j's charged sites
                    if (!T::qq_active(isp, jsp)) continue;
                    const float Rs[3] = {wrapf(Rf[0] + di[isp].x - dj[jsp].x, L[0], Li[0]),
                                         wrapf(Rf[1] + di[isp].y - dj[jsp].y, L[1], Li[1]),
                                         wrapf(Rf[2] + di[isp].z - dj[jsp].z, L[2], Li[2])};
                    const float d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                    float ts0, ts1;
                    smear01_m(d2, kp.ptf.apol_qq[isp][jsp], kp.ptf.ra_qq[isp][jsp], kp.ewf, kp.gq23, &ts0, &ts1);
                    const float qj = dj[jsp].w;
#pragma unroll
                    for (int c = 0; c < 3; c++) Fi[isp][c] += ts1 * qj * Rs[c];
                    Fi[isp][3] += ts0 * qj;
                    if (T::chg(isp)) {
                        const float qi = di[isp].w;
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
        }
        av[ACC_VIRIALC] += vc;
#pragma unroll
        for (int q = 0; q < 9; q++) av[ACC_VIRT + q] += vt[q];
    }
    // group sums of i's side (all lanes take part; lanes of i >= N hold zeros)
#pragma unroll
    for (int k = 1; k <= 4; k++)
#pragma unroll
        for (int c = 0; c < 4; c++) Fi[k][c] = group_sum<QL>(Fi[k][c]);
#pragma unroll
    for (int c = 0; c < 3; c++) gR[c] = group_sum<QL>(gR[c]);
    // the FP64 adds spread over the group's lanes, one value each (FP64 is a narrow pipe on this
    // part): lane sub adds component sub % 4 of site sub / 4 + 1, lanes 0-2 the O gradient
    if (i < N) {
        const int k = sub / 4 + 1, c = sub % 4;
        float v = 0.f;
#pragma unroll
        for (int kk = 1; kk <= 4; kk++)
#pragma unroll
            for (int cc = 0; cc < 4; cc++)
                if ((kk - 1) * 4 + cc == sub) v = Fi[kk][cc];
        if (!(MODEL != 2 && k == 1) && !(k == 1 && c == 3)) {
            double *Fd = reinterpret_cast<double *>(kp.F + (size_t)b * kp.S + (size_t)(k - 1) * N + i);
            Fd[c] += (double)v;
        }
        if (sub < 3) kp.dR[3 * ((size_t)b * kp.S + i) + sub] += (double)(sub == 0 ? gR[0] : sub == 1 ? gR[1] : gR[2]);
    }
    // each unordered pair was visited from both ends
#pragma unroll
    for (int q = 0; q < 14; q++) av[q] *= 0.5f;
    block_reduce_add_f<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// FP32 Thole-smeared dipole-tensor scalars for every entry (i, j) of the full neighbour list:
// (t1, 3 t2) of smear2 for the dipole site-kind pairs t = (isp, jsp) (pot_ttm.f90:320-338), and
// the partner j alone in its own array. The iterations rebuild the separation R from the O
// fixed-point sites and the site offsets (the same FP32 operations as here) and form
// T mu = 3 t2 (R . mu) R - t1 mu, so a list entry streams 4 + 8 ndd bytes per iteration instead
// of the 8 + 24 ndd of a stored tensor and (i, j) pair.
template <int MODEL>
__global__ void __launch_bounds__(128) k_dd_tensors_m(KP kp) {
    using T = TM<MODEL>;
    const int b = blockIdx.y, N = kp.N;
    const int ne = kp.fntot[b];
    const uint4 *of = kp.ofix + (size_t)b * N;
    const float4 *pf = kp.posf + (size_t)b * kp.S;
    const int2 *fl = reinterpret_cast<const int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    int *fj = kp.fj + (size_t)b * kp.fcap;
    const float L[3] = {kp.ptf.box[0], kp.ptf.box[1], kp.ptf.box[2]};
    const float Li[3] = {kp.ptf.boxi[0], kp.ptf.boxi[1], kp.ptf.boxi[2]};
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const int2 ij = fl[e];
        fj[e] = ij.y;
        float Rf[3];
        oo_min_image(kp, of[ij.x], of[ij.y], Rf);
        float2 *Te = kp.Tf + ((size_t)b * kp.fcap + e) * kp.ndd;
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
                smear2<float>(Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2], kp.ptf.apol_dd[isp][jsp], kp.ewf, &t1, &t2);
                Te[t] = make_float2(t1, 3.f * t2);
            }
        }
    }
}

// real-space dipole field of one iteration: gather over the full list, one warp per
// molecule, lanes striding over its entries, butterfly reduction in a fixed order
// (deterministic); writes Efdr (pot_ttm.f90:311-365). The separation of each site pair is
// rebuilt from the O fixed-point sites and the site offsets; its smear scalars (t1, 3 t2) come
// from the per-entry cache of k_dd_tensors_m, or, with OTF, from smear2 in the loop (no cache
// stream, more arithmetic; the autotuner tries both).
template <int MODEL, bool OTF>
PIMD_D void dd_real_mol(const KP &kp, int i, int b, int lane) {
    using T = TM<MODEL>;
    const int N = kp.N;
    const double *dip = kp.dip + (size_t)b * kp.S * 3;
    const float4 *dipf = dipf_cur(kp) + (size_t)b * kp.S;
    const int2 *fl = reinterpret_cast<const int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    const int *fj = kp.fj + (size_t)b * kp.fcap;
    const float2 *Tb = kp.Tf + (size_t)b * kp.fcap * kp.ndd;
    const int ne = kp.fntot[b];  // offsets run past the stored length when the list overflowed
    const int e0 = min(kp.foff[(size_t)b * N + i], ne);
    const int e1 = (i + 1 < N) ? min(kp.foff[(size_t)b * N + i + 1], ne) : ne;
    float ei[5][3];
#pragma unroll
    for (int k = 0; k < 5; k++) ei[k][0] = ei[k][1] = ei[k][2] = 0.f;
    const float4 *pf = kp.posf + (size_t)b * kp.S;
    const uint4 *of = kp.ofix + (size_t)b * N;
    const float L[3] = {kp.ptf.box[0], kp.ptf.box[1], kp.ptf.box[2]};
    const float Li[3] = {kp.ptf.boxi[0], kp.ptf.boxi[1], kp.ptf.boxi[2]};
    const uint4 oi = of[i];
    float4 si[5];
#pragma unroll
    for (int k = T::FDI; k <= T::LDI; k++) si[k] = pf[(k - 1) * N + i];
    uint64_t pol = 0;
    if (kp.l2keep) asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    for (int e = e0 + lane; e < e1; e += 32) {
        int j;
        if (OTF)
            j = fl[e].y;
        else if (kp.l2keep)
            asm volatile("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(j) : "l"(fj + e), "l"(pol));
        else
            j = fj[e];
        float Rf[3];
        oo_min_image(kp, oi, of[j], Rf);
        int t = 0;
#pragma unroll
        for (int isp = T::FDI; isp <= T::LDI; isp++)
#pragma unroll
            for (int jsp = T::FDI; jsp <= T::LDI; jsp++, t++) {
                const float4 c = pf[(jsp - 1) * N + j];
                const float4 m = dipf[(jsp - 1) * N + j];
                const float Rs[3] = {wrapf(Rf[0] + si[isp].x - c.x, L[0], Li[0]), wrapf(Rf[1] + si[isp].y - c.y, L[1], Li[1]),
                                     wrapf(Rf[2] + si[isp].z - c.z, L[2], Li[2])};
                float t1, t3;
                if (OTF) {
                    float t2;
                    smear2<float>(Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2], kp.ptf.apol_dd[isp][jsp], kp.ewf, &t1, &t2);
                    t3 = 3.f * t2;
                } else {
                    float2 ts;
                    const float2 *pt = Tb + (size_t)e * kp.ndd + t;
                    if (kp.l2keep)
                        asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
                                     : "=f"(ts.x), "=f"(ts.y)
                                     : "l"(pt), "l"(pol));
                    else
                        ts = *pt;
                    t1 = ts.x;
                    t3 = ts.y;
                }
                const float rm = t3 * (Rs[0] * m.x + Rs[1] * m.y + Rs[2] * m.z);
                ei[isp][0] += rm * Rs[0] - t1 * m.x;
                ei[isp][1] += rm * Rs[1] - t1 * m.y;
                ei[isp][2] += rm * Rs[2] - t1 * m.z;
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
    double *Ef = kp.Efdr + (size_t)b * kp.S * 3;
    if (MODEL != 2) {  // every lane holds the sums: lanes 0-2 store one component each
        if (lane < 3) {
#pragma unroll
            for (int k = T::FDI; k <= T::LDI; k++)
                Ef[3 * ((k - 1) * N + i) + lane] = (double)(lane == 0 ? ei[k][0] : lane == 1 ? ei[k][1] : ei[k][2]);
        }
        return;
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
#pragma unroll
    for (int k = T::FDI; k <= T::LDI; k++)
#pragma unroll
        for (int c = 0; c < 3; c++) Ef[3 * ((k - 1) * N + i) + c] = (double)ei[k][c];
}

// TTM3-F with the molecule records: the M-M separation is the wrapping difference of the M sites'
// fixed-point coordinates (the nearest image, one rounding to FP32), and an entry reads its
// partner's position and dipole in one 32-byte record besides its index and smear scalars (DBUF:
// the dipole from the double-buffered FP32 dipoles instead, for the asynchronous iterations)
template <bool OTF, bool DBUF>
PIMD_D void dd_real_rec(const KP &kp, int i, int b, int lane) {
    const int N = kp.N;
    const float4 *rec = kp.mrec + (size_t)b * N * 2;
    const float4 *dcur = dipf_cur(kp) + (size_t)b * kp.S + kp.fd;
    const int2 *fl = reinterpret_cast<const int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    const int *fj = kp.fj + (size_t)b * kp.fcap;
    const float2 *Tb = kp.Tf + (size_t)b * kp.fcap * kp.ndd;
    const int ne = kp.fntot[b];  // offsets run past the stored length when the list overflowed
    const int e0 = min(kp.foff[(size_t)b * N + i], ne);
    const int e1 = (i + 1 < N) ? min(kp.foff[(size_t)b * N + i + 1], ne) : ne;
    const float4 ri = rec[2 * i];
    const unsigned mi[3] = {__float_as_uint(ri.x), __float_as_uint(ri.y), __float_as_uint(ri.z)};
    float ei[3] = {0.f, 0.f, 0.f};
    uint64_t pol = 0;
    if (kp.l2keep) asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    for (int e = e0 + lane; e < e1; e += 32) {
        int j;
        if (OTF)
            j = fl[e].y;
        else if (kp.l2keep)
            asm volatile("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(j) : "l"(fj + e), "l"(pol));
        else
            j = fj[e];
        const float4 rj = rec[2 * j], m = DBUF ? dcur[j] : rec[2 * j + 1];
        const float R[3] = {(float)(int)(mi[0] - __float_as_uint(rj.x)) * kp.boxq[0],
                            (float)(int)(mi[1] - __float_as_uint(rj.y)) * kp.boxq[1],
                            (float)(int)(mi[2] - __float_as_uint(rj.z)) * kp.boxq[2]};
        float t1, t3;
        if (OTF) {
            float t2;
            smear2<float>(R[0] * R[0] + R[1] * R[1] + R[2] * R[2], kp.ptf.apol_dd[4][4], kp.ewf, &t1, &t2);
            t3 = 3.f * t2;
        } else {
            float2 ts;
            if (kp.l2keep)
                asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(ts.x), "=f"(ts.y) : "l"(Tb + e), "l"(pol));
            else
                ts = Tb[e];
            t1 = ts.x;
            t3 = ts.y;
        }
        const float rm = t3 * (R[0] * m.x + R[1] * m.y + R[2] * m.z);
        ei[0] += rm * R[0] - t1 * m.x;
        ei[1] += rm * R[1] - t1 * m.y;
        ei[2] += rm * R[2] - t1 * m.z;
    }
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ei[c] += __shfl_xor_sync(0xffffffffu, ei[c], o);
    if (lane < 3) kp.Efdr[3 * ((size_t)b * kp.S + kp.fd + i) + lane] = (double)(lane == 0 ? ei[0] : lane == 1 ? ei[1] : ei[2]);
}

// ASYNC (TTM3-F): the block then arrives at the units of its molecules' M sites and runs the
// SOR update of those it completes (dipole_check.cuh); converged beads and molecules past N
// still arrive.
template <int MODEL, bool OTF, bool ASYNC>
__global__ void __launch_bounds__(128) k_dd_real_m(KP kp) {
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, b = blockIdx.y;
    if (i < kp.N && !bead_converged(kp, b)) {
        if (MODEL == 3 && kp.mrec)
            dd_real_rec<OTF, ASYNC>(kp, i, b, lane);
        else
            dd_real_mol<MODEL, OTF>(kp, i, b, lane);
    }
    if constexpr (ASYNC) {
        const int m0 = blockIdx.x * 4, m1 = min(m0 + 4, kp.N) - 1;
        const int t0 = (kp.fd + m0 - kp.unit_sbase) >> 7, t1 = (kp.fd + m1 - kp.unit_sbase) >> 7;
        const float z[3] = {0.f, 0.f, 0.f};
        for (int t = t0; t <= t1; t++)
            if (dd_unit_arrive(kp, b, t)) dd_unit_sor<128>(kp, b, t, false, z);
    }
}

// After asynchronous iterations the last FP32 dipoles of a bead sit in either buffer: refresh
// the main one from the FP64 dipoles (the same rounding as the SOR update's)
__global__ void __launch_bounds__(128) k_dipf_sync(KP kp) {
    const int s = kp.fd + blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (s >= kp.ld) return;
    const size_t gs = (size_t)b * kp.S + s;
    const float4 mf = make_float4((float)kp.dip[3 * gs], (float)kp.dip[3 * gs + 1], (float)kp.dip[3 * gs + 2], 0.f);
    kp.dipf[gs] = mf;
    mrec_dipole(kp, b, s, mf);
}

// pot_ttm.f90:399-542 in FP32 pair arithmetic, as a gather like k_pair_qq_m: QL lanes per
// molecule i over its full-list entries accumulate i's side (gradients at i's sites, the
// potentials at i's sites from j's dipoles) with virials at weight 1/2, then lane 0 of the group
// adds the intramolecular terms (pot_ttm.f90:482-542) before the group sums go into dR and F.w.
// (at most 102 registers, 5 blocks a SM: 99.1 -> 91.6 us at 512 x 32; the charge gather k_pair_qq_m
// measured slower so bounded, 106.7 -> 108.3 us, and keeps its 121 registers)
template <int MODEL>
__global__ void __launch_bounds__(128, 5) k_pair_force_m(KP kp) {
    using T = TM<MODEL>;
    const int b = blockIdx.y, N = kp.N;
    const int sub = threadIdx.x & (QL - 1);
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) / QL;
    const float4 *pf = kp.posf + (size_t)b * kp.S;
    const float4 *rh = kp.rhof + (size_t)b * kp.S;
    const float4 *mf = kp.dipf + (size_t)b * kp.S;
    const uint4 *of = kp.ofix + (size_t)b * N;
    const float4 *orw = kp.orawf + (size_t)b * N;
    const int2 *fl = reinterpret_cast<const int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    const bool same_a = kp.same_acd != 0;
    const float L[3] = {kp.ptf.box[0], kp.ptf.box[1], kp.ptf.box[2]};
    const float Li[3] = {kp.ptf.boxi[0], kp.ptf.boxi[1], kp.ptf.boxi[2]};
    float av[14];  // per-lane FP32 partials, reduced in FP64 per warp (block_reduce_add_f)
#pragma unroll
    for (int q = 0; q < 14; q++) av[q] = 0.f;
    float gi[5][3], pi[5];
#pragma unroll
    for (int k = 0; k < 5; k++) gi[k][0] = gi[k][1] = gi[k][2] = pi[k] = 0.f;
    if (i < N) {
        // row bounds clamped to the stored length (offsets run past it when the list overflowed)
        const int ne = kp.fntot[b];
        const int e0 = min(kp.foff[(size_t)b * N + i], ne);
        const int e1 = (i + 1 < N) ? min(kp.foff[(size_t)b * N + i + 1], ne) : ne;
        const uint4 oi = of[i];
        const float4 owi = orw[i];
        float4 si[5], ri[5];
        float mi[5][3];
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            si[k] = pf[(k - 1) * N + i];
            ri[k] = rh[(k - 1) * N + i];
            const float4 m = T::dip(k) ? mf[(k - 1) * N + i] : make_float4(0.f, 0.f, 0.f, 0.f);
            mi[k][0] = m.x, mi[k][1] = m.y, mi[k][2] = m.z;
        }
        float vt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vc = 0.f;
        for (int e = e0 + sub; e < e1; e += QL) {
            const int j = fl[e].y;
            float Rf[3];
            oo_min_image(kp, oi, of[j], Rf);
            // raw O-O difference: the force phase's centroid virial uses unwrapped centroid
            // differences (its Rij0 is wrapped to zero, pot_ttm.f90:406-407 and :468)
            const float4 owj = orw[j];
            const float Cf[3] = {owi.x - owj.x, owi.y - owj.y, owi.z - owj.z};
#pragma unroll
            for (int isp = 1; isp <= 4; isp++) {
#pragma unroll
                for (int jsp = 1; jsp <= 4; jsp++) {
                    if (!T::f_active(isp, jsp)) continue;
                    const float4 c4 = pf[(jsp - 1) * N + j];
                    const float Rs[3] = {wrapf(Rf[0] + si[isp].x - c4.x, L[0], Li[0]),
                                         wrapf(Rf[1] + si[isp].y - c4.y, L[1], Li[1]),
                                         wrapf(Rf[2] + si[isp].z - c4.z, L[2], Li[2])};
                    const float d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                    const float qi = si[isp].w, qj = c4.w;
                    float dj[3] = {0, 0, 0};
                    if (T::dip(jsp)) {
                        const float4 m = mf[(jsp - 1) * N + j];
                        dj[0] = m.x, dj[1] = m.y, dj[2] = m.z;
                    }
                    const float *di = mi[isp];
                    float qd[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) qd[c] = qj * di[c] - qi * dj[c];
                    const float qd2 = qd[0] * qd[0] + qd[1] * qd[1] + qd[2] * qd[2];
                    float dij[3] = {0, 0, 0};
                    float ts1 = 0.f, ts2 = 0.f;
                    bool have = false;
                    if (T::dip(isp) && T::dip(jsp)) {
                        float t1, t2, t3;
                        smear3<float>(d2, kp.ptf.apol_dd[isp][jsp], kp.ewf, &t1, &t2, &t3);
                        dd_force_f(Rs, di, dj, t2, t3, dij);
                        if (same_a) {
                            ts1 = t1, ts2 = t2;
                            have = true;
                        }
                    }
                    if (qd2 > 1.e-9f) {
                        if (!have) smear2<float>(d2, kp.ptf.apol_cd[isp][jsp], kp.ewf, &ts1, &ts2);
                        const float rq = Rs[0] * qd[0] + Rs[1] * qd[1] + Rs[2] * qd[2];
#pragma unroll
                        for (int c = 0; c < 3; c++) dij[c] += 3.f * ts2 * rq * Rs[c] - ts1 * qd[c];
                        if (isp != 1) pi[isp] += ts1 * (Rs[0] * dj[0] + Rs[1] * dj[1] + Rs[2] * dj[2]);
                    }
#pragma unroll
                    for (int c = 0; c < 3; c++) gi[isp][c] += dij[c];
                    const float4 rb = rh[(jsp - 1) * N + j];
                    const float Rc[3] = {Cf[0] + ri[isp].x - rb.x, Cf[1] + ri[isp].y - rb.y, Cf[2] + ri[isp].z - rb.z};
                    vc += Rc[0] * dij[0] + Rc[1] * dij[1] + Rc[2] * dij[2];
#pragma unroll
                    for (int col = 0; col < 3; col++)
#pragma unroll
                        for (int c = 0; c < 3; c++) vt[c + 3 * col] += dij[c] * Rs[col];
                }
            }
        }
        // each unordered pair was visited from both ends
        av[ACC_VIRIALC] += 0.5f * vc;
#pragma unroll
        for (int q = 0; q < 9; q++) av[ACC_VIRT + q] += 0.5f * vt[q];
        if (sub == 0) {  // intramolecular (pot_ttm.f90:482-542)
            float vt1[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vc1 = 0.f;
#pragma unroll
            for (int isp = 1; isp <= 3; isp++)
#pragma unroll
                for (int jsp = isp + 1; jsp <= 4; jsp++) {
                    const float Rs[3] = {si[isp].x - si[jsp].x, si[isp].y - si[jsp].y, si[isp].z - si[jsp].z};
                    const float Rc[3] = {wrapf(ri[isp].x - ri[jsp].x, L[0], Li[0]), wrapf(ri[isp].y - ri[jsp].y, L[1], Li[1]),
                                         wrapf(ri[isp].z - ri[jsp].z, L[2], Li[2])};
                    const float d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                    float dij[3] = {0, 0, 0};
                    if (T::dip(isp) && T::dip(jsp)) {
                        float t1, t2, t3;
                        smear3<float>(d2, kp.ptf.apol_dd[isp][jsp], kp.ewf, &t1, &t2, &t3);
                        dd_force_f(Rs, mi[isp], mi[jsp], t2, t3, dij);
                    }
                    const float qi = si[isp].w, qj = si[jsp].w;
                    float qd[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) qd[c] = qj * mi[isp][c] - qi * mi[jsp][c];
                    // self2 (smear.f90:133-156) in FP32
                    float dd, dri;
                    rinv<float>(d2, dd, dri);
                    const float drsqi = dri * dri;
                    const float expon = __expf(-(kp.ewf.a2 * d2));
                    const float kr0 = erfc_as<float>(kp.ewf.aewald * dd) * dri;
                    const float kr1 = (kr0 + kp.ewf.cts1 * expon) * drsqi;
                    const float kr2 = (kr1 + kp.ewf.cts2 * expon) * drsqi;
                    const float ch1 = -dri * drsqi, ch2 = ch1 * drsqi;
                    const float ts1 = kr1 + ch1, ts2 = kr2 + ch2;
                    const float rq = Rs[0] * qd[0] + Rs[1] * qd[1] + Rs[2] * qd[2];
#pragma unroll
                    for (int c = 0; c < 3; c++) dij[c] += 3.f * ts2 * rq * Rs[c] - ts1 * qd[c];
                    pi[isp] += ts1 * (Rs[0] * mi[jsp][0] + Rs[1] * mi[jsp][1] + Rs[2] * mi[jsp][2]);
                    pi[jsp] -= ts1 * (Rs[0] * mi[isp][0] + Rs[1] * mi[isp][1] + Rs[2] * mi[isp][2]);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        gi[isp][c] += dij[c];
                        gi[jsp][c] -= dij[c];
                    }
                    vc1 += Rc[0] * dij[0] + Rc[1] * dij[1] + Rc[2] * dij[2];
#pragma unroll
                    for (int col = 0; col < 3; col++)
#pragma unroll
                        for (int c = 0; c < 3; c++) vt1[c + 3 * col] += dij[c] * Rs[col];
                }
            av[ACC_VIRIALC] += vc1;
#pragma unroll
            for (int q = 0; q < 9; q++) av[ACC_VIRT + q] += vt1[q];
        }
    }
    // group sums of i's side (all lanes take part; lanes of i >= N hold zeros)
#pragma unroll
    for (int k = 1; k <= 4; k++) {
#pragma unroll
        for (int c = 0; c < 3; c++) gi[k][c] = group_sum<QL>(gi[k][c]);
        if (k != 1) pi[k] = group_sum<QL>(pi[k]);
    }
    // the FP64 adds spread over the group's lanes: lanes 0-11 the gradient components (site
    // sub / 3 + 1, component sub % 3), lanes 12-14 the potentials of sites 2-4
    if (i < N) {
        float v = 0.f;
#pragma unroll
        for (int kk = 1; kk <= 4; kk++)
#pragma unroll
            for (int cc = 0; cc < 3; cc++)
                if ((kk - 1) * 3 + cc == sub) v = gi[kk][cc];
#pragma unroll
        for (int kk = 2; kk <= 4; kk++)
            if (10 + kk == sub) v = pi[kk];
        if (sub < 12) {
            const int k = sub / 3 + 1, c = sub % 3;
            kp.dR[3 * ((size_t)b * kp.S + (size_t)(k - 1) * N + i) + c] += (double)v;
        } else if (sub < 15) {
            kp.F[(size_t)b * kp.S + (size_t)(sub - 11) * N + i].w += (double)v;
        }
    }
    block_reduce_add_f<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// ---------------------------------------------------------------------------------------
// Differentiation form, mixed engine (TTM3-F): the real-space terms of the backward outside the
// dipole sweep (the FP64 engine's k_adj_pairs) as a gather over the full list like the force
// pass -- QL lanes per molecule i over its entries (i, j), FP32 pair arithmetic from the O
// fixed-point sites and the site offsets, only i's side accumulated (the gradient at i's sites
// and the potential of the adjoint dipoles nu at i's charges; j's side when j gathers i), so
// there are no atomics per entry. Per entry:
//   * van der Waals on O-O: eb grad(C/r^6 + D e^{-E r} + A/r^12 + B/r^10) at O(i);
//   * for the charged sites a of i and c of j (H1, H2, M), with the charge-dipole smear2
//     (ts1, ts2) at R = r_a(i) - r_c(j): if a = M, nu_M(i) in the field of q_c(j) gives
//     q_c (ts1 nu - 3 ts2 (R.nu) R) at M(i); if c = M, nu_M(j) in the field of q_a(i) gives
//     minus the same form (R -> -R, nu_M(j), q_a) at a(i) and ts1 (R.nu) to its potential;
//   * the theta sums (a_cc: e^{-a r^3} (R.nu) and the Uelec term q_a q_c dts0/da with
//     dts0/da = exp(-a r^3) h(a^(1/3) r) / (3 a^(2/3)) from the tabulated Q(2/3, x); vdW C, D, E),
//     which see every pair twice, at weight 1/2.
__global__ void __launch_bounds__(128) k_adj_pairs_m(KP kp, float4 pfa, const double *ebar, const double *nu,
                                                     double *grad, double *phin, double *thacc) {
    const int b = blockIdx.y, N = kp.N;
    const int sub = threadIdx.x & (QL - 1);
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) / QL;
    const float pf[5] = {0.f, pfa.x, pfa.y, pfa.z, pfa.w};  // polfac of site kinds 1..4
    const float eb = (float)ebar[b];
    const float vA = kp.ptf.vdw[0], vB = kp.ptf.vdw[1], vC = kp.ptf.vdw[2], vD = kp.ptf.vdw[3], vE = kp.ptf.vdw[4];
    float gI[5][3], phI[5], th[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 5; k++) gI[k][0] = gI[k][1] = gI[k][2] = phI[k] = 0.f;
    if (i < N) {
        const float4 *pf4 = kp.posf + (size_t)b * kp.S;
        const uint4 *of = kp.ofix + (size_t)b * N;
        const int2 *fl = reinterpret_cast<const int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
        const double *nub = nu + 3 * ((size_t)b * kp.S + 3 * N);
        const float L[3] = {kp.ptf.box[0], kp.ptf.box[1], kp.ptf.box[2]};
        const float Li[3] = {kp.ptf.boxi[0], kp.ptf.boxi[1], kp.ptf.boxi[2]};
        const int ne = kp.fntot[b];
        const int e0 = min(kp.foff[(size_t)b * N + i], ne);
        const int e1 = (i + 1 < N) ? min(kp.foff[(size_t)b * N + i + 1], ne) : ne;
        const uint4 oi = of[i];
        float4 di[5];
#pragma unroll
        for (int k = 2; k <= 4; k++) di[k] = pf4[(k - 1) * N + i];
        const float ni[3] = {(float)nub[3 * i], (float)nub[3 * i + 1], (float)nub[3 * i + 2]};
        for (int e = e0 + sub; e < e1; e += QL) {
            const int j = fl[e].y;
            float Rf[3];
            oo_min_image(kp, oi, of[j], Rf);
            {  // van der Waals, O-O
                const float r2 = Rf[0] * Rf[0] + Rf[1] * Rf[1] + Rf[2] * Rf[2], r = sqrtf(r2);
                const float r2i = 1.f / r2, r6i = r2i * r2i * r2i, ex = __expf(-vE * r);
                const float dur = (-12.f * vA * r6i * r6i - 10.f * vB * r6i * r2i * r2i - 6.f * vC * r6i) * r2i - vD * vE * ex / r;
#pragma unroll
                for (int c = 0; c < 3; c++) gI[1][c] += eb * dur * Rf[c];
                th[1] += eb * r6i;
                th[2] += eb * ex;
                th[3] -= eb * vD * r * ex;
            }
            float4 dj[5];
#pragma unroll
            for (int k = 2; k <= 4; k++) dj[k] = pf4[(k - 1) * N + j];
            const float nj[3] = {(float)nub[3 * j], (float)nub[3 * j + 1], (float)nub[3 * j + 2]};
#pragma unroll
            for (int a = 2; a <= 4; a++) {
#pragma unroll
                for (int c = 2; c <= 4; c++) {
                    const float Rs[3] = {wrapf(Rf[0] + di[a].x - dj[c].x, L[0], Li[0]),
                                         wrapf(Rf[1] + di[a].y - dj[c].y, L[1], Li[1]),
                                         wrapf(Rf[2] + di[a].z - dj[c].z, L[2], Li[2])};
                    const float d2 = Rs[0] * Rs[0] + Rs[1] * Rs[1] + Rs[2] * Rs[2];
                    const float a12 = kp.ptf.apol_cd[a][c];
                    float ts1, ts2;
                    smear2<float>(d2, a12, kp.ewf, &ts1, &ts2);
                    const float pfac = pf[a] * pf[c], qa = di[a].w, qc = dj[c].w;
                    float e1 = 0.f;
                    if (d2 < 25.f) {
                        const float dd = sqrtf(d2), ra = cbrtf(a12);
                        e1 = __expf(-a12 * d2 * dd);
                        th[0] += eb * qa * qc * (e1 * gq_h(kp.gq23, ra * dd) / (3.f * ra * ra)) * pfac;
                    }
                    if (a == 4) {  // nu at M(i) in the field of q_c(j)
                        const float rn = Rs[0] * ni[0] + Rs[1] * ni[1] + Rs[2] * ni[2];
#pragma unroll
                        for (int q = 0; q < 3; q++) gI[4][q] += qc * (ts1 * ni[q] - 3.f * ts2 * rn * Rs[q]);
                        th[0] += qc * e1 * rn * pfac;
                    }
                    if (c == 4) {  // nu at M(j) in the field of q_a(i): R = r_M(j) - r_a(i) = -Rs
                        const float rn = -(Rs[0] * nj[0] + Rs[1] * nj[1] + Rs[2] * nj[2]);
#pragma unroll
                        for (int q = 0; q < 3; q++) gI[a][q] -= qa * (ts1 * nj[q] + 3.f * ts2 * rn * Rs[q]);
                        phI[a] += ts1 * rn;
                        th[0] += qa * e1 * rn * pfac;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int k = 1; k <= 4; k++) {
#pragma unroll
        for (int c = 0; c < 3; c++) gI[k][c] = group_sum<QL>(gI[k][c]);
        phI[k] = group_sum<QL>(phI[k]);
    }
    if (i < N && sub == 0) {
        const size_t base = (size_t)b * kp.S;
#pragma unroll
        for (int k = 1; k <= 4; k++) {
            double *g = grad + 3 * (base + (k - 1) * N + i);
#pragma unroll
            for (int c = 0; c < 3; c++) g[c] += (double)gI[k][c];
            if (k >= 2) phin[base + (k - 1) * N + i] += (double)phI[k];
        }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) th[q] *= 0.5f;
    block_reduce_add_f<4, 128>(th, thacc + PIMD_TH_A_CC);  // slots A_CC, VDW_C, VDW_D, VDW_E (contiguous)
}

void launch_adj_pairs_m(Engine &E, const double pf[5], const double *ebar, const double *nu, double *grad, double *phin,
                        double *thacc) {
    dim3 g((E.kp.N * QL + 127) / 128, E.kp.P);
    const float4 pfa = make_float4((float)pf[1], (float)pf[2], (float)pf[3], (float)pf[4]);
    k_adj_pairs_m<<<g, 128, 0, E.stream>>>(E.kp, pfa, ebar, nu, grad, phin, thacc);
    ++E.nlaunch;
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
    dim3 g((E.kp.N * QL + 127) / 128, E.kp.P);
    DISPATCH_M(E, k_pair_qq_m, g, 128);
}

// the per-entry dipole-pair smear scalars of the iterations (none when they are formed in each
// iteration); after the full lists and the site offsets
void launch_dd_tensors_m(Engine &E) {
    if (E.dd_otf) return;
    dim3 g2(pair_blocks_m(E, 128), E.kp.P);
    DISPATCH_M(E, k_dd_tensors_m, g2, 128);
}

void launch_dd_real_m(Engine &E) {
    dim3 g((E.kp.N * 32 + 127) / 128, E.kp.P);
    E.kp.l2keep = E.l2_keep ? 1 : 0;
    if (E.kp.model == 2)
        E.dd_otf ? k_dd_real_m<2, true, false><<<g, 128, 0, E.stream>>>(E.kp)
                 : k_dd_real_m<2, false, false><<<g, 128, 0, E.stream>>>(E.kp);
    else if (E.kp.dd_async)
        E.dd_otf ? k_dd_real_m<3, true, true><<<g, 128, 0, E.stream>>>(E.kp)
                 : k_dd_real_m<3, false, true><<<g, 128, 0, E.stream>>>(E.kp);
    else if (E.dd_jpev_req && E.loop_jpev) {
        // a programmatic event once every block has started (see Engine::loop_jpev)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = g;
        cfg.blockDim = dim3(128);
        cfg.stream = E.stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticEvent;
        at[0].val.programmaticEvent.event = E.loop_jpev;
        at[0].val.programmaticEvent.flags = 0;
        at[0].val.programmaticEvent.triggerAtBlockStart = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaError_t e = E.dd_otf ? cudaLaunchKernelEx(&cfg, k_dd_real_m<3, true, false>, E.kp)
                                 : cudaLaunchKernelEx(&cfg, k_dd_real_m<3, false, false>, E.kp);
        if (e == cudaSuccess) {
            E.dd_jpev_armed = true;
        } else {
            cudaGetLastError();
            E.dd_otf ? k_dd_real_m<3, true, false><<<g, 128, 0, E.stream>>>(E.kp)
                     : k_dd_real_m<3, false, false><<<g, 128, 0, E.stream>>>(E.kp);
        }
    } else
        E.dd_otf ? k_dd_real_m<3, true, false><<<g, 128, 0, E.stream>>>(E.kp)
                 : k_dd_real_m<3, false, false><<<g, 128, 0, E.stream>>>(E.kp);
    ++E.nlaunch;
}

// Whether the dipole iterations can run with the asynchronous real-space field: mixed engine,
// TTM3-F (M-site dipoles, in molecule order), the tensor-core structure factor and field pass,
// the second stream, and the buffers of the protocol.
bool dd_async_ok(const Engine &E) {
    const KP &kp = E.kp;
    return E.dd_async && E.dd_overlap && E.loop_aux && E.precision == PIMD_MIXED && kp.model == 3 && E.tc_ready &&
           E.sf_tc && E.tf_ready && E.ff_tc && kp.Erec && kp.unit_cnt && kp.dipf_alt && kp.ld - kp.fd == kp.N;
}

void launch_dipf_sync(Engine &E) {
    dim3 g((E.kp.ld - E.kp.fd + 127) / 128, E.kp.P);
    k_dipf_sync<<<g, 128, 0, E.stream>>>(E.kp);
    ++E.nlaunch;
}

void launch_pair_force_m(Engine &E) {
    dim3 g((E.kp.N * QL + 127) / 128, E.kp.P);
    DISPATCH_M(E, k_pair_force_m, g, 128);
}

}  // namespace pimd
