// common.cuh -- device helpers shared by the force-engine kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define PIMD_HD __host__ __device__ __forceinline__
#define PIMD_D __device__ __forceinline__

namespace pimd {

// consts.f90:22-55
constexpr double CHARGECON = 18.22234397655801030455;
constexpr double DEBYE = 4.8033324;
constexpr double MASSCON = 418.4;
constexpr double PI = 3.14159265358979323844;
constexpr double TWOPI = 6.28318530717958647688;
constexpr double FOURPI = 12.56637061435917295376;
constexpr double TSP = 1.12837916709551257390;
constexpr double SQPI = 1.77245385090551602729;
constexpr double KB_AMU = 0.831447148;
constexpr double HBAR = 6.35077993041;

// ---------------------------------------------------------------------------------------
// Minimum image exactly as the reference: r - box*anint(r*boxi), each product and
// difference rounded separately (no FMA), anint = round half away from zero.
// find_neigh.f90:77, pot_ttm.f90:64 etc.
PIMD_D double min_image_rn(double r, double box, double boxi) {
    return __dsub_rn(r, __dmul_rn(box, round(__dmul_rn(r, boxi))));
}
// Round to the nearest integer, ties to even, for |x| < 2^22: adding and subtracting 1.5 x 2^23
// leaves an FP32 value whose last place is 1, so the addition rounds x to an integer (the
// classic magic-number rounding). The same value as rintf(x) on that range, in two FP32 adds.
PIMD_D float rint_small(float x) {
    const float m = 12582912.0f;
    return __fsub_rn(__fadd_rn(x, m), m);
}
PIMD_D double dot3_rn(double x, double y, double z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// ---------------------------------------------------------------------------------------
// math.f90:287-314: Abramowitz-Stegun 7.1.26 complementary error function.
template <typename R>
PIMD_D R erfc_as(R x);
template <>
PIMD_D double erfc_as<double>(double X) {
    const double A1 = 0.254829592, A2 = -0.284496736, A3 = 1.421413741, A4 = -1.453152027,
                 A5 = 1.061405429, P = 0.3275911;
    double T = 1.0 / (1.0 + P * X);
    double TP = T * (A1 + T * (A2 + T * (A3 + T * (A4 + T * A5))));
    return TP * exp(-(X * X));
}
template <>
PIMD_D float erfc_as<float>(float X) {
    const float A1 = 0.254829592f, A2 = -0.284496736f, A3 = 1.421413741f, A4 = -1.453152027f,
                A5 = 1.061405429f, P = 0.3275911f;
    float T = __frcp_rn(1.0f + P * X);
    float TP = T * (A1 + T * (A2 + T * (A3 + T * (A4 + T * A5))));
    return TP * __expf(-(X * X));
}

// math.f90:188-285: Q(2/3, x) by the Numerical-Recipes series / Lentz continued fraction,
// EPS = 3e-7, gln = ln Gamma(2/3). Failure to converge sets bit 2 of *err.
template <typename R>
PIMD_D R gammq2_3(R x, unsigned *err) {
    const R a = R(2.0 / 3.0), gln = R(0.303150275147547), EPS = R(3.e-7);
    if (x < a + R(1)) {
        if (x <= R(0)) return R(1);
        R ap = a, ssum = R(1) / a, del = ssum;
        for (int n = 1; n <= 800; n++) {
            ap = ap + R(1);
            del = del * x / ap;
            ssum = ssum + del;
            if (fabs(del) < fabs(ssum) * EPS) return R(1) - ssum * exp(-x + a * log(x) - gln);
        }
        *err |= 4u;
        return R(1);
    }
    const R FPMIN = R(1.e-30);
    R b = x + R(1) - a, c = R(1) / FPMIN, d = R(1) / b, h = d;
    for (int i = 1; i <= 100; i++) {
        R an = -R(i) * (R(i) - a);
        b = b + R(2);
        d = an * d + b;
        if (fabs(d) < FPMIN) d = FPMIN;
        c = b + an / c;
        if (fabs(c) < FPMIN) c = FPMIN;
        d = R(1) / d;
        R del = d * c;
        h = h * del;
        if (fabs(del - R(1)) < EPS) return exp(-x + a * log(x) - gln) * h;
    }
    *err |= 4u;
    return R(0);
}

// Ewald constants shared by the smear kernels (potential.f90:196-198)
struct EwC {
    double aewald, a2, cts1, cts2, cts3;
};
struct EwCf {
    float aewald, a2, cts1, cts2, cts3;
};

// smear.f90:2-34 PBCsmear01: screened + Thole-smeared charge-charge tensors ts0, ts1.
// ra = a_pol12^(1/3) is passed precomputed (a function of the site kinds only).
template <typename R, typename EC>
PIMD_D void smear01(R drsq, R a_pol12, R ra, const EC &e, R *ts0, R *ts1, unsigned *err) {
    const R g23 = R(1.3541179394264);
    R dd = sqrt(drsq);
    R dri = R(1) / dd;
    R drsqi = dri * dri;
    R expon = exp(-(R(e.a2) * drsq));
    R er = erfc_as<R>(R(e.aewald) * dd);
    R t0 = er * dri;
    R t1 = (t0 + R(e.cts1) * expon) * drsqi;
    if (drsq < R(25)) {
        R rA3 = dd * drsq * a_pol12;
        R exp1 = exp(-rA3);
        R ch1 = -dri * drsqi;
        R sr1 = (R(1) - exp1) * dri * drsqi;
        t1 = t1 + ch1 + sr1;
        t0 = t0 - exp1 * dri + ra * g23 * gammq2_3<R>(rA3, err);
    }
    *ts0 = t0;
    *ts1 = t1;
}

// dd = r, dri = 1/r from r^2, and exp: FP64 as the reference (sqrt, divide, exp); FP32 (the mixed
// engine) by the hardware reciprocal square root and exp2 (a few ulp, below the FP32 noise of
// the pair sums)
template <typename R>
PIMD_D void rinv(R drsq, R &dd, R &dri);
template <>
PIMD_D void rinv<double>(double drsq, double &dd, double &dri) {
    dd = sqrt(drsq);
    dri = 1.0 / dd;
}
template <>
PIMD_D void rinv<float>(float drsq, float &dd, float &dri) {
    dri = rsqrtf(drsq);
    dd = drsq * dri;
}
PIMD_D double exp_p(double x) { return exp(x); }
PIMD_D float exp_p(float x) { return __expf(x); }

// smear.f90:36-69 PBCsmear2
template <typename R, typename EC>
PIMD_D void smear2(R drsq, R a_pol12, const EC &e, R *ts1, R *ts2) {
    R dd, dri;
    rinv<R>(drsq, dd, dri);
    R drsqi = dri * dri;
    R expon = exp_p(-(R(e.a2) * drsq));
    R er = erfc_as<R>(R(e.aewald) * dd);
    R t1 = (er * dri + R(e.cts1) * expon) * drsqi;
    R t2 = (t1 + R(e.cts2) * expon) * drsqi;
    if (drsq < R(25)) {
        R rA3 = (dd * drsq) * a_pol12;
        R exp1 = exp_p(-rA3);
        R ch1 = -dri * drsqi;
        R ch2 = ch1 * drsqi;
        R sr1 = (R(1) - exp1) * dri * drsqi;
        R sr2 = (sr1 - exp1 * a_pol12) * drsqi;
        t1 = t1 + ch1 + sr1;
        t2 = t2 + ch2 + sr2;
    }
    *ts1 = t1;
    *ts2 = t2;
}

// smear.f90:71-107 PBCsmear3
template <typename R, typename EC>
PIMD_D void smear3(R drsq, R a_pol12, const EC &e, R *ts1, R *ts2, R *ts3) {
    R dd, dri;
    rinv<R>(drsq, dd, dri);
    R drsqi = dri * dri;
    R expon = exp_p(-(R(e.a2) * drsq));
    R er = erfc_as<R>(R(e.aewald) * dd);
    R t1 = (er * dri + R(e.cts1) * expon) * drsqi;
    R t2 = (t1 + R(e.cts2) * expon) * drsqi;
    R t3 = (t2 + R(e.cts3) * expon) * drsqi;
    if (drsq < R(25)) {
        R rA3 = (dd * drsq) * a_pol12;
        R exp1 = exp_p(-rA3);
        R ch1 = -dri * drsqi;
        R ch2 = ch1 * drsqi;
        R ch3 = ch2 * drsqi;
        R sr1 = (R(1) - exp1) * dri * drsqi;
        R sr2 = (sr1 - exp1 * a_pol12) * drsqi;
        R sr3 = (sr2 - R(0.6) * exp1 * dd * a_pol12 * a_pol12) * drsqi;
        t1 = t1 + ch1 + sr1;
        t2 = t2 + ch2 + sr2;
        t3 = t3 + ch3 + sr3;
    }
    *ts1 = t1;
    *ts2 = t2;
    *ts3 = t3;
}

// smear.f90:110-131 self1 (intramolecular Ewald exclusion)
PIMD_D void self1(double drsq, const EwC &e, double *ts0, double *ts1) {
    double dd = sqrt(drsq);
    double drsqi = 1.0 / drsq;
    double dri = sqrt(drsqi);
    double expon = exp(-(e.a2 * drsq));
    double kr0 = erfc_as<double>(e.aewald * dd) * dri;
    double kr1 = (kr0 + e.cts1 * expon) * drsqi;
    double ch0 = -dri;
    double ch1 = ch0 * drsqi;
    *ts0 = ch0 + kr0;
    *ts1 = kr1 + ch1;
}

// self1 in FP32 (the mixed engine; the A&S erfc and the exponential as in smear2<float>): ts0
// to ~1e-7 and ts1 to ~1e-6 relative (ts1 cancels by about (a r)^2 at intramolecular r)
PIMD_D void self1f(float drsq, const EwCf &e, float *ts0, float *ts1) {
    float dd, dri;
    rinv<float>(drsq, dd, dri);
    const float drsqi = dri * dri;
    const float expon = exp_p(-(e.a2 * drsq));
    const float kr0 = erfc_as<float>(e.aewald * dd) * dri;
    const float kr1 = (kr0 + e.cts1 * expon) * drsqi;
    *ts0 = kr0 - dri;
    *ts1 = kr1 - dri * drsqi;
}

// smear.f90:133-156 self2
PIMD_D void self2(double drsq, const EwC &e, double *ts1, double *ts2) {
    double dd = sqrt(drsq);
    double drsqi = 1.0 / drsq;
    double dri = sqrt(drsqi);
    double expon = exp(-(e.a2 * drsq));
    double kr0 = erfc_as<double>(e.aewald * dd) * dri;
    double kr1 = (kr0 + e.cts1 * expon) * drsqi;
    double kr2 = (kr1 + e.cts2 * expon) * drsqi;
    double ch0 = -dri;
    double ch1 = ch0 * drsqi;
    double ch2 = ch1 * drsqi;
    *ts1 = kr1 + ch1;
    *ts2 = kr2 + ch2;
}

// dij of the dipole-dipole term: sum_ab di_a T_abc dj_b for the rank-3 Thole tensor
// T_abc = 15 t3 R_a R_b R_c - 3 t2 (d_bc R_a + d_ac R_b + d_ab R_c)  (pot_ttm.f90:430-441)
PIMD_D void dd_force(const double R[3], const double di[3], const double dj[3], double t2, double t3, double dij[3]) {
    const double rdi = R[0] * di[0] + R[1] * di[1] + R[2] * di[2];
    const double rdj = R[0] * dj[0] + R[1] * dj[1] + R[2] * dj[2];
    const double didj = di[0] * dj[0] + di[1] * dj[1] + di[2] * dj[2];
    const double a = 15.0 * t3 * rdi * rdj - 3.0 * t2 * didj;
#pragma unroll
    for (int c = 0; c < 3; c++) dij[c] += a * R[c] - 3.0 * t2 * (rdi * dj[c] + rdj * di[c]);
}
// the same in FP32 (the mixed engine)
PIMD_D void dd_force_f(const float R[3], const float di[3], const float dj[3], float t2, float t3, float dij[3]) {
    const float rdi = R[0] * di[0] + R[1] * di[1] + R[2] * di[2];
    const float rdj = R[0] * dj[0] + R[1] * dj[1] + R[2] * dj[2];
    const float didj = di[0] * dj[0] + di[1] * dj[1] + di[2] * dj[2];
    const float a = 15.f * t3 * rdi * rdj - 3.f * t2 * didj;
#pragma unroll
    for (int c = 0; c < 3; c++) dij[c] += a * R[c] - 3.f * t2 * (rdi * dj[c] + rdj * di[c]);
}

// ---------------------------------------------------------------------------------------
// block-wide sum of NV doubles into per-bead accumulators (one atomic per value per block)
template <int NV, int NT>
PIMD_D void block_reduce_add(double (&v)[NV], double *dst) {
    __shared__ double red[NT / 32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        double x = v[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][i] = x;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0;
#pragma unroll
        for (int w = 0; w < NT / 32; w++) s += red[w][threadIdx.x];
        if (s != 0.0) atomicAdd(dst + threadIdx.x, s);
    }
    __syncthreads();
}

// The same for per-thread FP32 partials (the mixed engine's pair kernels, about one pair per
// thread): warp sums in FP32, then the warps' sums added in FP64 -- no FP64 arithmetic per lane.
template <int NV, int NT>
PIMD_D void block_reduce_add_f(float (&v)[NV], double *dst) {
    __shared__ double red[NT / 32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        float x = v[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][i] = (double)x;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0;
#pragma unroll
        for (int w = 0; w < NT / 32; w++) s += red[w][threadIdx.x];
        if (s != 0.0) atomicAdd(dst + threadIdx.x, s);
    }
    __syncthreads();
}

}  // namespace pimd
