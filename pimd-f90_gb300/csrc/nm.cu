// nm.cu -- ring-polymer normal modes, PILE Langevin thermostat and the velocity-Verlet PIMD
// step on the device. Restates NormalModes.f90 (EvolveRing 34-63, InitNormalModes 68-218,
// real2NM/NM2real 308-341), Langevin.f90 (Langevin_NM 30-64, Init_Langevin_NM 68-98),
// MD.f90:35-110 (PIMD_VV) and main_stuff.f90 (PBCs 107-125, calc_uk 349-388).
//
// One group of 3P threads owns one atom (thread = (bead j, component c)); the P x P mode
// matrix C sits in shared memory. The transforms are summed in the reference's order with
// every product and sum rounded separately, so they are bit-identical to the FP64 oracle.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/pimd_gb300.h"
#include "engine.h"

namespace pimd {

int run_forces(Engine &E, int t, int check_every, double *Upott, double *virialt, double *virialct, double *virt9);

// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, SC'11).
PIMD_D uint4 philox4x32(uint4 ctr, uint2 key) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const unsigned hi0 = __umulhi(0xD2511F53u, ctr.x), lo0 = 0xD2511F53u * ctr.x;
        const unsigned hi1 = __umulhi(0xCD9E8D57u, ctr.z), lo1 = 0xCD9E8D57u * ctr.z;
        ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
        key.x += 0x9E3779B9u;
        key.y += 0xBB67AE85u;
    }
    return ctr;
}
// standard normal from two uniform 32-bit words (Box-Muller, radius branch)
PIMD_D double gauss_from(unsigned a, unsigned b) {
    const double u1 = ((double)a + 1.0) * 2.3283064365386963e-10;  // (0, 1]
    const double u2 = (double)b * 2.3283064365386963e-10;          // [0, 1)
    return sqrt(-2.0 * log(u1)) * cos(TWOPI * u2);
}

PIMD_D double noise(const NMArgs &a, int atom, int j, int c) {
    if (a.xi) return a.xi[c + 3 * j + (size_t)3 * a.P * atom];
    const unsigned long long idx = ((unsigned long long)atom * a.P + j) * 3 + c;
    const unsigned long long ctr = a.tstep ? 2ull * (unsigned long long)(long long)a.tstep[0] + (unsigned long long)a.phase
                                           : a.counter;
    const uint4 r = philox4x32(make_uint4((unsigned)idx, (unsigned)(idx >> 32), (unsigned)ctr, (unsigned)(ctr >> 32)),
                               make_uint2((unsigned)a.seed, (unsigned)(a.seed >> 32)));
    return gauss_from(r.x, r.y);
}

// C(j,k) sits in shared memory at Cs[j + (P + 1) k]: the padded column keeps the rows of
// NM2real (threads of a warp at different j, same k) on different banks
__host__ __device__ inline int nm_ld(int P) { return P + 1; }
template <typename T>
PIMD_D void nm_load_C(T *Cs, const T *C, int P) {
    for (int i = threadIdx.x; i < P * P; i += blockDim.x) Cs[i % P + nm_ld(P) * (i / P)] = C[i];
}

// x~_j = sum_k C(j,k) x_k  (real2NM) or x_j = sum_k C(k,j) x~_k (NM2real), rounded per op
PIMD_D double nm_row(const double *Cs, const double *v, int P, int j, int c, bool fwd) {
    const int L = nm_ld(P);
    double s = 0.0;
    for (int k = 0; k < P; k++) {
        const double ck = fwd ? Cs[j + L * k] : Cs[k + L * j];
        s = __dadd_rn(s, __dmul_rn(ck, v[3 * k + c]));
    }
    return s;
}

// Langevin_NM on one atom's momenta held in shared memory p[3P] (group-local).
PIMD_D void langevin_atom(const NMArgs &a, const double *Cs, double *p, double *tr, int atom, int j, int c,
                          bool active) {
    if (active) tr[3 * j + c] = nm_row(Cs, p, a.P, j, c, true);
    __syncthreads();
    if (active) {
        const double m = (atom % 3 == 0) ? a.massO : a.massH;
        const double sqrtmass = sqrt(m * a.A[4 * a.P + j]);
        const double c1 = a.A[5 * a.P + j], c2 = a.A[6 * a.P + j];
        tr[3 * j + c] = __dadd_rn(__dmul_rn(c1, tr[3 * j + c]), __dmul_rn(c2, __dmul_rn(sqrtmass, noise(a, atom, j, c))));
    }
    __syncthreads();
    if (active) p[3 * j + c] = nm_row(Cs, tr, a.P, j, c, false);
    __syncthreads();
}

// Nose_Hoover.f90:33-112: one half step (delt2) of a chain-2 thermostat (vxi[0], vxi[1]) on the
// kinetic energy uk of L degrees of freedom at temperature temp; returns s and leaves uk s^2 in
// uk. Every product and sum rounded separately, as the FP64 oracle computes it.
PIMD_D double nh_half(double *vxi, double &uk, double tau, double delt2, int L, double temp) {
    const double delt4 = __ddiv_rn(delt2, 2.0), delt8 = __ddiv_rn(delt2, 4.0);
    const double kT = __dmul_rn(KB_AMU, temp), LkT = __dmul_rn((double)L, kT);
    const double M1 = __dmul_rn(LkT, __dmul_rn(tau, tau)), M2 = M1;
    double v1 = vxi[0], v2 = vxi[1];
    v2 = __dadd_rn(v2, __ddiv_rn(__dmul_rn(__dsub_rn(__dmul_rn(M1, __dmul_rn(v1, v1)), kT), delt4), M2));
    v1 = __dmul_rn(v1, exp(__dmul_rn(-v2, delt8)));
    v1 = __dadd_rn(v1, __ddiv_rn(__dmul_rn(__dsub_rn(__dmul_rn(2.0, uk), LkT), delt4), M1));
    v1 = __dmul_rn(v1, exp(__dmul_rn(-v2, delt8)));
    const double s = exp(__dmul_rn(-v1, delt2));
    uk = __dmul_rn(__dmul_rn(uk, s), s);
    v1 = __dmul_rn(v1, exp(__dmul_rn(-v2, delt8)));
    v1 = __dadd_rn(v1, __ddiv_rn(__dmul_rn(__dsub_rn(__dmul_rn(2.0, uk), LkT), delt4), M1));
    v1 = __dmul_rn(v1, exp(__dmul_rn(-v2, delt8)));
    v2 = __dadd_rn(v2, __ddiv_rn(__dmul_rn(__dsub_rn(__dmul_rn(M1, __dmul_rn(v1, v1)), kT), delt4), M2));
    vxi[0] = v1;
    vxi[1] = v2;
    return s;
}

// bead_thermostat 'Nose-Hoover' (main_stuff.f90:145-171) on one atom's momenta p[3P] in shared
// memory: to normal modes, one chain per (mode j, component c) with L = 1 at Nbeads T (tau =
// 1/omega_j; the centroid mode only with centroid_nh, tau_centroid), back to real space
PIMD_D void bead_nh_atom(const NMArgs &a, const double *Cs, double *p, double *tr, int atom, int j, int c,
                         bool active) {
    if (active) tr[3 * j + c] = nm_row(Cs, p, a.P, j, c, true);
    __syncthreads();
    if (active && (j > 0 || a.centroid_nh)) {
        const double imass = 1.0 / ((atom % 3 == 0) ? a.massO : a.massH);
        double *vx = a.vxib + 2 * ((size_t)atom + (size_t)a.natoms * ((size_t)j + (size_t)a.P * c));
        const double x = tr[3 * j + c];
        double ukb = __dmul_rn(__dmul_rn(0.5, imass), __dmul_rn(x, x));
        double tau = a.tau_centroid;
        if (j > 0) {
            ukb = __ddiv_rn(ukb, a.A[4 * a.P + j]);
            tau = __ddiv_rn(1.0, a.A[10 * a.P + j]);
        }
        double v[2] = {vx[0], vx[1]};
        const double sb = nh_half(v, ukb, tau, a.delt2, 1, a.nh_temp);
        vx[0] = v[0];
        vx[1] = v[1];
        tr[3 * j + c] = __dmul_rn(x, sb);
    }
    __syncthreads();
    if (active) p[3 * j + c] = nm_row(Cs, tr, a.P, j, c, false);
    __syncthreads();
}

// the bead thermostat of the step (Langevin_NM or the bead chains), then the global chain's s
PIMD_D void bead_thermostat(const NMArgs &a, const double *Cs, double *p, double *tr, int atom, int j, int c,
                            bool active) {
    if (a.langevin) langevin_atom(a, Cs, p, tr, atom, j, c, active);
    else if (a.bead_nh) bead_nh_atom(a, Cs, p, tr, atom, j, c, active);
}

// ---- the mixed engine's integrator: FP32-pair (double-float) arithmetic ----------------------
// The FP64 state enters and leaves as pairs x = h + l by bit operations (h: the mantissa cut to
// 24 bits, l: the remaining 29 bits rounded to FP32, ~2^-48 relative), so the step issues almost
// no FP64 instruction (this part runs FP64 at 1/64 of the FP32 rate). Error-free transforms:
// TwoSum (Knuth), Fast2Sum (Dekker), TwoProduct by FMA; pair sum and product after Joldes,
// Muller and Popescu, ACM TOMS 44 (2017), Algorithm 6 (AccurateDWPlusDW, <= 3u^2) and the
// FMA product (DWTimesDW, ~5u^2). Intrinsics keep every rounding.
struct dfl {
    float h, l;
};
PIMD_D dfl two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
PIMD_D dfl fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
PIMD_D dfl df_add(dfl a, dfl b) {
    const dfl s = two_sum(a.h, b.h), t = two_sum(a.l, b.l);
    const dfl v = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
    return fast_two_sum(v.h, __fadd_rn(t.l, v.l));
}
PIMD_D dfl df_neg(dfl a) { return {-a.h, -a.l}; }
PIMD_D dfl df_mul(dfl a, dfl b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
    return fast_two_sum(p, e);
}
// double -> pair by bit operations only (a branch to conversion instructions would be
// predicated and issued on every lane): exact to 2^-48 for 2^-70 <= |x| < 2^101; smaller
// magnitudes (zero included) give a signed zero, larger ones and NaN an infinity / NaN
PIMD_D dfl df_split(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned hw = (unsigned)(u >> 32), lw = (unsigned)u;
    const int eb = (int)((hw >> 20) & 0x7ffu) - 1023;
    const unsigned sign = hw & 0x80000000u;
    if (eb < -70) return {__uint_as_float(sign), 0.f};
    if (eb > 100) return {__uint_as_float(sign | 0x7f800000u | ((eb == 1024 && ((hw & 0xfffffu) | lw)) ? 0x400000u : 0u)), 0.f};
    const float h = __uint_as_float(sign | ((unsigned)(eb + 127) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
    const float l = __fmul_rn(__uint2float_rn(lw & 0x1fffffffu), __uint_as_float((unsigned)(eb + 75) << 23));
    return {h, __uint_as_float(__float_as_uint(l) | sign)};
}
// float -> double by bit operations (exact for every input)
PIMD_D double f2d_bits(float f) {
    const unsigned b = __float_as_uint(f), e = (b >> 23) & 0xffu;
    const unsigned long long sg = (unsigned long long)(b & 0x80000000u) << 32;
    unsigned m = b & 0x7fffffu, ed;
    if (e == 255) {
        ed = 0x7ffu;
    } else if (e != 0) {
        ed = e + 896;
    } else if (m == 0) {
        ed = 0;
    } else {  // subnormal: normalise the mantissa
        const int n = __clz(m) - 8;
        m = (m << n) & 0x7fffffu;
        ed = 897 - n;
    }
    return __longlong_as_double((long long)(sg | ((unsigned long long)ed << 52) | ((unsigned long long)m << 29)));
}
PIMD_D double df_double(dfl a) { return f2d_bits(a.h) + f2d_bits(a.l); }
PIMD_D dfl df_f(float2 v) { return {v.x, v.y}; }
PIMD_D float2 df_store(dfl a) { return make_float2(a.h, a.l); }

// Dot2 over the pairs of C and of the group's vector (as nm_row_pair), result as a pair
PIMD_D dfl nm_row_df(const float2 *Cf, const float2 *vf, int P, int j, int c, bool fwd) {
    const int L = nm_ld(P);
    float s = 0.f, comp = 0.f;
#pragma unroll 4
    for (int k = 0; k < P; k++) {
        const float2 ck = fwd ? Cf[j + L * k] : Cf[k + L * j];
        const float2 vk = vf[3 * k + c];
        const float ph = __fmul_rn(ck.x, vk.x);
        float pe = __fmaf_rn(ck.x, vk.x, -ph);
        pe = __fmaf_rn(ck.x, vk.y, __fmaf_rn(ck.y, vk.x, pe));
        const float t = __fadd_rn(s, ph);
        const float z = __fsub_rn(t, s);
        comp = __fadd_rn(comp, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(ph, z)), pe));
        s = t;
    }
    return two_sum(s, comp);
}

// per-bead constants of the fast kernels as pairs in shared memory: A11, A22, c1 (P each), then
// per atom type (O, H) A12 / (m msf), A21 m msf, c2 sqrt(m msf) (2 x 3P); from A's rows 7-9
// (A12 / msf, A21 msf, c2 sqrt(msf)) and the host-computed 1/m, m, sqrt(m) of NMArgs
PIMD_D void nm_fast_consts(const NMArgs &a, float2 *kf) {
    const int P = a.P;
    for (int i = threadIdx.x; i < 3 * P; i += blockDim.x) {
        const int row = i / P, j = i % P;
        kf[i] = df_store(df_split(a.A[(row == 0 ? 0 : row == 1 ? 3 : 5) * P + j]));
        for (int ty = 0; ty < 2; ty++) {
            const double f = row == 0 ? a.minv[ty] : row == 1 ? a.mass[ty] : a.msqrt[ty];
            const dfl v = df_mul(df_split(a.A[(7 + row) * P + j]), df_split(f));
            kf[3 * P + ty * 3 * P + i] = df_store(v);
        }
    }
}

PIMD_D float gauss_f(unsigned a, unsigned b) {
    const float u1 = ((float)a + 1.0f) * 2.3283064365386963e-10f;
    const float u2 = (float)b * 2.3283064365386963e-10f;
    return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}
PIMD_D dfl noise_df(const NMArgs &a, int atom, int j, int c) {
    if (a.xi) return df_split(a.xi[c + 3 * j + (size_t)3 * a.P * atom]);
    const unsigned long long idx = ((unsigned long long)atom * a.P + j) * 3 + c;
    const unsigned long long ctr = a.tstep ? 2ull * (unsigned long long)(long long)a.tstep[0] + (unsigned long long)a.phase
                                           : a.counter;
    const uint4 r = philox4x32(make_uint4((unsigned)idx, (unsigned)(idx >> 32), (unsigned)ctr, (unsigned)(ctr >> 32)),
                               make_uint2((unsigned)a.seed, (unsigned)(a.seed >> 32)));
    return {gauss_f(r.x, r.y), 0.f};
}

// Langevin_NM on the group's momenta as pairs (vp: the group's pair vector, pp: this thread's)
PIMD_D dfl langevin_df(const NMArgs &a, const float2 *Cf, const float2 *kf, float2 *vp, dfl pp, int atom, int j, int c,
                       bool active) {
    const int P = a.P, ty = (atom % 3 == 0) ? 0 : 1;
    if (active) vp[3 * j + c] = df_store(pp);
    __syncthreads();
    dfl t{0.f, 0.f};
    if (active) t = nm_row_df(Cf, vp, P, j, c, true);
    __syncthreads();
    if (active)
        vp[3 * j + c] = df_store(df_add(df_mul(df_f(kf[2 * P + j]), t), df_mul(df_f(kf[3 * P + ty * 3 * P + 2 * P + j]),
                                                                                 noise_df(a, atom, j, c))));
    __syncthreads();
    if (active) pp = nm_row_df(Cf, vp, P, j, c, false);
    __syncthreads();
    return pp;
}

// shared memory of the fast kernels: padded C and the constants as pairs, then per group two
// pair vectors and the centroid's image shift (3 floats, padded to 2 float2)
PIMD_D void nm_fast_layout(int P, int g, float2 *&Cf, float2 *&kf, float2 *&vx, float2 *&vp, float *&nsh) {
    extern __shared__ double sh[];
    Cf = reinterpret_cast<float2 *>(sh);
    kf = Cf + nm_ld(P) * P;
    vx = kf + 9 * P + g * (6 * P + 2);
    vp = vx + 3 * P;
    nsh = reinterpret_cast<float *>(vp + 3 * P);
}
size_t nm_fast_smem(int P, int G) { return sizeof(float2) * ((size_t)nm_ld(P) * P + 9 * (size_t)P + (size_t)G * (6 * P + 2)); }

void nm_fast_args(NMArgs &a) {
    const double m[2] = {a.massO, a.massH};
    for (int t = 0; t < 2; t++) {
        a.mass[t] = m[t];
        a.minv[t] = 1.0 / m[t];
        a.msqrt[t] = std::sqrt(m[t]);
    }
    auto pair = [](double v) {
        const float h = (float)v;
        return make_float2(h, (float)(v - (double)h));
    };
    a.kick = pair(MASSCON * a.delt2);
    a.hminv[0] = pair(0.5 / a.massO);
    a.hminv[1] = pair(0.5 / a.massH);
    a.pinv = pair(1.0 / a.P);
    a.boxf = pair(a.box0);
    a.boxif = (float)a.boxi0;
}

// The MD-step kernels' bodies take the block index blk (of the replica's own grid), so that a
// replica batch runs every replica's blocks in one launch (k_md_batch).
PIMD_D void md_pre_fast_body(const NMArgs &a, int blk, double *RRt, double *PPt, const double *dRRt, double *RRc) {
    const int P = a.P, G = blockDim.x / (3 * P);
    const int g = threadIdx.x / (3 * P), r = threadIdx.x % (3 * P), j = r / 3, c = r % 3;
    const int atom = blk * G + g;
    float2 *Cf, *kf, *vx, *vp;
    float *nsh;
    nm_fast_layout(P, min(g, G - 1), Cf, kf, vx, vp, nsh);
    nm_load_C(Cf, reinterpret_cast<const float2 *>(a.C + P * P), P);
    nm_fast_consts(a, kf);
    const bool active = g < G && atom < a.natoms;
    const size_t gi = (size_t)3 * a.natoms * j + 3 * atom + c;
    dfl px{0.f, 0.f}, pp{0.f, 0.f}, pg{0.f, 0.f};
    if (active) {
        px = df_split(RRt[gi]);
        pp = df_split(PPt[gi]);
        pg = df_split(dRRt[gi]);
    }
    __syncthreads();
    if (a.langevin) pp = langevin_df(a, Cf, kf, vp, pp, atom, j, c, active);
    pp = df_add(pp, df_neg(df_mul(df_f(a.kick), pg)));  // p -= MASSCON dt/2 dV/dx
    const int ty = (atom % 3 == 0) ? 0 : 1;
    if (a.evolve) {
        if (active) {
            vx[3 * j + c] = df_store(px);
            vp[3 * j + c] = df_store(pp);
        }
        __syncthreads();
        dfl xt{0.f, 0.f}, pt{0.f, 0.f};
        if (active) {
            xt = nm_row_df(Cf, vx, P, j, c, true);
            pt = nm_row_df(Cf, vp, P, j, c, true);
        }
        __syncthreads();
        if (active) {
            const float2 *kt = kf + 3 * P + ty * 3 * P;
            vx[3 * j + c] = df_store(df_add(df_mul(df_f(kf[j]), xt), df_mul(df_f(kt[j]), pt)));
            vp[3 * j + c] = df_store(df_add(df_mul(df_f(kt[P + j]), xt), df_mul(df_f(kf[P + j]), pt)));
        }
        __syncthreads();
        if (active) {
            px = nm_row_df(Cf, vx, P, j, c, false);
            pp = nm_row_df(Cf, vp, P, j, c, false);
        }
    } else if (active) {  // P = 1: free flight
        px = df_add(px, df_mul(pp, df_split(a.delt * a.minv[ty])));
    }
    __syncthreads();  // the transforms have read vx
    if (active) vx[3 * j + c] = df_store(px);
    __syncthreads();
    // centroid (main_stuff.f90:107-125) in pair arithmetic, its image from the FP32 value (any
    // whole number of boxes is a valid shift; the molecule moves as a whole)
    if (active && j == 0) {
        dfl sum{0.f, 0.f};
        for (int k = 0; k < P; k++) sum = df_add(sum, df_f(vx[3 * k + c]));
        const dfl rc = df_mul(sum, df_f(a.pinv));
        const float n = rintf(__fmul_rn(rc.h, a.boxif));
        const dfl rs = df_add(rc, df_neg(df_mul(df_f(a.boxf), dfl{n, 0.f})));
        RRc[3 * atom + c] = df_double(rs);
        nsh[c] = n;
    }
    __syncthreads();
    if (active) {
        RRt[gi] = df_double(df_add(px, df_neg(df_mul(df_f(a.boxf), dfl{nsh[c], 0.f}))));
        PPt[gi] = df_double(pp);
    }
}

PIMD_D void md_post_fast_body(const NMArgs &a, int blk, double *PPt, const double *dRRt, double *uk) {
    const int P = a.P, G = blockDim.x / (3 * P);
    const int g = threadIdx.x / (3 * P), r = threadIdx.x % (3 * P), j = r / 3, c = r % 3;
    const int atom = blk * G + g;
    float2 *Cf, *kf, *vx, *vp;
    float *nsh;
    nm_fast_layout(P, min(g, G - 1), Cf, kf, vx, vp, nsh);
    nm_load_C(Cf, reinterpret_cast<const float2 *>(a.C + P * P), P);
    nm_fast_consts(a, kf);
    const bool active = g < G && atom < a.natoms;
    const size_t gi = (size_t)3 * a.natoms * j + 3 * atom + c;
    dfl pp{0.f, 0.f};
    if (active) pp = df_add(df_split(PPt[gi]), df_neg(df_mul(df_f(a.kick), df_split(dRRt[gi]))));
    __syncthreads();
    if (a.langevin) pp = langevin_df(a, Cf, kf, vp, pp, atom, j, c, active);
    dfl ke{0.f, 0.f};
    if (active) {
        PPt[gi] = df_double(pp);
        ke = df_mul(df_mul(pp, pp), df_f(a.hminv[(atom % 3 == 0) ? 0 : 1]));
    }
    for (int o = 16; o > 0; o >>= 1)
        ke = df_add(ke, dfl{__shfl_xor_sync(0xffffffffu, ke.h, o), __shfl_xor_sync(0xffffffffu, ke.l, o)});
    __shared__ double wke[32];
    if ((threadIdx.x & 31) == 0) wke[threadIdx.x >> 5] = df_double(ke);
    __syncthreads();
    if (threadIdx.x == 0 && uk) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += wke[w];
        atomicAdd(uk, t);
    }
}

// MD.f90:40-73 up to the force call: Langevin, half kick, EvolveRing (or free flight for
// P = 1), centroid and the centroid-following PBC shift (main_stuff.f90:107-125).
PIMD_D void md_pre_body(const NMArgs &a, int blk, double *RRt, double *PPt, const double *dRRt, double *RRc) {
    extern __shared__ double sh[];
    const int P = a.P, G = blockDim.x / (3 * P);
    const int g = threadIdx.x / (3 * P), r = threadIdx.x % (3 * P), j = r / 3, c = r % 3;
    const int atom = blk * G + g;
    double *Cs = sh;
    double *x = Cs + nm_ld(P) * P + g * 9 * P, *p = x + 3 * P, *tr = p + 3 * P;
    nm_load_C(Cs, a.C, P);
    const bool active = g < G && atom < a.natoms;
    const size_t gi = (size_t)3 * a.natoms * j + 3 * atom + c;
    if (active) {
        x[3 * j + c] = RRt[gi];
        p[3 * j + c] = PPt[gi];
    }
    __syncthreads();
    bead_thermostat(a, Cs, p, tr, atom, j, c, active);
    if (active && a.s_pre) p[3 * j + c] = __dmul_rn(p[3 * j + c], *a.s_pre);  // MD.f90:43-46
    if (active) p[3 * j + c] = __dsub_rn(p[3 * j + c], __dmul_rn(__dmul_rn(MASSCON, dRRt[gi]), a.delt2));
    __syncthreads();
    const double m = (atom % 3 == 0) ? a.massO : a.massH;
    if (a.evolve && !a.nodrift) {
        double xt = 0, pt = 0;
        if (active) {
            xt = nm_row(Cs, x, P, j, c, true);
            pt = nm_row(Cs, p, P, j, c, true);
        }
        __syncthreads();
        if (active) {
            const double A11 = a.A[j], A12 = a.A[P + j], A21 = a.A[2 * P + j], A22 = a.A[3 * P + j], msf = a.A[4 * P + j];
            const double xn = __dadd_rn(__dmul_rn(A11, xt), __ddiv_rn(__dmul_rn(A12, pt), __dmul_rn(m, msf)));
            const double pn = __dadd_rn(__dmul_rn(__dmul_rn(__dmul_rn(A21, m), msf), xt), __dmul_rn(A22, pt));
            tr[3 * j + c] = xn;
            x[3 * j + c] = pn;  // reuse x as the momentum-mode buffer
        }
        __syncthreads();
        double xr = 0, pr = 0;
        if (active) {
            xr = nm_row(Cs, tr, P, j, c, false);
            pr = nm_row(Cs, x, P, j, c, false);
        }
        __syncthreads();
        if (active) {
            x[3 * j + c] = xr;
            p[3 * j + c] = pr;
        }
        __syncthreads();
    } else if (active && !a.nodrift) {
        x[3 * j + c] = __dadd_rn(x[3 * j + c], __dmul_rn(__dmul_rn(1.0 / m, p[3 * j + c]), a.delt));
    }
    __syncthreads();
    if (active && j == 0) {
        double s = 0.0;
        for (int k = 0; k < P; k++) s = __dadd_rn(s, x[3 * k + c]);
        double rc = __ddiv_rn(s, (double)P);
        const double shift = __dmul_rn(a.box0, round(__dmul_rn(rc, a.boxi0)));
        RRc[3 * atom + c] = __dsub_rn(rc, shift);
        tr[c] = shift;
    }
    __syncthreads();
    if (active) {
        RRt[gi] = __dsub_rn(x[3 * j + c], tr[c]);
        PPt[gi] = p[3 * j + c];
    }
}

// MD.f90:94-101: half kick with the new gradient, Langevin, kinetic energy (calc_uk)
PIMD_D void md_post_body(const NMArgs &a, int blk, double *PPt, const double *dRRt, double *uk) {
    extern __shared__ double sh[];
    const int P = a.P, G = blockDim.x / (3 * P);
    const int g = threadIdx.x / (3 * P), r = threadIdx.x % (3 * P), j = r / 3, c = r % 3;
    const int atom = blk * G + g;
    double *Cs = sh;
    double *p = Cs + nm_ld(P) * P + g * 9 * P, *tr = p + 3 * P;
    nm_load_C(Cs, a.C, P);
    const bool active = g < G && atom < a.natoms;
    const size_t gi = (size_t)3 * a.natoms * j + 3 * atom + c;
    if (active) p[3 * j + c] = __dsub_rn(PPt[gi], __dmul_rn(__dmul_rn(MASSCON, dRRt[gi]), a.delt2));
    __syncthreads();
    bead_thermostat(a, Cs, p, tr, atom, j, c, active);
    double ke = 0.0;
    if (active) {
        PPt[gi] = p[3 * j + c];
        const double m = (atom % 3 == 0) ? a.massO : a.massH;
        if (a.nm_ke) {  // calc_uk's normal-mode form (main_stuff.f90:367-384)
            const double pt = nm_row(Cs, p, P, j, c, true);
            ke = (1.0 / m) * pt * pt / a.A[4 * P + j];
        } else {
            ke = (1.0 / m) * p[3 * j + c] * p[3 * j + c];
        }
    }
    for (int o = 16; o > 0; o >>= 1) ke += __shfl_xor_sync(0xffffffffu, ke, o);
    // the block's warps in order, then one atomic per block (not per warp: one address)
    __shared__ double wke[32];
    if ((threadIdx.x & 31) == 0) wke[threadIdx.x >> 5] = ke;
    __syncthreads();
    if (threadIdx.x == 0 && uk) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += wke[w];
        atomicAdd(uk, 0.5 * t);
    }
}

__global__ void k_md_pre_fast(NMArgs a, double *RRt, double *PPt, const double *dRRt, double *RRc) {
    md_pre_fast_body(a, blockIdx.x, RRt, PPt, dRRt, RRc);
}
__global__ void k_md_post_fast(NMArgs a, double *PPt, const double *dRRt, double *uk) {
    md_post_fast_body(a, blockIdx.x, PPt, dRRt, uk);
}
__global__ void k_md_pre(NMArgs a, double *RRt, double *PPt, const double *dRRt, double *RRc) {
    md_pre_body(a, blockIdx.x, RRt, PPt, dRRt, RRc);
}
__global__ void k_md_post(NMArgs a, double *PPt, const double *dRRt, double *uk) {
    md_post_body(a, blockIdx.x, PPt, dRRt, uk);
}

// A replica batch's MD-step phase (PHASE 0: up to the force call, 1: after it) for every replica
// in one launch: block blockIdx.x runs block blkmap.y of replica blkmap.x with that replica's
// arguments (own P, matrices, Langevin coefficients, seed and state pointers); blocks of 256
// threads hold 256 / (3P) atoms each, as the replica's own launch shape.
template <int PHASE, bool FAST>
__global__ void __launch_bounds__(256) k_md_batch(const NMBatchRep *reps, const int2 *blkmap) {
    __shared__ NMBatchRep sr;
    const int2 m = blkmap[blockIdx.x];
    if (threadIdx.x == 0) {
        sr = reps[m.x];
        sr.a.phase = PHASE;
    }
    __syncthreads();
    if (PHASE == 0) {
        if (FAST)
            md_pre_fast_body(sr.a, m.y, sr.RRt, sr.PPt, sr.dRRt, sr.RRc);
        else
            md_pre_body(sr.a, m.y, sr.RRt, sr.PPt, sr.dRRt, sr.RRc);
    } else {
        if (FAST)
            md_post_fast_body(sr.a, m.y, sr.PPt, sr.dRRt, sr.uk);
        else
            md_post_body(sr.a, m.y, sr.PPt, sr.dRRt, sr.uk);
    }
}
void nm_launch_md_batch(int phase, bool fast, int nblk, size_t smem, cudaStream_t st, const NMBatchRep *reps,
                        const int2 *blkmap) {
    if (smem > 48 * 1024) {  // the opt-in above 48 KB (large bead counts), outside any capture
        static size_t set = 0;
        if (smem > set) {
            cudaFuncSetAttribute(k_md_batch<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaFuncSetAttribute(k_md_batch<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaFuncSetAttribute(k_md_batch<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaFuncSetAttribute(k_md_batch<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            set = smem;
        }
    }
    if (nblk <= 0) return;
    if (phase == 0)
        fast ? k_md_batch<0, true><<<nblk, 256, smem, st>>>(reps, blkmap)
             : k_md_batch<0, false><<<nblk, 256, smem, st>>>(reps, blkmap);
    else
        fast ? k_md_batch<1, true><<<nblk, 256, smem, st>>>(reps, blkmap)
             : k_md_batch<1, false><<<nblk, 256, smem, st>>>(reps, blkmap);
}

// EvolveRing alone for every atom (no kick, no thermostat)
__global__ void k_evolve(NMArgs a, double *RRt, double *PPt) {
    extern __shared__ double sh[];
    const int P = a.P, G = blockDim.x / (3 * P);
    const int g = threadIdx.x / (3 * P), r = threadIdx.x % (3 * P), j = r / 3, c = r % 3;
    const int atom = blockIdx.x * G + g;
    double *Cs = sh;
    double *x = Cs + nm_ld(P) * P + g * 9 * P, *p = x + 3 * P, *tr = p + 3 * P;
    nm_load_C(Cs, a.C, P);
    const bool active = g < G && atom < a.natoms;
    const size_t gi = (size_t)3 * a.natoms * j + 3 * atom + c;
    if (active) {
        x[3 * j + c] = RRt[gi];
        p[3 * j + c] = PPt[gi];
    }
    __syncthreads();
    const double m = (atom % 3 == 0) ? a.massO : a.massH;
    double xt = 0, pt = 0;
    if (active) {
        xt = nm_row(Cs, x, P, j, c, true);
        pt = nm_row(Cs, p, P, j, c, true);
    }
    __syncthreads();
    if (active) {
        const double A11 = a.A[j], A12 = a.A[P + j], A21 = a.A[2 * P + j], A22 = a.A[3 * P + j], msf = a.A[4 * P + j];
        tr[3 * j + c] = __dadd_rn(__dmul_rn(A11, xt), __ddiv_rn(__dmul_rn(A12, pt), __dmul_rn(m, msf)));
        x[3 * j + c] = __dadd_rn(__dmul_rn(__dmul_rn(__dmul_rn(A21, m), msf), xt), __dmul_rn(A22, pt));
    }
    __syncthreads();
    if (active) {
        RRt[gi] = nm_row(Cs, tr, P, j, c, false);
        PPt[gi] = nm_row(Cs, x, P, j, c, false);
    }
}

__global__ void k_langevin(NMArgs a, double *PPt) {
    extern __shared__ double sh[];
    const int P = a.P, G = blockDim.x / (3 * P);
    const int g = threadIdx.x / (3 * P), r = threadIdx.x % (3 * P), j = r / 3, c = r % 3;
    const int atom = blockIdx.x * G + g;
    double *Cs = sh;
    double *p = Cs + nm_ld(P) * P + g * 9 * P, *tr = p + 3 * P;
    nm_load_C(Cs, a.C, P);
    const bool active = g < G && atom < a.natoms;
    const size_t gi = (size_t)3 * a.natoms * j + 3 * atom + c;
    if (active) p[3 * j + c] = PPt[gi];
    __syncthreads();
    langevin_atom(a, Cs, p, tr, atom, j, c, active);
    if (active) PPt[gi] = p[3 * j + c];
}

// the global chain thermostat (MD.f90:43-46 at the start, 101-104 at the end of the step) on
// the reference's module variable uk: nh = [vxi1, vxi2, uk, s_pre, s_post, ...]; at the end the
// step's calc_uk (uk_end) replaces uk first
__global__ void k_nh_global(double *nh, const double *uk_end, int slot, double tau, double delt2, int L, double temp) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double uk = uk_end ? *uk_end : nh[2];
    double v[2] = {nh[0], nh[1]};
    nh[slot] = nh_half(v, uk, tau, delt2, L, temp);
    nh[0] = v[0];
    nh[1] = v[1];
    nh[2] = uk;
}

// PPt = PPt * s (MD.f90:103)
__global__ void k_nh_scale(double *PPt, size_t n, const double *s) {
    const double f = *s;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        PPt[i] = __dmul_rn(PPt[i], f);
}

// write_out's inputs after the force call: calc_uk (main_stuff.f90:349-388, real-space or
// normal-mode form) into sums[0] and the ring-spring sum K0 = sum m (r_k - r_(k-1))^2 of
// simple_quantum_estimators (estimators.f90:57-73) into sums[1]; one group of 3P threads per atom
__global__ void k_ring_sums(NMArgs a, const double *RRt, const double *PPt, double *sums) {
    extern __shared__ double sh[];
    const int P = a.P, G = blockDim.x / (3 * P);
    const int g = threadIdx.x / (3 * P), r = threadIdx.x % (3 * P), j = r / 3, c = r % 3;
    const int atom = blockIdx.x * G + g;
    double *Cs = sh;
    double *x = Cs + nm_ld(P) * P + g * 9 * P, *p = x + 3 * P;
    if (a.nm_ke) nm_load_C(Cs, a.C, P);
    const bool active = g < G && atom < a.natoms;
    const size_t gi = (size_t)3 * a.natoms * j + 3 * atom + c;
    if (active) {
        x[3 * j + c] = RRt[gi];
        p[3 * j + c] = PPt[gi];
    }
    __syncthreads();
    double ke = 0.0, k0 = 0.0;
    if (active) {
        const double m = (atom % 3 == 0) ? a.massO : a.massH;
        if (a.nm_ke) {
            const double pt = nm_row(Cs, p, P, j, c, true);
            ke = (1.0 / m) * pt * pt / a.A[4 * P + j];
        } else {
            ke = (1.0 / m) * p[3 * j + c] * p[3 * j + c];
        }
        const double d = x[3 * j + c] - x[3 * ((j + P - 1) % P) + c];
        k0 = m * (d * d);
    }
    for (int o = 16; o > 0; o >>= 1) {
        ke += __shfl_xor_sync(0xffffffffu, ke, o);
        k0 += __shfl_xor_sync(0xffffffffu, k0, o);
    }
    __shared__ double wsum[2][32];
    if ((threadIdx.x & 31) == 0) {
        wsum[0][threadIdx.x >> 5] = ke;
        wsum[1][threadIdx.x >> 5] = k0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            t0 += wsum[0][w];
            t1 += wsum[1][w];
        }
        atomicAdd(sums, 0.5 * t0);
        atomicAdd(sums + 1, t1);
    }
}

// the step's outputs (PIMD_MD_NOUT): sums of the force call, uk, write_out's calc_uk and K0, and
// the estimators of InputOutput.f90:566-571 / estimators.f90:30-96 with the reference's literal
// types (1.5*Natoms and 1.5*Natoms*Nbeads are default-real products)
__global__ void k_md_estimators(int P, int natoms, double volume, double omegan, const double *Upott,
                                const double *virialt, const double *virialct, const double *uk,
                                const double *sums, const double *s_post, double *out, const double *uvv) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double TEMPFACTOR = 0.80181484527, kb = 0.0019872041, PRESSCON2 = 69477.0, MASSCONi = 1.0 / 418.4;
    double U = 0, v = 0, vc = 0;
    if (uvv) {  // Upot, virial, virialc formed by the caller's step (contracted / monomer PIMD)
        U = uvv[0];
        v = uvv[1];
        vc = uvv[2];
    } else {
        for (int k = 0; k < P; k++) {
            U += Upott[k];
            v += virialt[k];
            vc += virialct[k];
        }
        vc = vc / P;
    }
    const int Nw = natoms / 3;
    const double ukm = sums[0], K0raw = sums[1];
    const double sys_temp = TEMPFACTOR * ukm / (double)(natoms * P * P);
    double KE = (double)(1.5f * (float)natoms) * kb * sys_temp;
    const double qE = (KE + 0.5 * (v - vc) / P + U / P) / Nw;
    const double qP = PRESSCON2 * (1 / (3 * volume)) * (2 * KE - vc / P) / Nw;
    KE = (double)((1.5f * (float)natoms) * (float)P) * kb * sys_temp * P;
    const double K0 = 0.5 * K0raw * (omegan * omegan) * MASSCONi;
    out[0] = U;
    out[1] = v;
    out[2] = vc;
    out[3] = *uk;
    out[4] = ukm;
    out[5] = K0raw;
    out[6] = sys_temp;
    out[7] = qE;
    out[8] = qP;
    out[9] = (KE - K0 + U) / (double)(Nw * P);
    out[10] = PRESSCON2 * (1 / (3 * volume)) * (2 * (KE - K0) - v) / Nw;
    out[11] = s_post ? *s_post : 1.0;
}

// one warp: lane-strided bead sums, then a fixed butterfly (FP64 is a narrow pipe on this part:
// a serial loop of dependent adds would take microseconds at the end of every step)
PIMD_D void md_sum_warp(int P, const double *Upott, const double *virialt, const double *virialct, const double *uk,
                           double *out4) {
    if (threadIdx.x >= 32) return;
    double u = 0, v = 0, vc = 0;
    for (int k = threadIdx.x; k < P; k += 32) {
        u += Upott[k];
        v += virialt[k];
        vc += virialct[k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        u += __shfl_xor_sync(0xffffffffu, u, o);
        v += __shfl_xor_sync(0xffffffffu, v, o);
        vc += __shfl_xor_sync(0xffffffffu, vc, o);
    }
    if (threadIdx.x == 0) {
        out4[0] = u;
        out4[1] = v;
        out4[2] = vc / P;
        out4[3] = *uk;
    }
}
__global__ void k_md_sum(int P, const double *Upott, const double *virialt, const double *virialct, const double *uk,
                         double *out4) {
    if (blockIdx.x == 0) md_sum_warp(P, Upott, virialt, virialct, uk, out4);
}

// the step outputs of every replica of a batch: one warp per replica (as k_md_sum)
__global__ void k_md_sum_batch(const NMSumRep *reps) {
    const NMSumRep s = reps[blockIdx.x];
    md_sum_warp(s.P, s.Upott, s.virialt, s.virialct, s.uk, s.out4);
}

// ---------------------------------------------------------------------------------------
void nm_launch_shape(int P, int natoms, int *threads, int *blocks, size_t *smem) {
    int G = 256 / (3 * P);
    if (G < 1) G = 1;
    *threads = ((G * 3 * P + 31) / 32) * 32;  // whole warps (the KE reduction shuffles)
    *blocks = (natoms + G - 1) / G;
    *smem = sizeof(double) * ((size_t)(P + 1) * P + (size_t)G * 9 * P);  // padded C, three vectors per group
}

// above 48 KB of dynamic shared memory (P > 40 beads) the kernels need the opt-in; called
// once per bead count, outside any stream capture
void nm_smem_optin(int P) {
    int threads, blocks;
    size_t smem;
    nm_launch_shape(P, 1, &threads, &blocks, &smem);
    smem = std::max(smem, nm_fast_smem(P, std::max(1, 256 / (3 * P))));
    if (smem <= 48 * 1024) return;
    cudaFuncSetAttribute(k_md_pre, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_md_post, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_evolve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_langevin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_md_pre_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_md_post_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// rows 7-9 of the device table (A12 / msf, A21 msf, c2 sqrt(msf)) from rows 1, 2, 4, 6, and
// row 10 the mode frequencies omegalist (the bead Nose-Hoover chains' 1/tau)
void nm_extend_A(std::vector<double> &A, int P, const std::vector<double> &omegalist) {
    A.resize(11 * (size_t)P);
    for (int j = 0; j < P; j++) {
        const double msf = A[4 * P + j];
        A[7 * P + j] = A[P + j] / msf;
        A[8 * P + j] = A[2 * P + j] * msf;
        A[9 * P + j] = A[6 * P + j] * std::sqrt(msf);
        A[10 * P + j] = omegalist[j];
    }
}

// the MD-step kernels: the exact ones, or for the mixed engine the FP32-pair ones
void nm_launch_md_pre(const NMArgs &a0, cudaStream_t st, double *RRt, double *PPt, const double *dRRt, double *RRc) {
    int threads, blocks;
    size_t smem;
    nm_launch_shape(a0.P, a0.natoms, &threads, &blocks, &smem);
    if (!a0.fast) {
        k_md_pre<<<blocks, threads, smem, st>>>(a0, RRt, PPt, dRRt, RRc);
        return;
    }
    NMArgs a = a0;
    nm_fast_args(a);
    k_md_pre_fast<<<blocks, threads, nm_fast_smem(a.P, std::max(1, 256 / (3 * a.P))), st>>>(a, RRt, PPt, dRRt, RRc);
}
void nm_launch_md_post(const NMArgs &a0, cudaStream_t st, double *PPt, const double *dRRt, double *uk) {
    int threads, blocks;
    size_t smem;
    nm_launch_shape(a0.P, a0.natoms, &threads, &blocks, &smem);
    if (!a0.fast) {
        k_md_post<<<blocks, threads, smem, st>>>(a0, PPt, dRRt, uk);
        return;
    }
    NMArgs a = a0;
    nm_fast_args(a);
    k_md_post_fast<<<blocks, threads, nm_fast_smem(a.P, std::max(1, 256 / (3 * a.P))), st>>>(a, PPt, dRRt, uk);
}

void nm_pair_copy(const std::vector<double> &C, std::vector<double> &out) {
    out = C;
    out.resize(2 * C.size());
    float *f = reinterpret_cast<float *>(out.data() + C.size());
    for (size_t i = 0; i < C.size(); i++) {
        const float h = (float)C[i];
        f[2 * i] = h;
        f[2 * i + 1] = (float)(C[i] - (double)h);
    }
}

static NMArgs nm_args(Engine &E, double massO, double massH) {
    NMArgs a{};
    a.P = E.nm_P;
    a.natoms = E.kp.natoms;
    a.C = E.d_nmC;
    a.A = E.d_nmA;
    a.massO = massO;
    a.massH = massH;
    a.box0 = E.kp.box[0];
    a.boxi0 = E.kp.boxi[0];
    return a;
}

// NormalModes.f90:68-218
void nm_init_host(int P, double omegan, double delta, double setNMfreq, std::vector<double> &A11,
                         std::vector<double> &A12, std::vector<double> &A21, std::vector<double> &A22,
                         std::vector<double> &om, std::vector<double> &msf, std::vector<double> &C) {
    A11.assign(P, 0);
    A12.assign(P, 0);
    A21.assign(P, 0);
    A22.assign(P, 0);
    om.assign(P, 0);
    msf.assign(P, 1.0);
    C.assign((size_t)P * P, 0);
    const int l = (P % 2 == 0) ? (P - 2) / 2 : (P - 1) / 2;
    for (int i = 1; i <= P; i++) {
        C[0 + P * (i - 1)] = std::sqrt(1.0 / P);
        for (int k = 1; k <= l; k++) {
            C[k + P * (i - 1)] = std::sqrt(2.0 / P) * std::cos((double)(k * i) * 2.0 * PI / P);
            C[k + l + P * (i - 1)] = std::sqrt(2.0 / P) * std::sin((double)(k * i) * 2.0 * PI / P);
        }
        if (P % 2 == 0) C[2 * l + 1 + P * (i - 1)] = std::sqrt(1.0 / P) * ((i % 2 == 0) ? 1.0 : -1.0);
    }
    A11[0] = 1.0;
    A12[0] = delta;
    A21[0] = 0.0;
    A22[0] = 1.0;
    auto set_mode = [&](int idx, int k) {
        // NormalModes.f90:126: abs(k)/real(Nbeads) is a single-precision quotient
        const float ratio = (float)std::abs(k) / (float)P;
        const double omega = 2 * omegan * std::sin(PI * (double)ratio);
        om[idx] = omega;
        A11[idx] = std::cos(omega * delta);
        A12[idx] = (1.0 / omega) * std::sin(omega * delta);
        A21[idx] = -omega * std::sin(omega * delta);
        A22[idx] = std::cos(omega * delta);
    };
    for (int k = 1; k <= l; k++) set_mode(k, k);
    for (int k = 1; k <= l; k++) set_mode(k + l, k);
    if (P % 2 == 0) set_mode(2 * l + 1, l + 1);
    if (setNMfreq != 0) {
        const double omega = (2 * PI) * setNMfreq / 33.33333;
        for (int i = 0; i < P; i++) msf[i] = (om[i] == 0) ? 1.0 : (om[i] / omega) * (om[i] / omega);
        const int hi = (P % 2 == 0) ? 2 * l + 1 : 2 * l;
        for (int i = 1; i <= hi; i++) {
            om[i] = omega;
            A11[i] = std::cos(omega * delta);
            A12[i] = (1.0 / omega) * std::sin(omega * delta);
            A21[i] = -omega * std::sin(omega * delta);
            A22[i] = std::cos(omega * delta);
        }
    }
}

}  // namespace pimd

using namespace pimd;

static int nm_err(Engine &E, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PIMD_OK;
    E.last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return PIMD_ERR_CUDA;
}

extern "C" {

int pimd_nm_init(pimd_ctx *ctx, int P, double omegan, double delta, double setNMfreq, double *A11, double *A12,
                 double *A21, double *A22, double *omegalist, double *msf, double *C) {
    if (!ctx || P < 1 || P > 64) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    std::vector<double> a11, a12, a21, a22, om, ms, CC;
    nm_init_host(P, omegan, delta, setNMfreq, a11, a12, a21, a22, om, ms, CC);
    if (E.nm_P != P) {
        if (E.d_nmC) cudaFree(E.d_nmC);
        if (E.d_nmA) cudaFree(E.d_nmA);
        if (cudaMalloc((void **)&E.d_nmC, sizeof(double) * 2 * P * P) != cudaSuccess ||
            cudaMalloc((void **)&E.d_nmA, sizeof(double) * 11 * P) != cudaSuccess)
            return PIMD_ERR_NOMEM;
        E.nm_P = P;
        nm_smem_optin(P);
    }
    if (!E.d_nh) {  // chain state and step sums: vxi_global = 1 (InputOutput.f90:397), uk = 0
        if (cudaMalloc((void **)&E.d_nh, sizeof(double) * 8) != cudaSuccess) return PIMD_ERR_NOMEM;
        E.allocs.push_back(E.d_nh);
        const double init[8] = {1.0, 1.0, 0.0, 1.0, 1.0, 0.0, 0.0, 0.0};
        cudaMemcpy(E.d_nh, init, sizeof init, cudaMemcpyHostToDevice);
    }
    std::vector<double> A(7 * P, 0.0);
    for (int j = 0; j < P; j++) {
        A[j] = a11[j];
        A[P + j] = a12[j];
        A[2 * P + j] = a21[j];
        A[3 * P + j] = a22[j];
        A[4 * P + j] = ms[j];
        A[5 * P + j] = 1.0;  // c1, c2 until pimd_langevin_init
        A[6 * P + j] = 0.0;
    }
    E.h_nm = A;
    E.h_nm.insert(E.h_nm.end(), om.begin(), om.end());
    E.h_nmC = CC;
    std::vector<double> CP;
    nm_pair_copy(CC, CP);
    cudaMemcpy(E.d_nmC, CP.data(), sizeof(double) * CP.size(), cudaMemcpyHostToDevice);
    nm_extend_A(A, P, om);
    cudaMemcpy(E.d_nmA, A.data(), sizeof(double) * 11 * P, cudaMemcpyHostToDevice);
    E.nm_omegan = omegan;
    E.nm_setfreq = setNMfreq;
    auto out = [&](double *dst, const std::vector<double> &v) {
        if (dst) std::memcpy(dst, v.data(), sizeof(double) * v.size());
    };
    out(A11, a11);
    out(A12, a12);
    out(A21, a21);
    out(A22, a22);
    out(omegalist, om);
    out(msf, ms);
    out(C, CC);
    return nm_err(E, cudaGetLastError(), "nm_init");
}

// real2NM / NM2real (NormalModes.f90:308-341) on the host: out(:,j) = sum_k C(j,k) A(:,k) (fwd)
// or sum_k C(k,j) A(:,k), accumulated in k order as the reference's loops
static void nm_host_transform(const std::vector<double> &C, int P, const double *A, double *out, bool fwd) {
    std::vector<double> r(3 * (size_t)P, 0.0);
    for (int j = 0; j < P; j++)
        for (int k = 0; k < P; k++) {
            const double c = fwd ? C[j + (size_t)P * k] : C[k + (size_t)P * j];
            for (int x = 0; x < 3; x++) r[3 * j + x] = r[3 * j + x] + c * A[3 * k + x];
        }
    std::memcpy(out, r.data(), sizeof(double) * 3 * P);
}

// standard normal draws of the context's host generator (splitmix64 words, Box-Muller)
static void host_normals(Engine &E, double *xi, int n) {
    auto next = [&E]() {
        unsigned long long z = (E.host_rng += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    for (int i = 0; i < n; i += 2) {
        const double u1 = ((double)(next() >> 11) + 1.0) * 0x1.0p-53, u2 = (double)(next() >> 11) * 0x1.0p-53;
        const double r = std::sqrt(-2.0 * std::log(u1));
        xi[i] = r * std::cos(2.0 * PI * u2);
        if (i + 1 < n) xi[i + 1] = r * std::sin(2.0 * PI * u2);
    }
}

int pimd_real2nm(pimd_ctx *ctx, const double *A, double *out, int P) {
    if (!ctx || !A || !out || P != ctx->E.nm_P || ctx->E.h_nmC.empty()) return PIMD_ERR_ARG;
    nm_host_transform(ctx->E.h_nmC, P, A, out, true);
    return PIMD_OK;
}

int pimd_nm2real(pimd_ctx *ctx, const double *A, double *out, int P) {
    if (!ctx || !A || !out || P != ctx->E.nm_P || ctx->E.h_nmC.empty()) return PIMD_ERR_ARG;
    nm_host_transform(ctx->E.h_nmC, P, A, out, false);
    return PIMD_OK;
}

// gen_rand_ring (NormalModes.f90:224-250): the free ring polymer at temp -- normal mode j drawn with
// standard deviation sqrt(omegan hbar / (mass msf_j omega_j^2)), omegan = kB temp Nbeads / hbar,
// the centroid (omega = 0) at zero -- then NM2real
int pimd_gen_rand_ring(pimd_ctx *ctx, double *RR, double mass, double temp, int P, const double *xi) {
    if (!ctx || !RR || P != ctx->E.nm_P || ctx->E.h_nmC.empty() || !(mass > 0) || !(temp > 0)) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    std::vector<double> x(3 * (size_t)P), tr(3 * (size_t)P, 0.0);
    if (xi) std::memcpy(x.data(), xi, sizeof(double) * 3 * P);
    else host_normals(E, x.data(), 3 * P);
    const double *om = E.h_nm.data() + 7 * (size_t)P, *msf = E.h_nm.data() + 4 * (size_t)P;
    const double omegan = KB_AMU * temp * P / HBAR;
    for (int j = 0; j < P; j++) {
        if (om[j] == 0.0) continue;
        const double sd = std::sqrt((omegan * HBAR) / (mass * msf[j] * (om[j] * om[j])));
        for (int c = 0; c < 3; c++) tr[3 * j + c] = sd * x[3 * j + c];
    }
    nm_host_transform(E.h_nmC, P, tr.data(), RR, false);
    return PIMD_OK;
}

// gen_rand_ring_momenta (NormalModes.f90:257-275): mode momenta with standard deviation
// sqrt(kB mass msf_j temp) (the caller passes temp*Nbeads, main_stuff.f90:306), then NM2real
int pimd_gen_rand_ring_momenta(pimd_ctx *ctx, double *PP, double mass, double temp, int P, const double *xi) {
    if (!ctx || !PP || P != ctx->E.nm_P || ctx->E.h_nmC.empty() || !(mass > 0) || !(temp > 0)) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    std::vector<double> x(3 * (size_t)P), tr(3 * (size_t)P);
    if (xi) std::memcpy(x.data(), xi, sizeof(double) * 3 * P);
    else host_normals(E, x.data(), 3 * P);
    const double *msf = E.h_nm.data() + 4 * (size_t)P;
    for (int j = 0; j < P; j++) {
        const double sd = std::sqrt(KB_AMU * mass * msf[j] * temp);
        for (int c = 0; c < 3; c++) tr[3 * j + c] = sd * x[3 * j + c];
    }
    nm_host_transform(E.h_nmC, P, tr.data(), PP, false);
    return PIMD_OK;
}

int pimd_langevin_init(pimd_ctx *ctx, double delt2, int centroid_thermostat, double tau_centroid, double temp_P) {
    if (!ctx) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (!E.nm_P) return PIMD_ERR_STATE;
    const int P = E.nm_P;
    std::vector<double> &A = E.h_nm;
    const double *om = A.data() + 7 * P;
    for (int i = 0; i < P; i++) {
        double gammak = (i == 0) ? (centroid_thermostat ? 1.0 / tau_centroid : 0.0) : 2 * om[i];
        const double c1 = std::exp(-delt2 * gammak);
        double c2 = std::sqrt(1 - c1 * c1);
        c2 = std::sqrt(KB_AMU * temp_P) * c2;
        A[5 * P + i] = c1;
        A[6 * P + i] = c2;
    }
    std::vector<double> Ad(A.begin(), A.begin() + 7 * P);
    nm_extend_A(Ad, P, std::vector<double>(om, om + P));
    cudaSetDevice(E.device);
    return nm_err(E, cudaMemcpy(E.d_nmA, Ad.data(), sizeof(double) * 11 * P, cudaMemcpyHostToDevice), "langevin_init");
}

int pimd_evolve_ring(pimd_ctx *ctx, double *RR, double *PP, int P, double mass) {
    if (!ctx || !RR || !PP || P != ctx->E.nm_P) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    double *d;
    if (cudaMalloc((void **)&d, sizeof(double) * 6 * P) != cudaSuccess) return PIMD_ERR_NOMEM;
    cudaMemcpy(d, RR, sizeof(double) * 3 * P, cudaMemcpyHostToDevice);
    cudaMemcpy(d + 3 * P, PP, sizeof(double) * 3 * P, cudaMemcpyHostToDevice);
    NMArgs a = nm_args(E, mass, mass);
    a.natoms = 1;
    int threads, blocks;
    size_t smem;
    nm_launch_shape(P, 1, &threads, &blocks, &smem);
    k_evolve<<<blocks, threads, smem, E.stream>>>(a, d, d + 3 * P); ++E.nlaunch;
    cudaMemcpyAsync(RR, d, sizeof(double) * 3 * P, cudaMemcpyDeviceToHost, E.stream);
    cudaMemcpyAsync(PP, d + 3 * P, sizeof(double) * 3 * P, cudaMemcpyDeviceToHost, E.stream);
    cudaError_t e = cudaStreamSynchronize(E.stream);
    cudaFree(d);
    return nm_err(E, e, "evolve_ring");
}

int pimd_evolve_all_device(pimd_ctx *ctx, double *RRt, double *PPt, double massO, double massH) {
    if (!ctx || !RRt || !PPt || !ctx->E.nm_P) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    NMArgs a = nm_args(E, massO, massH);
    int threads, blocks;
    size_t smem;
    nm_launch_shape(a.P, a.natoms, &threads, &blocks, &smem);
    k_evolve<<<blocks, threads, smem, E.stream>>>(a, RRt, PPt); ++E.nlaunch;
    return nm_err(E, cudaGetLastError(), "evolve_all");
}

int pimd_langevin_nm_device(pimd_ctx *ctx, double *PPt, const double *xi, double massO, double massH,
                            unsigned long long seed, unsigned long long counter) {
    if (!ctx || !PPt || !ctx->E.nm_P) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    NMArgs a = nm_args(E, massO, massH);
    a.xi = xi;
    a.seed = seed;
    a.counter = counter;
    a.langevin = 1;
    int threads, blocks;
    size_t smem;
    nm_launch_shape(a.P, a.natoms, &threads, &blocks, &smem);
    k_langevin<<<blocks, threads, smem, E.stream>>>(a, PPt); ++E.nlaunch;
    return nm_err(E, cudaGetLastError(), "langevin_nm");
}

}  // extern "C"

namespace pimd {
// The integrator kernels' arguments for one MD step of the context (first half: phase 0, the
// pre-kick thermostat draws xi1)
NMArgs nm_step_args(Engine &E, const pimd_md_params *mp, const double *xi1) {
    NMArgs a = nm_args(E, mp->massO, mp->massH);
    a.delt = mp->delt;
    a.delt2 = mp->delt / 2.0;
    a.langevin = mp->langevin;
    a.evolve = E.kp.P > 1;
    a.seed = mp->seed;
    a.tstep = E.kp.dstep;
    a.phase = 0;
    a.xi = xi1;
    a.nm_ke = (E.nm_setfreq != 0 && E.kp.P > 1) ? 1 : 0;
    a.bead_nh = E.nh_bead ? 1 : 0;
    a.centroid_nh = E.nh_centroid ? 1 : 0;
    a.tau_centroid = E.nh_tau_centroid;
    a.nh_temp = E.nh_temp;
    a.vxib = E.d_vxib;
    // the FP32-pair kernels of the mixed engine carry PILE only: the chains and the normal-mode
    // kinetic energy run in the exact kernels
    a.fast = E.precision == PIMD_MIXED && !E.nh_bead && !E.nh_global && !a.nm_ke;
    return a;
}

// launchers for the contracted / monomer-PIMD step (contracted.cu)
void nm_launch_evolve(const NMArgs &a, cudaStream_t st, double *RRt, double *PPt) {
    int threads, blocks;
    size_t smem;
    nm_launch_shape(a.P, a.natoms, &threads, &blocks, &smem);
    k_evolve<<<blocks, threads, smem, st>>>(a, RRt, PPt);
}
void nm_launch_ring_sums(const NMArgs &a, cudaStream_t st, const double *RRt, const double *PPt, double *sums) {
    int threads, blocks;
    size_t smem;
    nm_launch_shape(a.P, a.natoms, &threads, &blocks, &smem);
    cudaMemsetAsync(sums, 0, 2 * sizeof(double), st);
    k_ring_sums<<<blocks, threads, smem, st>>>(a, RRt, PPt, sums);
}
void nm_launch_nh_global(Engine &E, const double *uk_end, int slot, double delt2) {
    k_nh_global<<<1, 32, 0, E.stream>>>(E.d_nh, uk_end, slot, E.nh_tau, delt2, 3 * E.kp.natoms * E.kp.P, E.nh_temp);
}
void nm_launch_nh_scale(Engine &E, double *PPt) {
    const size_t n = (size_t)3 * E.kp.natoms * E.kp.P;
    k_nh_scale<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, E.stream>>>(PPt, n, E.d_nh + 4);
}
void nm_launch_estimators(Engine &E, const double *uk, const double *uvv, double *out) {
    k_md_estimators<<<1, 32, 0, E.stream>>>(E.kp.P, E.kp.natoms, E.kp.volume, E.nm_omegan, nullptr, nullptr, nullptr,
                                            uk, E.d_nh + 5, E.nh_global ? E.d_nh + 4 : nullptr, out, uvv);
}
}  // namespace pimd

extern "C" {

// Enqueue one PIMD_VV step on the context's stream (everything but the step word, which the
// force call or the graph launcher sets). out4: [Upot, virial, virialc, uk]; outx: the
// PIMD_MD_NOUT outputs with write_out's calc_uk, K0 and the estimators (either may be null).
static int md_step_enqueue(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt,
                           double *RRc, const double *xi1, const double *xi2, int t, double *out4, double *outx) {
    Engine &E = ctx->E;
    NMArgs a = nm_step_args(E, mp, xi1);
    const int L = 3 * E.kp.natoms * E.kp.P;
    int threads, blocks;
    size_t smem;
    nm_launch_shape(a.P, a.natoms, &threads, &blocks, &smem);
    if (!E.capturing) launch_set_step(E, t);  // the Langevin counter of k_md_pre reads t
    timer_begin(E, "md_pre");
    if (E.nh_global) {
        k_nh_global<<<1, 32, 0, E.stream>>>(E.d_nh, nullptr, 3, E.nh_tau, a.delt2, L, E.nh_temp);
        ++E.nlaunch;
        a.s_pre = E.d_nh + 3;
    }
    nm_launch_md_pre(a, E.stream, RRt, PPt, dRRt, RRc); ++E.nlaunch;
    a.s_pre = nullptr;
    if (outx) {
        cudaMemsetAsync(E.d_nh + 5, 0, 2 * sizeof(double), E.stream);
        k_ring_sums<<<blocks, threads, smem, E.stream>>>(a, RRt, PPt, E.d_nh + 5);
        ++E.nlaunch;
    }
    timer_end(E);
    KP saved = E.kp;
    E.kp.RRt = RRt;
    E.kp.RRc = RRc;
    E.kp.dRRt = dRRt;
    double *d = E.d_out;  // Upott, virialt, virialct (3P) then uk
    int rc = run_forces(E, t, ctx->check_every, d, d + E.kp.P, d + 2 * E.kp.P, nullptr);
    E.kp.RRt = saved.RRt;
    E.kp.RRc = saved.RRc;
    E.kp.dRRt = saved.dRRt;
    if (rc) return rc;
    double *uk = d + 3 * E.kp.P;
    cudaMemsetAsync(uk, 0, sizeof(double), E.stream);
    a.xi = xi2;
    a.phase = 1;
    timer_begin(E, "md_post");
    nm_launch_md_post(a, E.stream, PPt, dRRt, uk); ++E.nlaunch;
    const double *ukout = uk;
    if (E.nh_global) {
        k_nh_global<<<1, 32, 0, E.stream>>>(E.d_nh, uk, 4, E.nh_tau, a.delt2, L, E.nh_temp);
        const size_t n = (size_t)3 * E.kp.natoms * E.kp.P;
        k_nh_scale<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, E.stream>>>(PPt, n, E.d_nh + 4);
        E.nlaunch += 2;
        ukout = E.d_nh + 2;
    } else if (E.d_nh) {
        // the module variable uk follows calc_uk when no global chain runs (MD.f90:99)
        cudaMemcpyAsync(E.d_nh + 2, uk, sizeof(double), cudaMemcpyDeviceToDevice, E.stream);
    }
    if (out4) {
        k_md_sum<<<1, 32, 0, E.stream>>>(E.kp.P, d, d + E.kp.P, d + 2 * E.kp.P, ukout, out4);
        ++E.nlaunch;
    }
    if (outx) {
        k_md_estimators<<<1, 32, 0, E.stream>>>(E.kp.P, E.kp.natoms, E.kp.volume, E.nm_omegan, d, d + E.kp.P,
                                                d + 2 * E.kp.P, ukout, E.d_nh + 5, E.nh_global ? E.d_nh + 4 : nullptr,
                                                outx, nullptr);
        ++E.nlaunch;
    }
    timer_end(E);
    return nm_err(E, cudaGetLastError(), "md_step");
}

// Graph mode: the step is captured once per set of buffers and parameters (the dipole loop as a
// conditional while node) and replayed; only the step word is written before each launch.
static int md_step_graph(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt,
                         double *RRc, const double *xi1, const double *xi2, int t, double *out4, double *outx) {
    Engine &E = ctx->E;
    double mpv[3] = {mp->delt, mp->massO, mp->massH};
    std::vector<const void *> key = {RRt, PPt, dRRt, RRc, xi1, xi2, out4, outx, (const void *)(size_t)mp->langevin,
                                     (const void *)(size_t)mp->seed, (const void *)(size_t)E.nh_gen};
    for (double v : mpv) {
        unsigned long long u;
        std::memcpy(&u, &v, sizeof u);
        key.push_back((const void *)(size_t)u);
    }
    if (!E.gexec || key != E.gkey) {
        if (E.gexec) {
            cudaGraphExecDestroy(E.gexec);
            E.gexec = nullptr;
        }
        if (!E.body_stream && cudaStreamCreateWithFlags(&E.body_stream, cudaStreamNonBlocking) != cudaSuccess)
            return nm_err(E, cudaGetLastError(), "body stream");
        cudaError_t e = cudaStreamBeginCapture(E.stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return nm_err(E, e, "graph capture");
        const bool timers_on = E.timers.on;
        E.timers.on = false;  // event records cannot sit inside a conditional body
        E.capturing = true;
        int rc = md_step_enqueue(ctx, mp, RRt, PPt, dRRt, RRc, xi1, xi2, t, out4, outx);
        E.capturing = false;
        E.timers.on = timers_on;
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(E.stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return nm_err(E, e, "graph capture end");
        e = cudaGraphInstantiate(&E.gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return nm_err(E, e, "graph instantiate");
        E.gkey = key;
        E.graph_captures++;
    }
    launch_set_step(E, t);
    timer_begin(E, "md_graph");
    cudaError_t e = cudaGraphLaunch(E.gexec, E.stream);
    timer_end(E);
    E.graph_launches++;
    return nm_err(E, e, "graph launch");
}

static int md_step_any(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt, double *RRc,
                       const double *xi1, const double *xi2, int t, double *out4, double *outx) {
    if (!ctx || !mp || !RRt || !PPt || !dRRt || !RRc) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (E.nm_P != E.kp.P) return PIMD_ERR_STATE;
    if (E.nh_bead && mp->langevin) {
        E.last_error = "md_step: Langevin_NM and the bead Nose-Hoover chains exclude each other";
        return PIMD_ERR_ARG;
    }
    cudaSetDevice(E.device);
    if (E.graph_mode) return md_step_graph(ctx, mp, RRt, PPt, dRRt, RRc, xi1, xi2, t, out4, outx);
    return md_step_enqueue(ctx, mp, RRt, PPt, dRRt, RRc, xi1, xi2, t, out4, outx);
}

int pimd_md_step_device(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt, double *RRc,
                        const double *xi1, const double *xi2, int t, double *out4) {
    return md_step_any(ctx, mp, RRt, PPt, dRRt, RRc, xi1, xi2, t, out4, nullptr);
}

int pimd_md_step_ex_device(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt,
                           double *RRc, const double *xi1, const double *xi2, int t, double *out) {
    if (!out) return PIMD_ERR_ARG;
    return md_step_any(ctx, mp, RRt, PPt, dRRt, RRc, xi1, xi2, t, nullptr, out);
}

int pimd_set_thermostat(pimd_ctx *ctx, const pimd_thermostat *th) {
    if (!ctx || !th) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (!E.nm_P || !E.d_nh) return PIMD_ERR_STATE;
    if ((th->bead_thermostat != 0 && th->bead_thermostat != 2) || (th->global_thermostat && !(th->tau > 0)) ||
        !(th->temp > 0) || (th->bead_thermostat == 2 && th->centroid_thermostat && !(th->tau_centroid > 0)))
        return PIMD_ERR_ARG;
    cudaSetDevice(E.device);
    const int P = E.nm_P, na = E.kp.natoms;
    if (th->bead_thermostat == 2 && P < 2) return PIMD_ERR_ARG;  // InputOutput.f90:258-264
    if (th->bead_thermostat == 2 && !E.d_vxib) {
        if (cudaMalloc((void **)&E.d_vxib, sizeof(double) * 6 * (size_t)na * P) != cudaSuccess) return PIMD_ERR_NOMEM;
        E.allocs.push_back(E.d_vxib);
        cudaMemset(E.d_vxib, 0, sizeof(double) * 6 * (size_t)na * P);  // vxi_beads = 0 (InputOutput.f90:400-403)
    }
    E.nh_global = th->global_thermostat != 0;
    E.nh_bead = th->bead_thermostat == 2;
    E.nh_centroid = E.nh_bead && th->centroid_thermostat != 0;
    E.nh_tau = th->tau;
    E.nh_temp = th->temp * P;  // MD.f90:44 and main_stuff.f90:157, 165 pass temp*Nbeads
    E.nh_tau_centroid = th->tau_centroid;
    E.nh_gen++;
    return nm_err(E, cudaDeviceSynchronize(), "set_thermostat");
}

int pimd_get_thermostat_state(pimd_ctx *ctx, double *vxi_global, double *uk, double *vxi_beads) {
    if (!ctx) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (!E.d_nh) return PIMD_ERR_STATE;
    cudaSetDevice(E.device);
    double h[8];
    cudaError_t e = cudaStreamSynchronize(E.stream);
    if (e == cudaSuccess) e = cudaMemcpy(h, E.d_nh, sizeof h, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return nm_err(E, e, "get_thermostat_state");
    if (vxi_global) {
        vxi_global[0] = h[0];
        vxi_global[1] = h[1];
    }
    if (uk) *uk = h[2];
    if (vxi_beads) {
        if (!E.d_vxib) return PIMD_ERR_STATE;
        e = cudaMemcpy(vxi_beads, E.d_vxib, sizeof(double) * 6 * (size_t)E.kp.natoms * E.nm_P, cudaMemcpyDeviceToHost);
    }
    return nm_err(E, e, "get_thermostat_state");
}

int pimd_set_thermostat_state(pimd_ctx *ctx, const double *vxi_global, double uk, const double *vxi_beads) {
    if (!ctx) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (!E.d_nh) return PIMD_ERR_STATE;
    if (vxi_beads && !E.d_vxib) return PIMD_ERR_STATE;
    cudaSetDevice(E.device);
    cudaError_t e = cudaStreamSynchronize(E.stream);
    if (e == cudaSuccess && vxi_global) e = cudaMemcpy(E.d_nh, vxi_global, 2 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(E.d_nh + 2, &uk, sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && vxi_beads)
        e = cudaMemcpy(E.d_vxib, vxi_beads, sizeof(double) * 6 * (size_t)E.kp.natoms * E.nm_P, cudaMemcpyHostToDevice);
    return nm_err(E, e, "set_thermostat_state");
}

int pimd_set_graph(pimd_ctx *ctx, int enable) {
    if (!ctx) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    E.graph_mode = enable != 0;
    if (!E.graph_mode && E.gexec) {
        cudaSetDevice(E.device);
        cudaStreamSynchronize(E.stream);
        cudaGraphExecDestroy(E.gexec);
        E.gexec = nullptr;
        E.gkey.clear();
    }
    return PIMD_OK;
}

int pimd_graph_info(pimd_ctx *ctx, long long *captures, long long *launches) {
    if (!ctx) return PIMD_ERR_ARG;
    if (captures) *captures = ctx->E.graph_captures;
    if (launches) *launches = ctx->E.graph_launches;
    return PIMD_OK;
}

// ---- exact restart file ---------------------------------------------------------------------
// Little-endian binary (the byte order of both host architectures this builds for):
//   "PIMDCKPT", int32 version 1, int32 natoms, nbeads, pot_model, precision, sites S, t,
//   flags (1: bead chains, 2: global chain), uint64 seed,
//   RRt, PPt, dRRt (3 Natoms P doubles each), the predictor history (P x 4 x S x 3 doubles),
//   the chain state [vxi1, vxi2, uk] and, with the bead chains, vxi_beads (6 Natoms P doubles).
struct CkptHead {
    char magic[8];
    int32_t version, natoms, nbeads, pot_model, precision, sites, t, flags;
    uint64_t seed;
};

int pimd_checkpoint_write(pimd_ctx *ctx, const char *path, const double *RRt, const double *PPt, const double *dRRt,
                          int t, unsigned long long seed) {
    if (!ctx || !path || !RRt || !PPt || !dRRt) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    const size_t n = (size_t)3 * E.kp.natoms * E.kp.P, nh = (size_t)E.kp.P * 4 * E.kp.S * 3;
    const size_t nb = E.nh_bead && E.d_vxib ? (size_t)6 * E.kp.natoms * E.kp.P : 0;
    std::vector<double> hist(nh), chain(3, 0.0), vb(nb);
    cudaError_t e = cudaStreamSynchronize(E.stream);
    if (e == cudaSuccess) e = cudaMemcpy(hist.data(), E.kp.txdip, sizeof(double) * nh, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && E.d_nh) e = cudaMemcpy(chain.data(), E.d_nh, sizeof(double) * 3, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nb) e = cudaMemcpy(vb.data(), E.d_vxib, sizeof(double) * nb, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return nm_err(E, e, "checkpoint_write");
    CkptHead h{};
    std::memcpy(h.magic, "PIMDCKPT", 8);
    h.version = 1;
    h.natoms = E.kp.natoms;
    h.nbeads = E.kp.P;
    h.pot_model = E.kp.model;
    h.precision = E.precision;
    h.sites = E.kp.S;
    h.t = t;
    h.flags = (nb ? 1 : 0) | (E.nh_global ? 2 : 0);
    h.seed = seed;
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        E.last_error = std::string("checkpoint_write: cannot open ") + path;
        return PIMD_ERR_ARG;
    }
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 && std::fwrite(RRt, sizeof(double), n, f) == n &&
              std::fwrite(PPt, sizeof(double), n, f) == n && std::fwrite(dRRt, sizeof(double), n, f) == n &&
              std::fwrite(hist.data(), sizeof(double), nh, f) == nh && std::fwrite(chain.data(), sizeof(double), 3, f) == 3 &&
              (nb == 0 || std::fwrite(vb.data(), sizeof(double), nb, f) == nb);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) E.last_error = "checkpoint_write: write failed";
    return ok ? PIMD_OK : PIMD_ERR_ARG;
}

int pimd_checkpoint_read(pimd_ctx *ctx, const char *path, double *RRt, double *PPt, double *dRRt, int *t,
                         unsigned long long *seed) {
    if (!ctx || !path || !RRt || !PPt || !dRRt) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        E.last_error = std::string("checkpoint_read: cannot open ") + path;
        return PIMD_ERR_ARG;
    }
    CkptHead h{};
    bool ok = std::fread(&h, sizeof h, 1, f) == 1 && std::memcmp(h.magic, "PIMDCKPT", 8) == 0 && h.version == 1;
    if (ok && (h.natoms != E.kp.natoms || h.nbeads != E.kp.P || h.pot_model != E.kp.model || h.sites != E.kp.S ||
               ((h.flags & 1) && !(E.nh_bead && E.d_vxib)))) {
        E.last_error = "checkpoint_read: the file's system or thermostats differ from this context's";
        std::fclose(f);
        return PIMD_ERR_ARG;
    }
    const size_t n = (size_t)3 * E.kp.natoms * E.kp.P, nh = (size_t)E.kp.P * 4 * E.kp.S * 3;
    const size_t nb = (h.flags & 1) ? (size_t)6 * E.kp.natoms * E.kp.P : 0;
    std::vector<double> hist(nh), chain(3), vb(nb);
    ok = ok && std::fread(RRt, sizeof(double), n, f) == n && std::fread(PPt, sizeof(double), n, f) == n &&
         std::fread(dRRt, sizeof(double), n, f) == n && std::fread(hist.data(), sizeof(double), nh, f) == nh &&
         std::fread(chain.data(), sizeof(double), 3, f) == 3 && (nb == 0 || std::fread(vb.data(), sizeof(double), nb, f) == nb);
    std::fclose(f);
    if (!ok) {
        E.last_error = "checkpoint_read: not a complete checkpoint file of this format";
        return PIMD_ERR_ARG;
    }
    cudaError_t e = cudaStreamSynchronize(E.stream);
    if (e == cudaSuccess) e = cudaMemcpy(E.kp.txdip, hist.data(), sizeof(double) * nh, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && E.d_nh) e = cudaMemcpy(E.d_nh, chain.data(), sizeof(double) * 3, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nb) e = cudaMemcpy(E.d_vxib, vb.data(), sizeof(double) * nb, cudaMemcpyHostToDevice);
    if (t) *t = h.t;
    if (seed) *seed = h.seed;
    return nm_err(E, e, "checkpoint_read");
}

static int md_step_host(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt, double *RRc,
                        const double *xi1, const double *xi2, int t, double *out, int nout) {
    if (!ctx || !mp || !RRt || !PPt || !dRRt) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    cudaSetDevice(E.device);
    const size_t n = (size_t)E.kp.P * E.kp.natoms * 3, nc = (size_t)E.kp.natoms * 3;
    if (!E.d_md) {
        // device copies of the MD state: RRt, PPt, dRRt, RRc, xi1, xi2, and the step's outputs
        if (cudaMalloc((void **)&E.d_md, sizeof(double) * (5 * n + nc + 16)) != cudaSuccess) return PIMD_ERR_NOMEM;
        E.allocs.push_back(E.d_md);
    }
    double *dR = E.d_md, *dP = dR + n, *dG = dP + n, *dx1 = dG + n, *dx2 = dx1 + n, *dC = dx2 + n, *dO = dC + nc;
    cudaMemcpyAsync(dR, RRt, sizeof(double) * n, cudaMemcpyHostToDevice, E.stream);
    cudaMemcpyAsync(dP, PPt, sizeof(double) * n, cudaMemcpyHostToDevice, E.stream);
    cudaMemcpyAsync(dG, dRRt, sizeof(double) * n, cudaMemcpyHostToDevice, E.stream);
    if (xi1) cudaMemcpyAsync(dx1, xi1, sizeof(double) * n, cudaMemcpyHostToDevice, E.stream);
    if (xi2) cudaMemcpyAsync(dx2, xi2, sizeof(double) * n, cudaMemcpyHostToDevice, E.stream);
    int rc = md_step_any(ctx, mp, dR, dP, dG, dC, xi1 ? dx1 : nullptr, xi2 ? dx2 : nullptr, t,
                         nout == 4 ? dO : nullptr, nout == 4 ? nullptr : dO);
    if (rc) return rc;
    cudaMemcpyAsync(RRt, dR, sizeof(double) * n, cudaMemcpyDeviceToHost, E.stream);
    cudaMemcpyAsync(PPt, dP, sizeof(double) * n, cudaMemcpyDeviceToHost, E.stream);
    cudaMemcpyAsync(dRRt, dG, sizeof(double) * n, cudaMemcpyDeviceToHost, E.stream);
    if (RRc) cudaMemcpyAsync(RRc, dC, sizeof(double) * nc, cudaMemcpyDeviceToHost, E.stream);
    if (out) cudaMemcpyAsync(out, dO, sizeof(double) * nout, cudaMemcpyDeviceToHost, E.stream);
    return nm_err(E, cudaStreamSynchronize(E.stream), "md_step");
}

int pimd_md_step(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt, double *RRc,
                 const double *xi1, const double *xi2, int t, double *out4) {
    return md_step_host(ctx, mp, RRt, PPt, dRRt, RRc, xi1, xi2, t, out4, 4);
}

int pimd_md_step_ex(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt, double *RRc,
                    const double *xi1, const double *xi2, int t, double *out) {
    if (!out) return PIMD_ERR_ARG;
    return md_step_host(ctx, mp, RRt, PPt, dRRt, RRc, xi1, xi2, t, out, PIMD_MD_NOUT);
}

}  // extern "C"
