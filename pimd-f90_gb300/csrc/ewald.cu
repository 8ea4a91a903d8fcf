// ewald.cu -- Ewald reciprocal-space sums for all beads.
// Restates pot_ttm/ewald.f90: ssincos (403-437), ewald_std_qq (1-52), ewald_std_dd (56-119),
// ewald_std_qd (123-226), with the k-vector list of ewald_set (293-378).
//
// Structure factors S(k) = sum_s w_s e^{i k.r_s} are k-parallel: a block stages a tile of
// sites' e^{i kz z} tables and the per-(kx,ky)-run products e^{i(kx x + ky y)} in shared
// memory, and each thread owns one k-vector and sums over the tile. Per-tile partial sums go
// to HBM and a second kernel adds them in FP64 in a fixed order (deterministic, no atomics).
//
// Fields at the sites are site-parallel: each thread owns one site and walks the k-list run
// by run, using e^{ik.r} = e^{i(kx x+ky y)} e^{i kz z} so that inside a run only the kz
// factor changes: U0 = sum_kz e^{i kz z} W_k, U1 = sum_kz e^{i kz z} W_k kz, then
// E += Im(e^{i(kx x+ky y)} U0) (kx, ky) + Im(e^{i(kx x+ky y)} U1) z-hat, phi += Re(...).
//
// Precision: the template type R is the arithmetic of the phases and per-tile / per-chunk
// sums (double in the FP64 engine, float in the mixed engine). The e^{i n 2pi x/L} tables
// always come from the FP64 recurrence (k.r reduced in FP64) and are stored as R; tile
// partials and chunk partials are added in FP64.
#include <algorithm>

#include "dipole_check.cuh"
#include "engine.h"

namespace pimd {

template <typename R>
struct C2;
template <>
struct C2<double> {
    using T = double2;
    PIMD_D static T make(double x, double y) { return make_double2(x, y); }
};
template <>
struct C2<float> {
    using T = float2;
    PIMD_D static T make(float x, float y) { return make_float2(x, y); }
};

template <typename V>
PIMD_D V cmul(V a, V b) {
    V r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.y * b.x + a.x * b.y;
    return r;
}
template <typename V>
PIMD_D V cconj(V a) {
    a.y = -a.y;
    return a;
}

template <typename R>
PIMD_D typename C2<R>::T *tab_base(const KP &kp);
template <>
PIMD_D double2 *tab_base<double>(const KP &kp) {
    return kp.tab;
}
template <>
PIMD_D float2 *tab_base<float>(const KP &kp) {
    return kp.tabf;
}

// ewald.f90:403-437 ssincos: cos/sin(2 pi n x / L) for n = 0..nmax by the angle-addition
// recurrence from n = 1, each product and sum rounded separately like the reference.
template <typename R>
__global__ void __launch_bounds__(128) k_ewald_tables(KP kp) {
    using V = typename C2<R>::T;
    const int s = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (s >= kp.S) return;
    const double4_32a r = kp.pos[(size_t)b * kp.S + s];
    const double xyz[3] = {r.x, r.y, r.z};
    const int nmx[3] = {kp.hmax, kp.kmax, kp.lmax};
    int off = 0;
    V *T = tab_base<R>(kp) + (size_t)b * kp.ntab * kp.S + s;
    for (int d = 0; d < 3; d++) {
        T[(size_t)off * kp.S] = C2<R>::make(R(1), R(0));
        if (nmx[d] >= 1) {
            const double arg = __dmul_rn(__dmul_rn(TWOPI, kp.boxi[d]), xyz[d]);
            const double c1 = cos(arg), s1 = sin(arg);
            double c = c1, sn = s1;
            T[(size_t)(off + 1) * kp.S] = C2<R>::make(R(c1), R(s1));
            for (int n = 2; n <= nmx[d]; n++) {
                const double cn = __dsub_rn(__dmul_rn(c, c1), __dmul_rn(sn, s1));
                const double snn = __dadd_rn(__dmul_rn(c, s1), __dmul_rn(sn, c1));
                c = cn;
                sn = snn;
                T[(size_t)(off + n) * kp.S] = C2<R>::make(R(c), R(sn));
            }
        }
        off += nmx[d] + 1;
    }
}

// The FP32 tables of the mixed engine without the FP64 recurrence: the site's coordinate as a
// 32-bit fraction u of the box edge (wrapped, rounded once from FP64), n u modulo 2^32 is the
// exact phase fraction of harmonic n (a wrapping integer multiply), read as signed it is the
// angle pi ph / 2^31 in [-pi, pi) for sincospif. Each entry carries only FP32 rounding (of the
// phase and of the sine and cosine), like the rounded FP64 recurrence it replaces.
__global__ void __launch_bounds__(128) k_ewald_tables_m(KP kp) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (s >= kp.S) return;
    const double4_32a r = kp.pos[(size_t)b * kp.S + s];
    const double xyz[3] = {r.x, r.y, r.z};
    const int nmx[3] = {kp.hmax, kp.kmax, kp.lmax};
    int off = 0;
    float2 *T = kp.tabf + (size_t)b * kp.ntab * kp.S + s;
    for (int d = 0; d < 3; d++) {
        const double t = xyz[d] * kp.boxi[d];
        const unsigned u = (unsigned)(unsigned long long)__double2ll_rn((t - floor(t)) * 0x1p32);
        T[(size_t)off * kp.S] = make_float2(1.f, 0.f);
        for (int n = 1; n <= nmx[d]; n++) {
            const int ph = (int)(u * (unsigned)n);
            float sn, cs;
            sincospif((float)ph * 0x1p-31f, &sn, &cs);
            T[(size_t)(off + n) * kp.S] = make_float2(cs, sn);
        }
        off += nmx[d] + 1;
    }
}

// k-vector components in the arithmetic type of the phase sums: FP64 from kinfo, FP32 from
// the precomputed FP32 tables (no double-to-float conversion inside the mixed kernels)
template <typename R>
struct KV;
template <>
struct KV<double> {
    PIMD_D static void run_xy(const KP &kp, int r, double &x, double &y) {
        const double4_32a v = kp.kinfo[kp.runs[r].kbeg];
        x = v.x;
        y = v.y;
    }
    PIMD_D static double z(const KP &kp, int k) { return kp.kinfo[k].z; }
};
template <>
struct KV<float> {
    PIMD_D static void run_xy(const KP &kp, int r, float &x, float &y) {
        const float2 v = kp.runkf[r];
        x = v.x;
        y = v.y;
    }
    PIMD_D static float z(const KP &kp, int k) { return kp.kzf[k]; }
};

enum { OP_Q = 0, OP_MU = 1, OP_DIP = 2 };
constexpr int SP_NT = 256;  // threads (k-vectors) per structure-factor block
constexpr int SP_TS = 64;   // sites per shared-memory tile

template <typename R>
PIMD_D typename C2<R>::T tab_x(const KP &kp, int b, int n, int s) {
    return tab_base<R>(kp)[((size_t)b * kp.ntab + n) * kp.S + s];
}
template <typename R>
PIMD_D typename C2<R>::T tab_y(const KP &kp, int b, int n, int s) {
    const typename C2<R>::T v = tab_base<R>(kp)[((size_t)b * kp.ntab + kp.hmax + 1 + (n < 0 ? -n : n)) * kp.S + s];
    return n < 0 ? cconj(v) : v;
}
template <typename R>
PIMD_D typename C2<R>::T tab_z(const KP &kp, int b, int n, int s) {
    return tab_base<R>(kp)[((size_t)b * kp.ntab + kp.hmax + 1 + kp.kmax + 1 + n) * kp.S + s];
}

// Per-tile partial structure factors.
//   OP_Q : sum_s q_s e_s                        (ewald.f90:41-42)
//   OP_MU: sum_s (k.mu_s) e_s                   (ewald.f90:99-108)
//   OP_DIP: sum_s mu_{s,c} e_s, c = x, y, z     (ewald.f90:208-213)
template <int OP, typename R>
__global__ void __launch_bounds__(SP_NT) k_spass(KP kp, int s0, int nsites, int tsg, int ngroups, int skipconv) {
    using V = typename C2<R>::T;
    constexpr int NC = (OP == OP_DIP) ? 3 : 1;
    const int b = blockIdx.z;
    if (skipconv && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    const int grp = blockIdx.y;
    const KChunk ch = kp.chunks[blockIdx.x];
    const int nr = ch.r1 - ch.r0;
    const int LZ = 2 * kp.lmax + 1;
    extern __shared__ double smem[];
    V *ez = reinterpret_cast<V *>(smem);               // [TS][LZ]
    V *exy = ez + SP_TS * LZ;                          // [TS][nr]
    R *aa = reinterpret_cast<R *>(exy + SP_TS * nr);   // [TS][nr] (OP_MU)
    R *wt = aa + SP_TS * nr;                           // [TS][4]
    const int k = ch.k0 + threadIdx.x;
    const bool valid = k < ch.k1;
    int rk = 0, kz = 0;
    R kzv = R(0);
    if (valid) {
        const int2 ki = kp.kidx[k];
        rk = ki.x - ch.r0;
        kz = ki.y;
        kzv = KV<R>::z(kp, k);
    }
    V acc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = C2<R>::make(R(0), R(0));
    const int gbeg = s0 + grp * tsg, gend = min(s0 + nsites, gbeg + tsg);
    for (int sb = gbeg; sb < gend; sb += SP_TS) {
        const int nloc = min(SP_TS, gend - sb);
        __syncthreads();
        if (threadIdx.x < nloc) {
            const size_t gs = (size_t)b * kp.S + sb + threadIdx.x;
            if (OP == OP_Q) {
                wt[4 * threadIdx.x] = R(kp.pos[gs].w);
            } else {
                wt[4 * threadIdx.x + 0] = R(kp.dip[3 * gs + 0]);
                wt[4 * threadIdx.x + 1] = R(kp.dip[3 * gs + 1]);
                wt[4 * threadIdx.x + 2] = R(kp.dip[3 * gs + 2]);
            }
        }
        for (int idx = threadIdx.x; idx < nloc * (kp.lmax + 1); idx += SP_NT) {
            const int site = idx % nloc, n = idx / nloc;
            const V v = tab_z<R>(kp, b, n, sb + site);
            ez[site * LZ + kp.lmax + n] = v;
            ez[site * LZ + kp.lmax - n] = cconj(v);
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < nloc * nr; idx += SP_NT) {
            const int site = idx % nloc, r = idx / nloc;
            const KRun run = kp.runs[ch.r0 + r];
            const V ex = tab_x<R>(kp, b, run.kx, sb + site);
            const V ey = tab_y<R>(kp, b, run.ky, sb + site);
            // ewald.f90:30-31: coskxky = cx cy - sx sy, sinkxky = sx cy + cx sy
            exy[site * nr + r] = C2<R>::make(ex.x * ey.x - ex.y * ey.y, ex.y * ey.x + ex.x * ey.y);
            if (OP == OP_MU) {
                R kx, ky;
                KV<R>::run_xy(kp, ch.r0 + r, kx, ky);
                aa[site * nr + r] = kx * wt[4 * site] + ky * wt[4 * site + 1];
            }
        }
        __syncthreads();
        if (valid) {
            for (int site = 0; site < nloc; site++) {
                const V a = exy[site * nr + rk];
                const V z = ez[site * LZ + kp.lmax + kz];
                // ewald.f90:37-39: coskr = cxy cz - sxy sz, sinkr = sxy cz + cxy sz
                const V e = C2<R>::make(a.x * z.x - a.y * z.y, a.y * z.x + a.x * z.y);
                if (OP == OP_Q) {
                    const R q = wt[4 * site];
                    acc[0].x += q * e.x;
                    acc[0].y += q * e.y;
                } else if (OP == OP_MU) {
                    const R t = aa[site * nr + rk] + kzv * wt[4 * site + 2];
                    acc[0].x += t * e.x;
                    acc[0].y += t * e.y;
                } else {
#pragma unroll
                    for (int c = 0; c < NC; c++) {
                        acc[c].x += wt[4 * site + c] * e.x;
                        acc[c].y += wt[4 * site + c] * e.y;
                    }
                }
            }
        }
    }
    if (valid) {
        V *out = reinterpret_cast<V *>(kp.Spart) + (((size_t)b * ngroups + grp) * kp.nk + k) * NC;
#pragma unroll
        for (int c = 0; c < NC; c++) out[c] = acc[c];
    }
}

// Register-tiled FP32 structure factors of the mixed engine. With e^{ik.r} = exy(kx,ky) ez(kz)
// every structure factor is a set of M small complex GEMMs over the sites of a group,
//   G_m[run][kz] = sum_s A_m[s][run] ez[s][kz],   A_m = w_m exy(run)
// (OP_Q: w = q; OP_MU: w = kx mu_x + ky mu_y and mu_z, S = G_0 + k_z G_1; OP_DIP: w = mu_c).
// Runs are processed in tiles of SF_RT runs of similar kz extent (sorted by nkz on the host,
// kp.sfrun / kp.sftile), so a tile only spans the kz window its runs need. A block owns one
// tile of one bead and one site group; lane = run, warp = group of SF_TK kz slots, so per site
// a thread reads its A values with one conflict-free shared load and its ez slots with
// broadcast 128-bit loads, then issues SF_TK * M * 4 FFMAs in registers. Slots outside a run's
// own kz range are computed and dropped. Partials per site group go to Spart like k_spass's.
constexpr int SF_RT = 32;                // runs per tile (one per lane)
constexpr int SF_TK = 4;                 // kz slots per thread
constexpr int SF_TS = 32;                // sites per shared-memory tile
constexpr int SF_MAXT = 416;             // threads per block: kz window <= 52 slots

// acc += a * e (complex), as four FFMAs
PIMD_D void cmac(float2 &acc, float2 a, float2 e) {
    acc.x = fmaf(a.x, e.x, acc.x);
    acc.x = fmaf(-a.y, e.y, acc.x);
    acc.y = fmaf(a.y, e.x, acc.y);
    acc.y = fmaf(a.x, e.y, acc.y);
}

template <int OP>
__global__ void __launch_bounds__(SF_MAXT) k_sfac_f(KP kp, int s0, int nsites, int tsg, int ngroups, int skipconv) {
    constexpr int M = (OP == OP_Q) ? 1 : (OP == OP_MU) ? 2 : 3;
    constexpr int NC = (OP == OP_DIP) ? 3 : 1;
    const int b = blockIdx.z;
    if (skipconv && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    const int grp = blockIdx.y;
    const int4 tile = kp.sftile[blockIdx.x];  // first ez slot, kz groups, runs, offset into sfrun
    const int zb = tile.x, nkg = tile.y, nr = tile.z;
    const int KZP = nkg * SF_TK;
    const int L = kp.lmax;
    const int tid = threadIdx.x, lane = tid % SF_RT, kg = tid / SF_RT;
    extern __shared__ float4 smf[];
    float2 *A = reinterpret_cast<float2 *>(smf);  // [TS][RT][M]
    float2 *ez = A + SF_TS * SF_RT * M;            // [TS][KZP]: slots zb .. zb + KZP - 1
    float4 *wt = reinterpret_cast<float4 *>(ez + SF_TS * KZP);  // [TS]
    __shared__ int2 rxy[SF_RT];
    __shared__ float2 rkv[SF_RT];
    if (tid < SF_RT) {
        if (tid < nr) {
            const int r = kp.sfrun[tile.w + tid];
            const KRun run = kp.runs[r];
            rxy[tid] = make_int2(run.kx, run.ky);
            rkv[tid] = kp.runkf[r];
        } else {
            rxy[tid] = make_int2(0, 0);
            rkv[tid] = make_float2(0.f, 0.f);
        }
    }
    float2 acc[SF_TK][M];
#pragma unroll
    for (int j = 0; j < SF_TK; j++)
#pragma unroll
        for (int m = 0; m < M; m++) acc[j][m] = make_float2(0.f, 0.f);
    const int gbeg = s0 + grp * tsg, gend = min(s0 + nsites, gbeg + tsg);
    for (int sb = gbeg; sb < gend; sb += SF_TS) {
        const int nloc = min(SF_TS, gend - sb);
        __syncthreads();
        if (tid < SF_TS) {
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            if (tid < nloc) {
                const size_t gs = (size_t)b * kp.S + sb + tid;
                if (OP == OP_Q)
                    w.x = (float)kp.pos[gs].w;
                else
                    w = dipf_cur(kp)[gs];  // FP32 copy written with every dipole update
            }
            wt[tid] = w;
        }
        for (int idx = tid; idx < SF_TS * KZP; idx += blockDim.x) {
            const int site = idx / KZP, kz = zb + (idx - site * KZP) - L;
            float2 v = make_float2(0.f, 0.f);
            if (site < nloc && kz <= L) {
                v = tab_z<float>(kp, b, kz < 0 ? -kz : kz, sb + site);
                if (kz < 0) v = cconj(v);
            }
            ez[idx] = v;
        }
        __syncthreads();
        for (int idx = tid; idx < SF_TS * SF_RT; idx += blockDim.x) {
            // lane = run: the stores of a warp are contiguous (the table reads repeat few rows)
            const int r = idx % SF_RT, site = idx / SF_RT;
            float2 a[M];
#pragma unroll
            for (int m = 0; m < M; m++) a[m] = make_float2(0.f, 0.f);
            if (site < nloc && r < nr) {
                const int2 xy = rxy[r];
                const float2 ex = tab_x<float>(kp, b, xy.x, sb + site);
                const float2 ey = tab_y<float>(kp, b, xy.y, sb + site);
                // ewald.f90:30-31: coskxky = cx cy - sx sy, sinkxky = sx cy + cx sy
                const float2 exy = make_float2(ex.x * ey.x - ex.y * ey.y, ex.y * ey.x + ex.x * ey.y);
                const float4 w = wt[site];
                if (OP == OP_Q) {
                    a[0] = make_float2(w.x * exy.x, w.x * exy.y);
                } else if (OP == OP_MU) {
                    const float2 kv = rkv[r];
                    const float t = kv.x * w.x + kv.y * w.y;
                    a[0] = make_float2(t * exy.x, t * exy.y);
                    a[M - 1] = make_float2(w.z * exy.x, w.z * exy.y);
                } else {
                    a[0] = make_float2(w.x * exy.x, w.x * exy.y);
                    a[1] = make_float2(w.y * exy.x, w.y * exy.y);
                    a[M - 1] = make_float2(w.z * exy.x, w.z * exy.y);
                }
            }
            if (M == 2) {
                *reinterpret_cast<float4 *>(A + (site * SF_RT + r) * M) = make_float4(a[0].x, a[0].y, a[M - 1].x, a[M - 1].y);
            } else {
#pragma unroll
                for (int m = 0; m < M; m++) A[(site * SF_RT + r) * M + m] = a[m];
            }
        }
        __syncthreads();
        if (kg < nkg) {
            for (int site = 0; site < nloc; site++) {
                float2 a[M], e[SF_TK];
                const float2 *ap = A + (site * SF_RT + lane) * M;
                if (M == 2) {
                    const float4 v = *reinterpret_cast<const float4 *>(ap);
                    a[0] = make_float2(v.x, v.y);
                    a[M - 1] = make_float2(v.z, v.w);
                } else {
#pragma unroll
                    for (int m = 0; m < M; m++) a[m] = ap[m];
                }
                const float4 *ep = reinterpret_cast<const float4 *>(ez + site * KZP + kg * SF_TK);
#pragma unroll
                for (int j = 0; j < SF_TK / 2; j++) {
                    const float4 v = ep[j];
                    e[2 * j] = make_float2(v.x, v.y);
                    e[2 * j + 1] = make_float2(v.z, v.w);
                }
                // ewald.f90:37-39: coskr = cxy cz - sxy sz, sinkr = sxy cz + cxy sz
#pragma unroll
                for (int j = 0; j < SF_TK; j++)
#pragma unroll
                    for (int m = 0; m < M; m++) cmac(acc[j][m], a[m], e[j]);
            }
        }
    }
    if (kg >= nkg || lane >= nr) return;
    const KRun run = kp.runs[kp.sfrun[tile.w + lane]];
#pragma unroll
    for (int j = 0; j < SF_TK; j++) {
        const int kz = zb + kg * SF_TK + j - L;
        if (kz < run.kzlo || kz >= run.kzlo + run.nkz) continue;
        const int k = run.kbeg + kz - run.kzlo;
        float2 *out = reinterpret_cast<float2 *>(kp.Spart) + (((size_t)b * ngroups + grp) * kp.nk + k) * NC;
        if (OP == OP_MU) {
            const float kzv = kp.kzf[k];
            out[0] = make_float2(fmaf(kzv, acc[j][M - 1].x, acc[j][0].x), fmaf(kzv, acc[j][M - 1].y, acc[j][0].y));
        } else {
#pragma unroll
            for (int c = 0; c < NC; c++) out[c] = acc[j][c];
        }
    }
}

// Sum the tile partials in FP64 in a fixed order. OP_MU stores (rQm, iQm) = (-Im, Re) of
// sum (k.mu) e (ewald.f90:106-107).
template <int OP, typename R>
__global__ void __launch_bounds__(256) k_sreduce(KP kp, int ngroups, int skipconv) {
    using V = typename C2<R>::T;
    constexpr int NC = (OP == OP_DIP) ? 3 : 1;
    const int k = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (k >= kp.nk) return;
    if (skipconv && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    double2 s[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) s[c] = make_double2(0.0, 0.0);
    const V *part = reinterpret_cast<const V *>(kp.Spart);
    for (int g = 0; g < ngroups; g++) {
        const V *p = part + (((size_t)b * ngroups + g) * kp.nk + k) * NC;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            s[c].x += (double)p[c].x;
            s[c].y += (double)p[c].y;
        }
    }
    if (OP == OP_Q) kp.Sq[(size_t)b * kp.nk + k] = s[0];
    if (OP == OP_MU) kp.Sm[(size_t)b * kp.nk + k] = make_double2(-s[0].y, s[0].x);
    if (sizeof(R) == 4 && OP != OP_DIP) {
        // FP32 field weights 4 pi Ak / V conj(S) of the mixed engine's field passes
        const double w = kp.kinfo[k].w;
        const double2 a = (OP == OP_Q) ? s[0] : make_double2(-s[0].y, s[0].x);
        kp.Wf[((size_t)b * 2 + (OP == OP_Q ? 0 : 1)) * kp.nk + k] = make_float2((float)(w * a.x), (float)(-w * a.y));
    }
    if (OP == OP_DIP)
#pragma unroll
        for (int c = 0; c < 3; c++) kp.Sdip[((size_t)b * kp.nk + k) * 3 + c] = s[c];
}

// ---------------------------------------------------------------------------------------
// Site-parallel field passes.
//   FQ : charge field and potential from Sq     (ewald.f90:45-49)
//   FD : dipole field from Sm, then the SOR update and convergence sums of one iteration
//        (ewald.f90:114-117 and pot_ttm.f90:371-381)
//   QD : reciprocal forces on charges and dipoles and the dipole part of phi
//        (ewald.f90:184-193)
enum { F_Q = 0, F_D = 1, F_QD = 2 };
constexpr int KCH = 256;  // k-vectors staged per chunk (== SP_NT)

// The k-list is split over gridDim.z slices (whole chunks each); every block writes its
// slice's FP64 partial (E or G, phi) per site to Fpart[slice][bead][site], and
// k_field_finish adds the slices in a fixed order and applies the epilogue.
template <int MODE, int NT, typename R>
__global__ void __launch_bounds__(NT) k_field(KP kp, int s0, int s1) {
    using V = typename C2<R>::T;
    const int b = blockIdx.y, slice = blockIdx.z, nslice = gridDim.z;
    if (MODE == F_D && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    const int s = s0 + blockIdx.x * NT + threadIdx.x;
    const bool valid = s < s1;
    const int LZ = 2 * kp.lmax + 1;
    extern __shared__ double smem[];
    V *ez = reinterpret_cast<V *>(smem);  // [LZ][NT]
    V *W1 = ez + LZ * NT;                 // [KCH]
    V *W2 = W1 + KCH;                     // [KCH] (QD)
    R *kzs = reinterpret_cast<R *>(W2 + KCH);  // [KCH]
    const size_t gs = (size_t)b * kp.S + (valid ? s : s0);
    for (int n = 0; n <= kp.lmax; n++) {
        const V v = valid ? tab_z<R>(kp, b, n, s) : C2<R>::make(R(0), R(0));
        ez[(kp.lmax + n) * NT + threadIdx.x] = v;
        ez[(kp.lmax - n) * NT + threadIdx.x] = cconj(v);
    }
    double q = 0.0, mu[3] = {0, 0, 0};
    bool isdip = false;
    if (valid) {
        q = kp.pos[gs].w;
        isdip = s >= kp.fd && s < kp.ld;
        if (MODE != F_Q && isdip) {
            mu[0] = kp.dip[3 * gs];
            mu[1] = kp.dip[3 * gs + 1];
            mu[2] = kp.dip[3 * gs + 2];
        }
    }
    const R qr = R(q), mur[3] = {R(mu[0]), R(mu[1]), R(mu[2])};
    double E[3] = {0, 0, 0}, phi = 0.0, G[3] = {0, 0, 0};
    const double2 *S1 = (MODE == F_Q) ? kp.Sq : kp.Sm;
    const int c0 = (int)((long)slice * kp.nchunk / nslice), c1 = (int)((long)(slice + 1) * kp.nchunk / nslice);
    for (int chn = c0; chn < c1; chn++) {
        const KChunk ch = kp.chunks[chn];
        __syncthreads();
        for (int i = threadIdx.x; i < ch.k1 - ch.k0; i += NT) {
            const int k = ch.k0 + i;
            if constexpr (sizeof(R) == 4) {
                const float2 wq = kp.Wf[((size_t)b * 2) * kp.nk + k], wm = kp.Wf[((size_t)b * 2 + 1) * kp.nk + k];
                W1[i] = (MODE == F_Q) ? wq : wm;
                if (MODE == F_QD) W2[i] = make_float2(wq.x + wm.x, wq.y + wm.y);
                kzs[i] = kp.kzf[k];
            } else {
                const double4_32a ki = kp.kinfo[k];
                const double2 a = S1[(size_t)b * kp.nk + k];
                W1[i] = C2<R>::make(R(ki.w * a.x), R(-ki.w * a.y));  // 4 pi Ak / V conj(S)
                if (MODE == F_QD) {
                    const double2 c = kp.Sq[(size_t)b * kp.nk + k];
                    W2[i] = C2<R>::make(R(ki.w * (c.x + a.x)), R(-ki.w * (c.y + a.y)));
                }
                kzs[i] = R(ki.z);
            }
        }
        __syncthreads();
        if (!valid) continue;
        // per-chunk partial sums in R, added to the FP64 totals once per chunk
        R cE[3] = {R(0), R(0), R(0)}, cphi = R(0), cG[3] = {R(0), R(0), R(0)};
        for (int r = ch.r0; r < ch.r1; r++) {
            const KRun run = kp.runs[r];
            R kvx, kvy;
            KV<R>::run_xy(kp, r, kvx, kvy);
            const V ex = tab_x<R>(kp, b, run.kx, s);
            const V ey = tab_y<R>(kp, b, run.ky, s);
            const V exy = C2<R>::make(ex.x * ey.x - ex.y * ey.y, ex.y * ey.x + ex.x * ey.y);
            V U0 = C2<R>::make(R(0), R(0)), U1 = U0, V0 = U0, V1 = U0, V2 = U0;
            const int i0 = run.kbeg - ch.k0;
            for (int j = 0; j < run.nkz; j++) {
                const V z = ez[(kp.lmax + run.kzlo + j) * NT + threadIdx.x];
                const R kz = kzs[i0 + j];
                const V t = cmul(z, W1[i0 + j]);
                U0.x += t.x;
                U0.y += t.y;
                U1.x += kz * t.x;
                U1.y += kz * t.y;
                if (MODE == F_QD && isdip) {
                    const V u = cmul(z, W2[i0 + j]);
                    V0.x += u.x;
                    V0.y += u.y;
                    V1.x += kz * u.x;
                    V1.y += kz * u.y;
                    V2.x += kz * kz * u.x;
                    V2.y += kz * kz * u.y;
                }
            }
            const V z0 = cmul(exy, U0), z1 = cmul(exy, U1);
            if (MODE == F_QD) {
                cphi += z0.x;
                cG[0] -= qr * z0.y * kvx;
                cG[1] -= qr * z0.y * kvy;
                cG[2] -= qr * z1.y;
                if (isdip) {
                    const R R0 = exy.x * V0.x - exy.y * V0.y;
                    const R R1 = exy.x * V1.x - exy.y * V1.y;
                    const R R2 = exy.x * V2.x - exy.y * V2.y;
                    const R a = kvx * mur[0] + kvy * mur[1];
                    cG[0] -= kvx * (a * R0 + mur[2] * R1);
                    cG[1] -= kvy * (a * R0 + mur[2] * R1);
                    cG[2] -= a * R1 + mur[2] * R2;
                }
            } else {
                cphi += z0.x;
                cE[0] += z0.y * kvx;
                cE[1] += z0.y * kvy;
                cE[2] += z1.y;
            }
        }
        phi += (double)cphi;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            E[c] += (double)cE[c];
            G[c] += (double)cG[c];
        }
    }
    if (valid) {
        double4_32a *o = kp.Fpart + ((size_t)slice * kp.P + b) * (s1 - s0) + (s - s0);
        if (MODE == F_QD)
            *o = make_double4_32a(G[0], G[1], G[2], phi);
        else
            *o = make_double4_32a(E[0], E[1], E[2], phi);
    }
}

// FP32 field pass of the mixed engine with the site's e^{i kz z} row held in registers, centred
// at slot LM = LZM / 2 (slot LM + kz, |kz| <= lmax <= LM). Per chunk the weights are staged
// densely as [run][slot] (zero outside the run's kz range). A run with kz in [-m, m] (every run
// but kx = ky = 0) dispatches on m to a fully unrolled loop over exactly its 2m + 1 slots, so
// each useful (site, k) costs one broadcast shared load and eight FP32 operations on register
// operands: U0 = sum ez W, U1 = sum kz ez W (and V0..V2 with W2 = W_q + W_mu for QD). Same
// slicing and FP64 per-chunk accumulation as k_field.
constexpr int FF_NT = 128;
constexpr int FF_RUNS = 64;  // runs per chunk (KChunk limit)

struct FAcc {
    float2 U0, U1, V0, V1, V2;
};

template <int MODE>
PIMD_D void field_slot(const float2 &ez, float2 W, float2 W2, float kz, FAcc &a) {
    const float2 t = make_float2(ez.x * W.x - ez.y * W.y, ez.y * W.x + ez.x * W.y);
    a.U0.x += t.x;
    a.U0.y += t.y;
    a.U1.x = fmaf(kz, t.x, a.U1.x);
    a.U1.y = fmaf(kz, t.y, a.U1.y);
    if (MODE == F_QD) {
        const float2 u = make_float2(ez.x * W2.x - ez.y * W2.y, ez.y * W2.x + ez.x * W2.y);
        a.V0.x += u.x;
        a.V0.y += u.y;
        a.V1.x = fmaf(kz, u.x, a.V1.x);
        a.V1.y = fmaf(kz, u.y, a.V1.y);
        a.V2.x = fmaf(kz * kz, u.x, a.V2.x);
        a.V2.y = fmaf(kz * kz, u.y, a.V2.y);
    }
}

template <int MODE, int LZM, int MM>
PIMD_D void field_sym(const float2 (&ez)[LZM], const float2 *w1, const float2 *w2, FAcc &a) {
    constexpr int LM = LZM / 2;
    if constexpr (MM <= LM) {
#pragma unroll
        for (int j = LM - MM; j <= LM + MM; j++)
            field_slot<MODE>(ez[j], w1[j], MODE == F_QD ? w2[j] : make_float2(0.f, 0.f), (float)(j - LM), a);
    }
}

template <int MODE, int LZM>
__global__ void __launch_bounds__(FF_NT) k_field_f(KP kp, int s0, int s1) {
    constexpr int LM = LZM / 2;
    const int b = blockIdx.y, slice = blockIdx.z, nslice = gridDim.z;
    if (MODE == F_D && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    const int s = s0 + blockIdx.x * FF_NT + threadIdx.x;
    const bool valid = s < s1;
    const int L = kp.lmax;
    extern __shared__ float4 smf[];
    float2 *Wd = reinterpret_cast<float2 *>(smf);  // [1 or 2 (QD)][FF_RUNS][LZM]
    __shared__ int4 rinfo[FF_RUNS];                // kx, ky, first slot, last slot + 1
    __shared__ float2 rkv[FF_RUNS];
    float2 ez[LZM];
#pragma unroll
    for (int j = 0; j < LZM; j++) {
        const int kz = j - LM;
        float2 v = make_float2(0.f, 0.f);
        if (valid && kz >= -L && kz <= L) {
            v = tab_z<float>(kp, b, kz < 0 ? -kz : kz, s);
            if (kz < 0) v = cconj(v);
        }
        ez[j] = v;
    }
    const size_t gs = (size_t)b * kp.S + (valid ? s : s0);
    float qr = 0.f, mur[3] = {0.f, 0.f, 0.f};
    bool isdip = false;
    if (valid) {
        qr = (float)kp.pos[gs].w;
        isdip = s >= kp.fd && s < kp.ld;
        if (MODE == F_QD && isdip) {
            mur[0] = (float)kp.dip[3 * gs];
            mur[1] = (float)kp.dip[3 * gs + 1];
            mur[2] = (float)kp.dip[3 * gs + 2];
        }
    }
    // the k-vector's z component is 2 pi kz / Lz; the loops accumulate with the integer kz
    const float kzs = (float)(TWOPI * kp.boxi[2]);
    double E[3] = {0, 0, 0}, phi = 0.0, G[3] = {0, 0, 0};
    const int c0 = (int)((long)slice * kp.nchunk / nslice), c1 = (int)((long)(slice + 1) * kp.nchunk / nslice);
    for (int chn = c0; chn < c1; chn++) {
        const KChunk ch = kp.chunks[chn];
        const int nr = ch.r1 - ch.r0;
        __syncthreads();
        if (threadIdx.x < nr) {
            const KRun run = kp.runs[ch.r0 + threadIdx.x];
            rinfo[threadIdx.x] = make_int4(run.kx, run.ky, run.kzlo + LM, run.kzlo + LM + run.nkz);
            rkv[threadIdx.x] = kp.runkf[ch.r0 + threadIdx.x];
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < nr * LZM; idx += FF_NT) {
            const int rl = idx / LZM, j = idx - rl * LZM;
            const int4 ri = rinfo[rl];
            float2 w1 = make_float2(0.f, 0.f), w2 = w1;
            if (j >= ri.z && j < ri.w) {
                const int k = kp.runs[ch.r0 + rl].kbeg + (j - ri.z);
                const float2 wq = kp.Wf[((size_t)b * 2) * kp.nk + k], wm = kp.Wf[((size_t)b * 2 + 1) * kp.nk + k];
                w1 = (MODE == F_Q) ? wq : wm;
                if (MODE == F_QD) w2 = make_float2(wq.x + wm.x, wq.y + wm.y);
            }
            Wd[idx] = w1;
            if (MODE == F_QD) Wd[FF_RUNS * LZM + idx] = w2;
        }
        __syncthreads();
        if (!valid) continue;
        float cE[3] = {0.f, 0.f, 0.f}, cphi = 0.f, cG[3] = {0.f, 0.f, 0.f};
        for (int rl = 0; rl < nr; rl++) {
            const int4 ri = rinfo[rl];
            const float2 kv = rkv[rl];
            const float2 ex = tab_x<float>(kp, b, ri.x, s);
            const float2 ey = tab_y<float>(kp, b, ri.y, s);
            const float2 exy = make_float2(ex.x * ey.x - ex.y * ey.y, ex.y * ey.x + ex.x * ey.y);
            FAcc a;
            a.U0 = a.U1 = a.V0 = a.V1 = a.V2 = make_float2(0.f, 0.f);
            const float2 *w1 = Wd + rl * LZM;
            const float2 *w2 = Wd + FF_RUNS * LZM + rl * LZM;
            const int m = LM - ri.z;
            if (ri.z + ri.w == 2 * LM + 1) {  // kz in [-m, m]
                switch (m) {
#define PIMD_FF_CASE(MM) \
    case MM: field_sym<MODE, LZM, MM>(ez, w1, w2, a); break;
                    PIMD_FF_CASE(0) PIMD_FF_CASE(1) PIMD_FF_CASE(2) PIMD_FF_CASE(3) PIMD_FF_CASE(4)
                    PIMD_FF_CASE(5) PIMD_FF_CASE(6) PIMD_FF_CASE(7) PIMD_FF_CASE(8) PIMD_FF_CASE(9)
                    PIMD_FF_CASE(10) PIMD_FF_CASE(11) PIMD_FF_CASE(12) PIMD_FF_CASE(13) PIMD_FF_CASE(14)
                    PIMD_FF_CASE(15) PIMD_FF_CASE(16) PIMD_FF_CASE(17) PIMD_FF_CASE(18) PIMD_FF_CASE(19)
                    PIMD_FF_CASE(20) PIMD_FF_CASE(21) PIMD_FF_CASE(22) PIMD_FF_CASE(23) PIMD_FF_CASE(24)
#undef PIMD_FF_CASE
                    default: break;
                }
            } else {  // kx = ky = 0: kz >= 1 only
#pragma unroll
                for (int j = LM + 1; j < LZM; j++) {
                    if (j >= ri.w) continue;
                    field_slot<MODE>(ez[j], w1[j], MODE == F_QD ? w2[j] : make_float2(0.f, 0.f), (float)(j - LM), a);
                }
            }
            const float2 z0 = cmul(exy, a.U0), z1 = cmul(exy, a.U1);
            if (MODE == F_QD) {
                cphi += z0.x;
                cG[0] -= qr * z0.y * kv.x;
                cG[1] -= qr * z0.y * kv.y;
                cG[2] -= qr * z1.y * kzs;
                if (isdip) {
                    const float R0 = exy.x * a.V0.x - exy.y * a.V0.y;
                    const float R1 = (exy.x * a.V1.x - exy.y * a.V1.y) * kzs;
                    const float R2 = (exy.x * a.V2.x - exy.y * a.V2.y) * (kzs * kzs);
                    const float aa = kv.x * mur[0] + kv.y * mur[1];
                    cG[0] -= kv.x * (aa * R0 + mur[2] * R1);
                    cG[1] -= kv.y * (aa * R0 + mur[2] * R1);
                    cG[2] -= aa * R1 + mur[2] * R2;
                }
            } else {
                cphi += z0.x;
                cE[0] += z0.y * kv.x;
                cE[1] += z0.y * kv.y;
                cE[2] += z1.y * kzs;
            }
        }
        phi += (double)cphi;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            E[c] += (double)cE[c];
            G[c] += (double)cG[c];
        }
    }
    if (valid) {
        double4_32a *o = kp.Fpart + ((size_t)slice * kp.P + b) * (s1 - s0) + (s - s0);
        if (MODE == F_QD)
            *o = make_double4_32a(G[0], G[1], G[2], phi);
        else
            *o = make_double4_32a(E[0], E[1], E[2], phi);
    }
}

// Sum the slices of k_field in order and apply the pass's epilogue, one thread per site.
// F_D also runs the iteration's convergence test (dipole_check.cuh) in whichever block finishes
// last (a device counter, reset by that block), so an iteration needs no separate launch.
template <int MODE, int NT>
__global__ void __launch_bounds__(NT) k_field_finish(KP kp, int s0, int s1, int nslice) {
    const int b = blockIdx.y;
    const int iter = kp.dstep[1] + 1;  // dipole iteration of this update (F_D)
    const bool done = MODE == F_D && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0;
    if (done) {  // converged bead: no update, but the block still counts towards the test
        const double zero[2] = {0.0, 0.0};
        dd_block_end<NT>(kp, b, zero, false);
        return;
    }
    const int s = s0 + blockIdx.x * NT + threadIdx.x;
    const bool valid = s < s1;
    const size_t gs = (size_t)b * kp.S + (valid ? s : s0);
    double E[3] = {0, 0, 0}, phi = 0.0;
    if (valid) {
        for (int z = 0; z < nslice; z++) {
            const double4_32a p = kp.Fpart[((size_t)z * kp.P + b) * (s1 - s0) + (s - s0)];
            E[0] += p.x;
            E[1] += p.y;
            E[2] += p.z;
            phi += p.w;
        }
    }
    if (MODE == F_Q) {
        if (valid) {
            double4_32a f = kp.F[gs];
            f.x += E[0];
            f.y += E[1];
            f.z += E[2];
            if (s >= kp.fq) f.w += phi;
            kp.F[gs] = f;
        }
    } else if (MODE == F_QD) {
        if (valid) {
            if (s >= kp.fq) kp.F[gs].w += phi;
            kp.dR[3 * gs + 0] += E[0];
            kp.dR[3 * gs + 1] += E[1];
            kp.dR[3 * gs + 2] += E[2];
        }
    } else {
        // pot_ttm.f90:371-381 Efd = Efd_real + Efd_rec + Efq + factor mu; SOR update (FP64)
        double av[2] = {0.0, 0.0};
        if (valid) dd_sor_site(kp, b, s, E, iter, av);
        dd_block_end<NT>(kp, b, av, true);
    }
}

// Reciprocal-space virial, one thread per (k, bead), FP64. DIP: ewald.f90:194-224 (charges
// and induced dipoles, also the centroid-virial trace); !DIP: ewald.f90:276-289
// (ewald_pw_std_qq, charges only).
template <bool DIP>
__global__ void __launch_bounds__(128) k_qd_virial(KP kp) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    double av[14];
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.0;
    if (k < kp.nk) {
        const double4_32a ki = kp.kinfo[k];
        const double kv[3] = {ki.x, ki.y, ki.z};
        const double Akk = kp.kAk[k];
        const double2 sq = kp.Sq[(size_t)b * kp.nk + k];
        const double2 sm = DIP ? kp.Sm[(size_t)b * kp.nk + k] : make_double2(0.0, 0.0);
        const double rQqm = sq.x + sm.x, iQqm = sq.y + sm.y;
        const double ksq = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
        const double coeff2 = 2.0 / ksq + 0.5 / (kp.ew.aewald * kp.ew.aewald);
        const double Ureck = Akk * (rQqm * rQqm + iQqm * iQqm);
        double rdip[3] = {0, 0, 0}, idip[3] = {0, 0, 0};
        if (DIP) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double2 d = kp.Sdip[((size_t)b * kp.nk + k) * 3 + c];
                rdip[c] = -d.y;
                idip[c] = d.x;
            }
        }
        const double sc = -0.5 * FOURPI / kp.volume;
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int bb = 0; bb < 3; bb++) {
                const double v = ((a == bb) ? Ureck : 0.0) - Ureck * coeff2 * kv[a] * kv[bb];
                const double v1 = 2.0 * Akk * kv[a] * (rQqm * rdip[bb] + iQqm * idip[bb]);
                av[ACC_VIRT + a + 3 * bb] = sc * (v + v1);
            }
        if (DIP) av[ACC_VIRIALC] = av[ACC_VIRT + 0] + av[ACC_VIRT + 4] + av[ACC_VIRT + 8];
    }
    block_reduce_add<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// The same in FP32 per k-vector (the mixed engine): structure factors rounded from FP64 once,
// per-k constants precomputed, warp sums in FP32 and block sums in FP64 (block_reduce_add_f).
template <bool DIP>
__global__ void __launch_bounds__(128) k_qd_virial_m(KP kp, float sc) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    float av[14];
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.f;
    if (k < kp.nk) {
        const float4 q = kp.kvirf[k];
        const float kv[3] = {q.x, q.y, q.z};
        const float coeff2 = kp.kc2f[k];
        const double2 sq = kp.Sq[(size_t)b * kp.nk + k];
        const double2 sm = DIP ? kp.Sm[(size_t)b * kp.nk + k] : make_double2(0.0, 0.0);
        const float rQqm = (float)(sq.x + sm.x), iQqm = (float)(sq.y + sm.y);
        const float Ureck = q.w * (rQqm * rQqm + iQqm * iQqm);
        float rdip[3] = {0.f, 0.f, 0.f}, idip[3] = {0.f, 0.f, 0.f};
        if (DIP) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double2 d = kp.Sdip[((size_t)b * kp.nk + k) * 3 + c];
                rdip[c] = -(float)d.y;
                idip[c] = (float)d.x;
            }
        }
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int bb = 0; bb < 3; bb++) {
                const float v = ((a == bb) ? Ureck : 0.f) - Ureck * coeff2 * kv[a] * kv[bb];
                const float v1 = 2.f * q.w * kv[a] * (rQqm * rdip[bb] + iQqm * idip[bb]);
                av[ACC_VIRT + a + 3 * bb] = sc * (v + v1);
            }
        if (DIP) av[ACC_VIRIALC] = av[ACC_VIRT + 0] + av[ACC_VIRT + 4] + av[ACC_VIRT + 8];
    }
    block_reduce_add_f<14, 128>(av, kp.acc + (size_t)b * NACC);
}

static void launch_qd_virial(Engine &E, bool dip) {
    dim3 g((E.kp.nk + 127) / 128, E.kp.P);
    if (E.precision == PIMD_PREC_MIXED && E.kp.kvirf) {
        const float sc = (float)(-0.5 * FOURPI / E.kp.volume);
        if (dip)
            k_qd_virial_m<true><<<g, 128, 0, E.stream>>>(E.kp, sc);
        else
            k_qd_virial_m<false><<<g, 128, 0, E.stream>>>(E.kp, sc);
    } else if (dip) {
        k_qd_virial<true><<<g, 128, 0, E.stream>>>(E.kp);
    } else {
        k_qd_virial<false><<<g, 128, 0, E.stream>>>(E.kp);
    }
    ++E.nlaunch;
}

// ---------------------------------------------------------------------------------------
static int spass_groups(const Engine &E, int nsites) {
    const int ntile = (nsites + SP_TS - 1) / SP_TS;
    const long per = (long)E.nchunk * E.kp.P;
    int g = (int)((152L * 8 + per - 1) / per);
    if (g < 1) g = 1;
    if (g > ntile) g = ntile;
    if (g > E.sp_cap) g = E.sp_cap;
    return g;
}

template <int OP, typename R>
static void run_spass_t(Engine &E, int s0, int nsites, int skipconv) {
    const int ng = spass_groups(E, nsites);
    const int ntile = (nsites + SP_TS - 1) / SP_TS;
    const int tsg = ((ntile + ng - 1) / ng) * SP_TS;
    const int ngr = (nsites + tsg - 1) / tsg;
    const int LZ = 2 * E.kp.lmax + 1;
    const size_t smem = ((size_t)SP_TS * LZ * 2 + (size_t)SP_TS * E.max_runs_chunk * 3 + (size_t)SP_TS * 4) * sizeof(R);
    dim3 g(E.nchunk, ngr, E.kp.P);
    k_spass<OP, R><<<g, SP_NT, smem, E.stream>>>(E.kp, s0, nsites, tsg, ngr, skipconv);
    ++E.nlaunch;
    dim3 g2((E.kp.nk + 255) / 256, E.kp.P);
    k_sreduce<OP, R><<<g2, 256, 0, E.stream>>>(E.kp, ngr, skipconv);
    ++E.nlaunch;
}

// the mixed engine's register-tiled structure factor; site groups of whole 32-site tiles sized
// for about 8 blocks per SM
template <int OP>
static void run_sfac_f(Engine &E, int s0, int nsites, int skipconv) {
    const KP &kp = E.kp;
    constexpr int M = (OP == OP_Q) ? 1 : (OP == OP_MU) ? 2 : 3;
    const int ntile = (nsites + SF_TS - 1) / SF_TS;
    const long per = (long)E.sf_ntiles * kp.P;
    const int KZP = E.sf_nkg_max * SF_TK;
    const size_t smem = sizeof(float2) * ((size_t)SF_TS * SF_RT * M + (size_t)SF_TS * KZP) + sizeof(float4) * SF_TS;
    const int gmax = std::max(1, std::min(ntile, E.sp_cap));
    int ng;
    if (E.sf_groups > 0)
        ng = E.sf_groups;
    else if (E.wave_shapes)
        ng = wave_split(E, k_sfac_f<OP>, SF_RT * E.sf_nkg_max, smem, per, gmax);
    else
        ng = (int)((152L * 8 + per - 1) / per);
    ng = std::max(1, std::min(ng, gmax));
    const int tsg = ((ntile + ng - 1) / ng) * SF_TS;
    const int ngr = (nsites + tsg - 1) / tsg;
    dim3 g(E.sf_ntiles, ngr, kp.P);
    k_sfac_f<OP><<<g, SF_RT * E.sf_nkg_max, smem, E.stream>>>(E.kp, s0, nsites, tsg, ngr, skipconv);
    ++E.nlaunch;
    dim3 g2((kp.nk + 255) / 256, kp.P);
    k_sreduce<OP, float><<<g2, 256, 0, E.stream>>>(E.kp, ngr, skipconv);
    ++E.nlaunch;
}

template <int OP>
static void run_spass(Engine &E, int s0, int nsites, int skipconv) {
    // tensor-core structure factors (ewald_tc.cu), which also write Sq/Sm/Sdip and the weights
    if (E.precision == PIMD_PREC_MIXED && launch_sfac_tc(E, OP, s0, nsites, skipconv)) return;
    if (E.precision == PIMD_PREC_MIXED) {
        if (E.sf_tiled && E.sf_nkg_max * SF_RT <= SF_MAXT)
            run_sfac_f<OP>(E, s0, nsites, skipconv);
        else
            run_spass_t<OP, float>(E, s0, nsites, skipconv);
    } else {
        run_spass_t<OP, double>(E, s0, nsites, skipconv);
    }
}

// Launch shapes by wave quantisation. A grid of B blocks with R resident per SM runs in
// ceil(B / (SMs R)) waves; when the split count c divides the work (each block does ~1/c of it),
// the time goes as waves(c) / c. Pick the c in [1, cmax] that minimises it (ties: smallest c,
// fewest partials to add afterwards). R comes from the occupancy calculator for the kernel.
static int sm_count(const Engine &E) {
    static int cached[64] = {0};
    const int d = E.device & 63;
    if (!cached[d]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, E.device);
        cached[d] = n > 0 ? n : 152;
    }
    return cached[d];
}

template <typename K>
static int wave_split(const Engine &E, K kernel, int threads, size_t smem, long base_blocks, int cmax) {
    int R = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&R, kernel, threads, smem);
    const long slots = (long)sm_count(E) * std::max(R, 1);
    int best = 1;
    double best_t = 1e300;
    for (int c = 1; c <= std::max(1, cmax); c++) {
        const long waves = (base_blocks * c + slots - 1) / slots;
        const double t = (double)waves / c;
        if (t < best_t - 1e-12) {
            best_t = t;
            best = c;
        }
    }
    return best;
}

template <int MODE, int NT, typename R>
static void launch_field_nt(Engine &E, int s0, int s1) {
    const int LZ = 2 * E.kp.lmax + 1;
    const size_t smem = ((size_t)LZ * NT * 2 + (size_t)KCH * 5) * sizeof(R);
    // k-slices: enough blocks for ~8 (FP32) / ~4 (FP64) resident blocks per SM
    const int sblocks = (s1 - s0 + NT - 1) / NT;
    const long want = (sizeof(R) == 4 ? 8L : 4L) * 152;
    int ns = (int)((want + (long)sblocks * E.kp.P - 1) / ((long)sblocks * E.kp.P));
    ns = std::max(1, std::min(ns, std::min(E.nchunk, E.max_slices)));
    dim3 g(sblocks, E.kp.P, ns);
    k_field<MODE, NT, R><<<g, NT, smem, E.stream>>>(E.kp, s0, s1);
    dim3 g2((s1 - s0 + 127) / 128, E.kp.P);
    k_field_finish<MODE, 128><<<g2, 128, 0, E.stream>>>(E.kp, s0, s1, ns);
    E.nlaunch += 2;
}

template <int MODE, int LZM>
static void launch_field_f(Engine &E, int s0, int s1) {
    const size_t smem = sizeof(float2) * ((MODE == F_QD) ? 2 : 1) * FF_RUNS * LZM;
    const int sblocks = (s1 - s0 + FF_NT - 1) / FF_NT;
    const int cmax = std::min(E.nchunk, E.max_slices);
    const int ns = E.wave_shapes ? wave_split(E, k_field_f<MODE, LZM>, FF_NT, smem, (long)sblocks * E.kp.P, cmax)
                                 : std::max(1, std::min((int)((8L * 152 + (long)sblocks * E.kp.P - 1) /
                                                              ((long)sblocks * E.kp.P)), cmax));
    dim3 g(sblocks, E.kp.P, ns);
    k_field_f<MODE, LZM><<<g, FF_NT, smem, E.stream>>>(E.kp, s0, s1);
    dim3 g2((s1 - s0 + 127) / 128, E.kp.P);
    k_field_finish<MODE, 128><<<g2, 128, 0, E.stream>>>(E.kp, s0, s1, ns);
    E.nlaunch += 2;
}

template <int MODE>
static void run_field(Engine &E, int s0, int s1) {
    const int LZ = 2 * E.kp.lmax + 1;
    // tensor-core field passes (ewald_tc.cu): dipole field with the SOR update and convergence
    // test, and the charge field and potential
    if (MODE != F_QD && E.precision == PIMD_PREC_MIXED && launch_field_tc(E, MODE, s0, s1)) return;
    if (MODE == F_D && E.field_needs_join) cudaStreamWaitEvent(E.stream, E.loop_join, 0);
    if (MODE == F_QD && E.precision == PIMD_PREC_MIXED && launch_field_qd_tc(E, s0, s1)) return;
    if (E.precision == PIMD_PREC_MIXED && E.ff_regs && LZ <= 49) {
        if (LZ <= 17)
            launch_field_f<MODE, 17>(E, s0, s1);
        else if (LZ <= 25)
            launch_field_f<MODE, 25>(E, s0, s1);
        else if (LZ <= 33)
            launch_field_f<MODE, 33>(E, s0, s1);
        else
            launch_field_f<MODE, 49>(E, s0, s1);
        return;
    }
    if (E.precision == PIMD_PREC_MIXED) {
        if ((size_t)LZ * 128 * 8 <= 64 * 1024)
            launch_field_nt<MODE, 128, float>(E, s0, s1);
        else
            launch_field_nt<MODE, 64, float>(E, s0, s1);
    } else {
        if ((size_t)LZ * 128 * 16 <= 64 * 1024)
            launch_field_nt<MODE, 128, double>(E, s0, s1);
        else
            launch_field_nt<MODE, 64, double>(E, s0, s1);
    }
}

// dynamic shared-memory limits of the Ewald kernels, set once per context on its device
template <typename R>
static void ewald_attrs() {
    const int lim = 200 * 1024;
    cudaFuncSetAttribute(k_spass<OP_Q, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_spass<OP_MU, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_spass<OP_DIP, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_field<F_Q, 128, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_field<F_D, 128, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_field<F_QD, 128, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_field<F_Q, 64, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_field<F_D, 64, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_field<F_QD, 64, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
}
// Tiles of the register-tiled structure factor: runs sorted by kz extent (longest first), 32 per
// tile; each tile records the first ez slot of its kz window and the number of kz groups.
// Returns 0, or 1 if the device tables could not be allocated.
static int sfac_tiles(Engine &E) {
    KP &kp = E.kp;
    std::vector<int> order(kp.nrun);
    for (int r = 0; r < kp.nrun; r++) order[r] = r;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return E.h_runs[a].nkz > E.h_runs[b].nkz; });
    std::vector<int4> tiles;
    E.sf_nkg_max = 0;
    for (int t0 = 0; t0 < kp.nrun; t0 += SF_RT) {
        const int nr = std::min(SF_RT, kp.nrun - t0);
        int lo = 1 << 30, hi = -(1 << 30);
        for (int i = 0; i < nr; i++) {
            const KRun &r = E.h_runs[order[t0 + i]];
            lo = std::min(lo, r.kzlo);
            hi = std::max(hi, r.kzlo + r.nkz - 1);
        }
        const int nkg = (hi - lo + 1 + SF_TK - 1) / SF_TK;
        E.sf_nkg_max = std::max(E.sf_nkg_max, nkg);
        tiles.push_back(make_int4(lo + kp.lmax, nkg, nr, t0));
    }
    E.sf_ntiles = (int)tiles.size();
    int *d_order;
    int4 *d_tiles;
    if (cudaMalloc((void **)&d_order, sizeof(int) * kp.nrun) != cudaSuccess ||
        cudaMalloc((void **)&d_tiles, sizeof(int4) * tiles.size()) != cudaSuccess)
        return 1;
    E.allocs.push_back(d_order);
    E.allocs.push_back(d_tiles);
    cudaMemcpy(d_order, order.data(), sizeof(int) * kp.nrun, cudaMemcpyHostToDevice);
    cudaMemcpy(d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice);
    kp.sfrun = d_order;
    kp.sftile = d_tiles;
    return 0;
}

void ewald_init(Engine &E) {
    if (sfac_tiles(E) != 0) E.sf_tiled = false;  // allocation failed: untiled kernel
    tc_init(E);
    ewald_attrs<double>();
    ewald_attrs<float>();
    // k_field_f stages [1 or 2][64 runs][LZM] complex weights: 50 KB for LZM = 49 in QD mode
#define PIMD_FF_ATTR(MODE, LZM) cudaFuncSetAttribute(k_field_f<MODE, LZM>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    PIMD_FF_ATTR(F_Q, 17) PIMD_FF_ATTR(F_D, 17) PIMD_FF_ATTR(F_QD, 17)
    PIMD_FF_ATTR(F_Q, 25) PIMD_FF_ATTR(F_D, 25) PIMD_FF_ATTR(F_QD, 25)
    PIMD_FF_ATTR(F_Q, 33) PIMD_FF_ATTR(F_D, 33) PIMD_FF_ATTR(F_QD, 33)
    PIMD_FF_ATTR(F_Q, 49) PIMD_FF_ATTR(F_D, 49) PIMD_FF_ATTR(F_QD, 49)
#undef PIMD_FF_ATTR
    cudaFuncSetAttribute(k_sfac_f<OP_Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_sfac_f<OP_MU>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_sfac_f<OP_DIP>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
}

void launch_ewald_tables(Engine &E) {
    dim3 g((E.kp.S + 127) / 128, E.kp.P);
    if (E.precision == PIMD_PREC_MIXED)
        k_ewald_tables_m<<<g, 128, 0, E.stream>>>(E.kp);
    else
        k_ewald_tables<double><<<g, 128, 0, E.stream>>>(E.kp);
    ++E.nlaunch;
}

// ---------------------------------------------------------------------------------------
// Backward (adjoint) helpers of the differentiation form. They follow the context's precision:
// FP64 tables and arithmetic on the FP64 engine; on the mixed engine the FP32 tables of the
// forward with FP32 products and FP64 sums (per tile, chunk or run), like its FP32-pipe passes.

// Structure factor of the dipole set dipbuf ([P][S][3], dipole sites filled) into Sout in the
// forward's rotated form (-Im, Re) of sum_s (k.mu_s) e^{ik.r_s}; beads with bacc[ACC_CONV] != 0
// are skipped. Mixed engine: also the FP32 field weights of Sout (Wf), which the field pass
// of adj_dipole_field reads, so the last structure factor before it must be its own.
// dipf32: the same dipoles as FP32 float4 [P][S] (mixed engine), read by the forward's passes.
void adj_structure_factor(Engine &E, const double *dipbuf, const float4 *dipf32, double2 *Sout, double *bacc) {
    const KP keep = E.kp;
    E.kp.dip = const_cast<double *>(dipbuf);
    E.kp.Sm = Sout;
    E.kp.acc = bacc;
    E.kp.dd_async = 0;
    if (E.precision == PIMD_PREC_MIXED && dipf32) {
        // the forward's own passes on the FP32 copy: tensor cores (the X operand cached by this
        // force call's first iteration), else the register-tiled FP32 pass
        E.kp.dipf = const_cast<float4 *>(dipf32);
        if (!launch_sfac_tc(E, OP_MU, E.kp.fd, E.kp.ld - E.kp.fd, 1)) {
            if (E.sf_tiled && E.sf_nkg_max * SF_RT <= SF_MAXT)
                run_sfac_f<OP_MU>(E, E.kp.fd, E.kp.ld - E.kp.fd, 1);
            else
                run_spass_t<OP_MU, float>(E, E.kp.fd, E.kp.ld - E.kp.fd, 1);
        }
    } else if (E.precision == PIMD_PREC_MIXED) {
        run_spass_t<OP_MU, float>(E, E.kp.fd, E.kp.ld - E.kp.fd, 1);
    } else {
        run_spass_t<OP_MU, double>(E, E.kp.fd, E.kp.ld - E.kp.fd, 1);
    }
    E.kp = keep;
}

// Dr[b][s] += reciprocal dipole field at the dipole sites from the structure factor Sm_u (the
// forward's k_field<F_D> without the SOR update)
__global__ void __launch_bounds__(128) k_adj_fsum(KP kp, int s0, int s1, int nslice, double *Dr) {
    const int b = blockIdx.y, s = s0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= s1 || kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    double E[3] = {0, 0, 0};
    for (int z = 0; z < nslice; z++) {
        const double4_32a p = kp.Fpart[((size_t)z * kp.P + b) * (s1 - s0) + (s - s0)];
        E[0] += p.x;
        E[1] += p.y;
        E[2] += p.z;
    }
    double *o = Dr + 3 * ((size_t)b * kp.S + s);
    o[0] += E[0];
    o[1] += E[1];
    o[2] += E[2];
}

template <int NT, typename R>
static void adj_field_t(Engine &E, double *Dr) {
    const int s0 = E.kp.fd, s1 = E.kp.ld;
    const int LZ = 2 * E.kp.lmax + 1;
    const size_t smem = ((size_t)LZ * NT * 2 + (size_t)KCH * 5) * sizeof(R);
    const int sblocks = (s1 - s0 + NT - 1) / NT;
    const long want = (sizeof(R) == 4 ? 8L : 4L) * 152;
    int ns = (int)((want + (long)sblocks * E.kp.P - 1) / ((long)sblocks * E.kp.P));
    ns = std::max(1, std::min(ns, std::min(E.nchunk, E.max_slices)));
    dim3 g(sblocks, E.kp.P, ns);
    k_field<F_D, NT, R><<<g, NT, smem, E.stream>>>(E.kp, s0, s1);
    dim3 g2((s1 - s0 + 127) / 128, E.kp.P);
    k_adj_fsum<<<g2, 128, 0, E.stream>>>(E.kp, s0, s1, ns, Dr);
    E.nlaunch += 2;
}

template <int LZM>
static void adj_field_f(Engine &E, double *Dr) {
    const int s0 = E.kp.fd, s1 = E.kp.ld;
    const size_t smem = sizeof(float2) * FF_RUNS * LZM;
    const int sblocks = (s1 - s0 + FF_NT - 1) / FF_NT;
    const int cmax = std::min(E.nchunk, E.max_slices);
    const int ns = std::max(1, std::min((int)((8L * 152 + (long)sblocks * E.kp.P - 1) / ((long)sblocks * E.kp.P)), cmax));
    dim3 g(sblocks, E.kp.P, ns);
    k_field_f<F_D, LZM><<<g, FF_NT, smem, E.stream>>>(E.kp, s0, s1);
    dim3 g2((s1 - s0 + 127) / 128, E.kp.P);
    k_adj_fsum<<<g2, 128, 0, E.stream>>>(E.kp, s0, s1, ns, Dr);
    E.nlaunch += 2;
}

// Dr += the reciprocal dipole field of the structure factor Sm_u at the dipole sites (the
// forward's field pass without the SOR update; mixed engine: from the FP32 weights that the
// last adj_structure_factor wrote, which must be Sm_u's)
void adj_dipole_field(Engine &E, double2 *Sm_u, double *bacc, double *Dr) {
    const KP keep = E.kp;
    E.kp.Sm = Sm_u;
    E.kp.acc = bacc;
    const int LZ = 2 * E.kp.lmax + 1;
    if (E.precision == PIMD_PREC_MIXED && E.ff_regs && LZ <= 49) {
        if (LZ <= 17)
            adj_field_f<17>(E, Dr);
        else if (LZ <= 25)
            adj_field_f<25>(E, Dr);
        else if (LZ <= 33)
            adj_field_f<33>(E, Dr);
        else
            adj_field_f<49>(E, Dr);
    } else if (E.precision == PIMD_PREC_MIXED) {
        if ((size_t)LZ * 128 * 8 <= 64 * 1024)
            adj_field_t<128, float>(E, Dr);
        else
            adj_field_t<64, float>(E, Dr);
    } else {
        if ((size_t)LZ * 128 * 16 <= 64 * 1024)
            adj_field_t<128, double>(E, Dr);
        else
            adj_field_t<64, double>(E, Dr);
    }
    E.kp = keep;
}

// Reciprocal-space gradients of the backward, thread per site, direct sum over the
// k-list (c_k = 4 pi A_k / V, S raw = sum (k.mu) e^{ik.r} or sum q e^{ik.r}):
//   BIL  : d/dr_s [u^T D_rec v] = sum_k c_k k [(k.u_s) Im(e_s conj S_v) + (k.v_s) Im(e_s conj S_u)]
//   CROSS: d/dr_s [nu^T E_q,rec] = sum_k c_k k (k.nu_s) Re(e_s conj S_q) (dipole sites)
//                                 - q_s sum_k c_k k Re(e_s conj S_nu)    (charged sites)
//          and the potential of the nu dipoles phi_s = -sum_k c_k Im(e_s conj S_nu).
// Derived from the forward's field formula E_s = sum_k c_k k Im(e_s conj S) (ewald.f90:45-49,
// 114-117): the k-space operator is the Hessian of a quadratic form, so these are exact.
// The mixed engine's instance reads the FP32 tables and forms each product in FP32; each chunk's
// sums go to the FP64 totals. A block stages each chunk's k-vectors, weights and structure
// factors in shared memory (converted once per block, not per site). The k-list is split over
// gridDim.z slices of whole chunks; each slice's per-site sums (G, phi) go to Fpart, and
// k_adj_rfin adds the slices in a fixed order.
enum { ADJ_BIL = 0, ADJ_CROSS = 1 };
template <int MODE, typename R>
__global__ void __launch_bounds__(128) k_adj_rec(KP kp, int s0, int s1, const double *a, const double *bvec,
                                                 const double2 *SA, const double2 *SB, const double *ebw,
                                                 double *grad, double *phi) {
    using V = typename C2<R>::T;
    __shared__ R sk[KCH][4];            // kx, ky, kz, c_k
    __shared__ R s1x[KCH][2], s2x[KCH][2];  // BIL: conj(raw S_u), conj(raw S_v); CROSS: raw S_q, conj(raw S_nu)
    const int b = blockIdx.y, s = s0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (ebw[b] == 0.0) return;  // the whole block: bead inactive
    const bool valid = s < s1;
    const size_t gs = (size_t)b * kp.S + (valid ? s : s0);
    const R q = valid ? R(kp.pos[gs].w) : R(0);
    const bool isdip = valid && s >= kp.fd && s < kp.ld;
    const bool act = (MODE == ADJ_BIL) ? isdip : valid;
    R av[3] = {R(0), R(0), R(0)}, bv[3] = {R(0), R(0), R(0)};
    if (isdip) {
        for (int c = 0; c < 3; c++) {
            av[c] = R(a[3 * gs + c]);
            if (MODE == ADJ_BIL) bv[c] = R(bvec[3 * gs + c]);
        }
    }
    // FP32: this site's kz table column in shared memory (dynamic, (lmax + 1) x 128), read in
    // the k loop instead of from the global table
    extern __shared__ float2 adj_ez[];
    if constexpr (sizeof(R) == 4)
        for (int n = 0; n <= kp.lmax; n++)
            adj_ez[n * 128 + threadIdx.x] = valid ? tab_z<float>(kp, b, n, s) : make_float2(0.f, 0.f);
    double G[3] = {0, 0, 0}, ph = 0.0;
    const int slice = blockIdx.z, nslice = gridDim.z;
    const int c0 = (int)((long)slice * kp.nchunk / nslice), c1 = (int)((long)(slice + 1) * kp.nchunk / nslice);
    for (int chn = c0; chn < c1; chn++) {
        const KChunk ch = kp.chunks[chn];
        __syncthreads();
        for (int i = threadIdx.x; i < ch.k1 - ch.k0; i += blockDim.x) {
            const int k = ch.k0 + i;
            const double4_32a ki = kp.kinfo[k];
            sk[i][0] = R(ki.x);
            sk[i][1] = R(ki.y);
            sk[i][2] = R(ki.z);
            sk[i][3] = R(ki.w);
            const double2 x1 = (MODE == ADJ_BIL) ? SA[(size_t)b * kp.nk + k] : kp.Sq[(size_t)b * kp.nk + k];
            const double2 x2 = (MODE == ADJ_BIL) ? SB[(size_t)b * kp.nk + k] : SA[(size_t)b * kp.nk + k];
            // rotated (-Im, Re) forms: conj(raw) = (y, x); the raw charge structure factor as is
            s1x[i][0] = (MODE == ADJ_BIL) ? R(x1.y) : R(x1.x);
            s1x[i][1] = (MODE == ADJ_BIL) ? R(x1.x) : R(x1.y);
            s2x[i][0] = R(x2.y);
            s2x[i][1] = R(x2.x);
        }
        __syncthreads();
        if (!act) continue;
        // per-chunk partial sums in R, added to the FP64 totals once per chunk (FP64 is a narrow
        // pipe on this part)
        R Gr[3] = {R(0), R(0), R(0)}, phr = R(0);
        for (int r = ch.r0; r < ch.r1; r++) {
            const KRun run = kp.runs[r];
            const V ex = tab_x<R>(kp, b, run.kx, s);
            const V ey = tab_y<R>(kp, b, run.ky, s);
            const V exy = C2<R>::make(ex.x * ey.x - ex.y * ey.y, ex.y * ey.x + ex.x * ey.y);
            const int i0 = run.kbeg - ch.k0;
            for (int j = 0; j < run.nkz; j++) {
                const int kz = run.kzlo + j, i = i0 + j;
                V z;
                if constexpr (sizeof(R) == 4)
                    z = adj_ez[(kz < 0 ? -kz : kz) * 128 + threadIdx.x];
                else
                    z = tab_z<R>(kp, b, kz < 0 ? -kz : kz, s);
                if (kz < 0) z = cconj(z);
                const V e = C2<R>::make(exy.x * z.x - exy.y * z.y, exy.y * z.x + exy.x * z.y);
                const R kv[3] = {sk[i][0], sk[i][1], sk[i][2]}, ck = sk[i][3];
                if (MODE == ADJ_BIL) {
                    const R imu = e.x * s1x[i][1] + e.y * s1x[i][0], imv = e.x * s2x[i][1] + e.y * s2x[i][0];
                    const R ku = kv[0] * av[0] + kv[1] * av[1] + kv[2] * av[2];
                    const R kw = kv[0] * bv[0] + kv[1] * bv[1] + kv[2] * bv[2];
                    const R f = ck * (ku * imv + kw * imu);
                    for (int c = 0; c < 3; c++) Gr[c] += f * kv[c];
                } else {
                    if (isdip) {
                        const R re = e.x * s1x[i][0] + e.y * s1x[i][1];  // Re(e conj Sq)
                        const R kn = kv[0] * av[0] + kv[1] * av[1] + kv[2] * av[2];
                        for (int c = 0; c < 3; c++) Gr[c] += ck * kn * re * kv[c];
                    }
                    if (q != R(0)) {
                        const R re = e.x * s2x[i][0] - e.y * s2x[i][1], im = e.x * s2x[i][1] + e.y * s2x[i][0];
                        for (int c = 0; c < 3; c++) Gr[c] -= q * ck * re * kv[c];
                        phr -= ck * im;
                    }
                }
            }
        }
        for (int c = 0; c < 3; c++) G[c] += (double)Gr[c];
        ph += (double)phr;
    }
    if (valid)
        kp.Fpart[((size_t)slice * kp.P + b) * (s1 - s0) + (s - s0)] = make_double4_32a(G[0], G[1], G[2], ph);
}

// grad += w (sum of the slices' G), phi += w (sum of their potentials) (CROSS), slices in order
template <int MODE>
__global__ void __launch_bounds__(128) k_adj_rfin(KP kp, int s0, int s1, int nslice, const double *ebw, double *grad,
                                                  double *phi) {
    const int b = blockIdx.y, s = s0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= s1 || ebw[b] == 0.0) return;
    double G[3] = {0, 0, 0}, ph = 0.0;
    for (int z = 0; z < nslice; z++) {
        const double4_32a p = kp.Fpart[((size_t)z * kp.P + b) * (s1 - s0) + (s - s0)];
        G[0] += p.x;
        G[1] += p.y;
        G[2] += p.z;
        ph += p.w;
    }
    const size_t gs = (size_t)b * kp.S + s;
    const double w = ebw[b];  // per-bead scale
    for (int c = 0; c < 3; c++) grad[3 * gs + c] += w * G[c];
    if (MODE == ADJ_CROSS && phi) phi[gs] += w * ph;
}

void adj_rec(Engine &E, int mode, const double *a, const double *bvec, const double2 *SA, const double2 *SB,
             const double *ebw, double *grad, double *phi) {
    const int s0 = (mode == ADJ_BIL) ? E.kp.fd : 0, s1 = (mode == ADJ_BIL) ? E.kp.ld : E.kp.S;
    const int sblocks = (s1 - s0 + 127) / 128;
    const int ns = std::max(1, std::min((int)((8L * 152 + (long)sblocks * E.kp.P - 1) / ((long)sblocks * E.kp.P)),
                                        std::min(E.kp.nchunk, E.max_slices)));
    dim3 g(sblocks, E.kp.P, ns), g2(sblocks, E.kp.P);
    const bool f = E.precision == PIMD_PREC_MIXED;
    const size_t ezb = sizeof(float2) * 128 * (E.kp.lmax + 1);  // FP32 kz column, <= 128 KB (lmax <= 127)
    if (f && ezb > 48 * 1024) {
        cudaFuncSetAttribute(k_adj_rec<ADJ_BIL, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ezb);
        cudaFuncSetAttribute(k_adj_rec<ADJ_CROSS, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ezb);
    }
    if (mode == ADJ_BIL) {
        if (f)
            k_adj_rec<ADJ_BIL, float><<<g, 128, ezb, E.stream>>>(E.kp, s0, s1, a, bvec, SA, SB, ebw, grad, phi);
        else
            k_adj_rec<ADJ_BIL, double><<<g, 128, 0, E.stream>>>(E.kp, s0, s1, a, bvec, SA, SB, ebw, grad, phi);
        k_adj_rfin<ADJ_BIL><<<g2, 128, 0, E.stream>>>(E.kp, s0, s1, ns, ebw, grad, phi);
    } else {
        if (f)
            k_adj_rec<ADJ_CROSS, float><<<g, 128, ezb, E.stream>>>(E.kp, s0, s1, a, bvec, SA, SB, ebw, grad, phi);
        else
            k_adj_rec<ADJ_CROSS, double><<<g, 128, 0, E.stream>>>(E.kp, s0, s1, a, bvec, SA, SB, ebw, grad, phi);
        k_adj_rfin<ADJ_CROSS><<<g2, 128, 0, E.stream>>>(E.kp, s0, s1, ns, ebw, grad, phi);
    }
    E.nlaunch += 2;
}

// first site whose charge field is read: TTM3-F never reads the O-site field (no charge, no
// dipole); TTM2.1-F polarises O; the SPC models charge O
static int field_s0(const Engine &E) { return (E.kp.model == 3) ? E.kp.N : 0; }

// ewald_std_qq: S(k) over the charged sites, then the field at the sites that need it
void launch_ewald_sq(Engine &E) { run_spass<OP_Q>(E, E.kp.fq, E.kp.S - E.kp.fq, 0); }
void launch_ewald_fq(Engine &E) { run_field<F_Q>(E, field_s0(E), E.kp.S); }
// one induced-dipole iteration's reciprocal part (ewald_std_dd) fused with the update
void launch_ewald_smu(Engine &E) { run_spass<OP_MU>(E, E.kp.fd, E.kp.ld - E.kp.fd, 1); }
void launch_dd_update(Engine &E) { run_field<F_D>(E, E.kp.fd, E.kp.ld); }
// ewald_std_qd
void launch_ewald_qd(Engine &E) {
    run_spass<OP_DIP>(E, E.kp.fd, E.kp.ld - E.kp.fd, 0);
    launch_qd_virial(E, true);
    run_field<F_QD>(E, field_s0(E), E.kp.S);
}
// ewald_pw_std_qq (ewald.f90:230-291): charge structure factor over all sites, field and
// potential at all sites, reciprocal virial
void launch_ewald_pw(Engine &E) {
    launch_ewald_sq(E);
    launch_ewald_fq(E);
    launch_qd_virial(E, false);
}

}  // namespace pimd
