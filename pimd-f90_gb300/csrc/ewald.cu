// ewald.cu -- Ewald reciprocal-space sums for all beads (FP64).
// Restates pot_ttm/ewald.f90: ssincos (403-437), ewald_std_qq (1-52), ewald_std_dd (56-119),
// ewald_std_qd (123-226), with the k-vector list of ewald_set (293-378).
//
// Structure factors S(k) = sum_s w_s e^{i k.r_s} are k-parallel: a block stages a tile of
// sites' e^{i kz z} tables and the per-(kx,ky)-run products e^{i(kx x + ky y)} in shared
// memory, and each thread owns one k-vector and sums over the tile. Per-tile partial sums go
// to HBM and a second kernel adds them in a fixed order (deterministic, no FP64 atomics).
//
// Fields at the sites are site-parallel: each thread owns one site and walks the k-list run
// by run, using e^{ik.r} = e^{i(kx x+ky y)} e^{i kz z} so that inside a run only the kz
// factor changes: U0 = sum_kz e^{i kz z} W_k, U1 = sum_kz e^{i kz z} W_k kz, then
// E += Im(e^{i(kx x+ky y)} U0) (kx, ky) + Im(e^{i(kx x+ky y)} U1) z-hat, phi += Re(...).
#include "engine.h"

namespace pimd {

PIMD_D double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.y * b.x + a.x * b.y); }
PIMD_D double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// ewald.f90:403-437 ssincos: cos/sin(2 pi n x / L) for n = 0..nmax by the angle-addition
// recurrence from n = 1, each product and sum rounded separately like the reference.
__global__ void __launch_bounds__(128) k_ewald_tables(KP kp) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (s >= kp.S) return;
    const double4_32a r = kp.pos[(size_t)b * kp.S + s];
    const double xyz[3] = {r.x, r.y, r.z};
    const int nmx[3] = {kp.hmax, kp.kmax, kp.lmax};
    int off = 0;
    double2 *T = kp.tab + (size_t)b * kp.ntab * kp.S + s;
    for (int d = 0; d < 3; d++) {
        T[(size_t)off * kp.S] = make_double2(1.0, 0.0);
        if (nmx[d] >= 1) {
            const double arg = __dmul_rn(__dmul_rn(TWOPI, kp.boxi[d]), xyz[d]);
            const double c1 = cos(arg), s1 = sin(arg);
            double c = c1, sn = s1;
            T[(size_t)(off + 1) * kp.S] = make_double2(c1, s1);
            for (int n = 2; n <= nmx[d]; n++) {
                const double cn = __dsub_rn(__dmul_rn(c, c1), __dmul_rn(sn, s1));
                const double snn = __dadd_rn(__dmul_rn(c, s1), __dmul_rn(sn, c1));
                c = cn;
                sn = snn;
                T[(size_t)(off + n) * kp.S] = make_double2(c, sn);
            }
        }
        off += nmx[d] + 1;
    }
}

enum { OP_Q = 0, OP_MU = 1, OP_DIP = 2 };
constexpr int SP_NT = 256;  // threads (k-vectors) per structure-factor block
constexpr int SP_TS = 64;   // sites per shared-memory tile

PIMD_D double2 tab_x(const KP &kp, int b, int n, int s) {
    return kp.tab[((size_t)b * kp.ntab + n) * kp.S + s];
}
PIMD_D double2 tab_y(const KP &kp, int b, int n, int s) {
    const double2 v = kp.tab[((size_t)b * kp.ntab + kp.hmax + 1 + (n < 0 ? -n : n)) * kp.S + s];
    return n < 0 ? cconj(v) : v;
}
PIMD_D double2 tab_z(const KP &kp, int b, int n, int s) {
    return kp.tab[((size_t)b * kp.ntab + kp.hmax + 1 + kp.kmax + 1 + n) * kp.S + s];
}

// Per-tile partial structure factors.
//   OP_Q : sum_s q_s e_s                        (ewald.f90:41-42)
//   OP_MU: sum_s (k.mu_s) e_s                   (ewald.f90:99-108)
//   OP_DIP: sum_s mu_{s,c} e_s, c = x, y, z     (ewald.f90:208-213)
template <int OP>
__global__ void __launch_bounds__(SP_NT) k_spass(KP kp, int s0, int nsites, int tsg, int ngroups, int skipconv) {
    constexpr int NC = (OP == OP_DIP) ? 3 : 1;
    const int b = blockIdx.z;
    if (skipconv && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    const int grp = blockIdx.y;
    const KChunk ch = kp.chunks[blockIdx.x];
    const int nr = ch.r1 - ch.r0;
    const int LZ = 2 * kp.lmax + 1;
    extern __shared__ double smem[];
    double2 *ez = reinterpret_cast<double2 *>(smem);        // [TS][LZ]
    double2 *exy = ez + SP_TS * LZ;                          // [TS][nr]
    double *aa = reinterpret_cast<double *>(exy + SP_TS * nr);  // [TS][nr] (OP_MU)
    double *wt = aa + SP_TS * nr;                            // [TS][4]
    const int k = ch.k0 + threadIdx.x;
    const bool valid = k < ch.k1;
    int rk = 0, kz = 0;
    double kzv = 0.0;
    if (valid) {
        const int2 ki = kp.kidx[k];
        rk = ki.x - ch.r0;
        kz = ki.y;
        kzv = kp.kinfo[k].z;
    }
    double2 acc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = make_double2(0.0, 0.0);
    const int gbeg = s0 + grp * tsg, gend = min(s0 + nsites, gbeg + tsg);
    for (int sb = gbeg; sb < gend; sb += SP_TS) {
        const int nloc = min(SP_TS, gend - sb);
        __syncthreads();
        if (threadIdx.x < nloc) {
            const size_t gs = (size_t)b * kp.S + sb + threadIdx.x;
            if (OP == OP_Q) {
                wt[4 * threadIdx.x] = kp.pos[gs].w;
            } else {
                wt[4 * threadIdx.x + 0] = kp.dip[3 * gs + 0];
                wt[4 * threadIdx.x + 1] = kp.dip[3 * gs + 1];
                wt[4 * threadIdx.x + 2] = kp.dip[3 * gs + 2];
            }
        }
        for (int idx = threadIdx.x; idx < nloc * (kp.lmax + 1); idx += SP_NT) {
            const int site = idx % nloc, n = idx / nloc;
            const double2 v = tab_z(kp, b, n, sb + site);
            ez[site * LZ + kp.lmax + n] = v;
            ez[site * LZ + kp.lmax - n] = cconj(v);
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < nloc * nr; idx += SP_NT) {
            const int site = idx % nloc, r = idx / nloc;
            const KRun run = kp.runs[ch.r0 + r];
            const double2 ex = tab_x(kp, b, run.kx, sb + site);
            const double2 ey = tab_y(kp, b, run.ky, sb + site);
            // ewald.f90:30-31: coskxky = cx cy - sx sy, sinkxky = sx cy + cx sy
            exy[site * nr + r] = make_double2(ex.x * ey.x - ex.y * ey.y, ex.y * ey.x + ex.x * ey.y);
            if (OP == OP_MU) {
                const double4_32a kv = kp.kinfo[run.kbeg];
                aa[site * nr + r] = kv.x * wt[4 * site] + kv.y * wt[4 * site + 1];
            }
        }
        __syncthreads();
        if (valid) {
            for (int site = 0; site < nloc; site++) {
                const double2 a = exy[site * nr + rk];
                const double2 z = ez[site * LZ + kp.lmax + kz];
                // ewald.f90:37-39: coskr = cxy cz - sxy sz, sinkr = sxy cz + cxy sz
                const double2 e = make_double2(a.x * z.x - a.y * z.y, a.y * z.x + a.x * z.y);
                if (OP == OP_Q) {
                    const double q = wt[4 * site];
                    acc[0].x += q * e.x;
                    acc[0].y += q * e.y;
                } else if (OP == OP_MU) {
                    const double t = aa[site * nr + rk] + kzv * wt[4 * site + 2];
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
        double2 *out = kp.Spart + (((size_t)b * ngroups + grp) * kp.nk + k) * NC;
#pragma unroll
        for (int c = 0; c < NC; c++) out[c] = acc[c];
    }
}

// Sum the tile partials in a fixed order. OP_MU stores (rQm, iQm) = (-Im, Re) of
// sum (k.mu) e (ewald.f90:106-107).
template <int OP>
__global__ void __launch_bounds__(256) k_sreduce(KP kp, int ngroups, int skipconv) {
    constexpr int NC = (OP == OP_DIP) ? 3 : 1;
    const int k = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (k >= kp.nk) return;
    if (skipconv && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    double2 s[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) s[c] = make_double2(0.0, 0.0);
    for (int g = 0; g < ngroups; g++) {
        const double2 *p = kp.Spart + (((size_t)b * ngroups + g) * kp.nk + k) * NC;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            s[c].x += p[c].x;
            s[c].y += p[c].y;
        }
    }
    if (OP == OP_Q) kp.Sq[(size_t)b * kp.nk + k] = s[0];
    if (OP == OP_MU) kp.Sm[(size_t)b * kp.nk + k] = make_double2(-s[0].y, s[0].x);
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

template <int MODE, int NT>
__global__ void __launch_bounds__(NT) k_field(KP kp, int s0, int s1, int iter) {
    const int b = blockIdx.y;
    if (MODE == F_D && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    const int s = s0 + blockIdx.x * NT + threadIdx.x;
    const bool valid = s < s1;
    const int LZ = 2 * kp.lmax + 1;
    extern __shared__ double smem[];
    double2 *ez = reinterpret_cast<double2 *>(smem);  // [LZ][NT]
    double2 *W1 = ez + LZ * NT;                        // [KCH]
    double2 *W2 = W1 + KCH;                            // [KCH] (QD)
    double *kzs = reinterpret_cast<double *>(W2 + KCH);  // [KCH]
    const size_t gs = (size_t)b * kp.S + (valid ? s : s0);
    for (int n = 0; n <= kp.lmax; n++) {
        const double2 v = valid ? tab_z(kp, b, n, s) : make_double2(0.0, 0.0);
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
    double E[3] = {0, 0, 0}, phi = 0.0, G[3] = {0, 0, 0};
    const double2 *S1 = (MODE == F_Q) ? kp.Sq : kp.Sm;
    for (int chn = 0; chn < kp.nchunk; chn++) {
        const KChunk ch = kp.chunks[chn];
        __syncthreads();
        for (int i = threadIdx.x; i < ch.k1 - ch.k0; i += NT) {
            const int k = ch.k0 + i;
            const double4_32a ki = kp.kinfo[k];
            const double2 a = S1[(size_t)b * kp.nk + k];
            W1[i] = make_double2(ki.w * a.x, -ki.w * a.y);  // 4 pi Ak / V conj(S)
            if (MODE == F_QD) {
                const double2 c = kp.Sq[(size_t)b * kp.nk + k];
                W2[i] = make_double2(ki.w * (c.x + a.x), -ki.w * (c.y + a.y));
            }
            kzs[i] = ki.z;
        }
        __syncthreads();
        if (!valid) continue;
        for (int r = ch.r0; r < ch.r1; r++) {
            const KRun run = kp.runs[r];
            const double4_32a kv = kp.kinfo[run.kbeg];
            const double2 ex = tab_x(kp, b, run.kx, s);
            const double2 ey = tab_y(kp, b, run.ky, s);
            const double2 exy = make_double2(ex.x * ey.x - ex.y * ey.y, ex.y * ey.x + ex.x * ey.y);
            double2 U0 = make_double2(0, 0), U1 = make_double2(0, 0);
            double2 V0 = make_double2(0, 0), V1 = make_double2(0, 0), V2 = make_double2(0, 0);
            const int i0 = run.kbeg - ch.k0;
            for (int j = 0; j < run.nkz; j++) {
                const double2 z = ez[(kp.lmax + run.kzlo + j) * NT + threadIdx.x];
                const double kz = kzs[i0 + j];
                const double2 t = cmul(z, W1[i0 + j]);
                U0.x += t.x;
                U0.y += t.y;
                U1.x += kz * t.x;
                U1.y += kz * t.y;
                if (MODE == F_QD && isdip) {
                    const double2 u = cmul(z, W2[i0 + j]);
                    V0.x += u.x;
                    V0.y += u.y;
                    V1.x += kz * u.x;
                    V1.y += kz * u.y;
                    V2.x += kz * kz * u.x;
                    V2.y += kz * kz * u.y;
                }
            }
            const double2 z0 = cmul(exy, U0), z1 = cmul(exy, U1);
            if (MODE == F_QD) {
                phi += z0.x;
                G[0] -= q * z0.y * kv.x;
                G[1] -= q * z0.y * kv.y;
                G[2] -= q * z1.y;
                if (isdip) {
                    const double R0 = exy.x * V0.x - exy.y * V0.y;
                    const double R1 = exy.x * V1.x - exy.y * V1.y;
                    const double R2 = exy.x * V2.x - exy.y * V2.y;
                    const double a = kv.x * mu[0] + kv.y * mu[1];
                    G[0] -= kv.x * (a * R0 + mu[2] * R1);
                    G[1] -= kv.y * (a * R0 + mu[2] * R1);
                    G[2] -= a * R1 + mu[2] * R2;
                }
            } else {
                phi += z0.x;
                E[0] += z0.y * kv.x;
                E[1] += z0.y * kv.y;
                E[2] += z1.y;
            }
        }
    }
    if (MODE == F_Q) {
        if (valid) {
            double4_32a f = kp.F[gs];
            f.x += E[0];
            f.y += E[1];
            f.z += E[2];
            if (s >= kp.N) f.w += phi;
            kp.F[gs] = f;
        }
    } else if (MODE == F_QD) {
        if (valid) {
            if (s >= kp.N) kp.F[gs].w += phi;
            kp.dR[3 * gs + 0] += G[0];
            kp.dR[3 * gs + 1] += G[1];
            kp.dR[3 * gs + 2] += G[2];
        }
    } else {
        // pot_ttm.f90:371-381 Efd = Efd_real + Efd_rec + Efq + factor mu; SOR update
        double av[2] = {0.0, 0.0};
        if (valid) {
            const double4_32a f = kp.F[gs];
            const double efq[3] = {f.x, f.y, f.z};
            const int kind = s / kp.N + 1;
            const double pol = kp.polar_sor * kp.polar[kind];
            double mn[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double efd = (kp.Efdr[3 * gs + c] + E[c]) + efq[c] + kp.factor * mu[c];
                mn[c] = (1.0 - kp.polar_sor) * mu[c] + pol * efd;
                const double dd = (iter == 1) ? mn[c] : mn[c] - mu[c];
                av[0] += dd * dd;
                av[1] += mn[c] * efq[c];
                kp.dip[3 * gs + c] = mn[c];
                kp.Efdr[3 * gs + c] = 0.0;
            }
        }
        // reduce into acc[ACC_DSQ], acc[ACC_MUEFQ]
        __shared__ double red[NT / 32][2];
        const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
        for (int i = 0; i < 2; i++) {
            double x = av[i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) red[wp][i] = x;
        }
        __syncthreads();
        if (threadIdx.x < 2) {
            double t = 0;
            for (int w = 0; w < NT / 32; w++) t += red[w][threadIdx.x];
            atomicAdd(kp.acc + (size_t)b * NACC + ACC_DSQ + threadIdx.x, t);
        }
    }
}

// ewald.f90:194-224: reciprocal-space virial, one thread per (k, bead)
__global__ void __launch_bounds__(128) k_qd_virial(KP kp) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    double av[14];
#pragma unroll
    for (int i = 0; i < 14; i++) av[i] = 0.0;
    if (k < kp.nk) {
        const double4_32a ki = kp.kinfo[k];
        const double kv[3] = {ki.x, ki.y, ki.z};
        const double Akk = kp.kAk[k];
        const double2 sq = kp.Sq[(size_t)b * kp.nk + k], sm = kp.Sm[(size_t)b * kp.nk + k];
        const double rQqm = sq.x + sm.x, iQqm = sq.y + sm.y;
        const double ksq = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
        const double coeff2 = 2.0 / ksq + 0.5 / (kp.ew.aewald * kp.ew.aewald);
        const double Ureck = Akk * (rQqm * rQqm + iQqm * iQqm);
        double rdip[3] = {0, 0, 0}, idip[3] = {0, 0, 0};
        if (kp.Sdip) {
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
        av[ACC_VIRIALC] = av[ACC_VIRT + 0] + av[ACC_VIRT + 4] + av[ACC_VIRT + 8];
    }
    block_reduce_add<14, 128>(av, kp.acc + (size_t)b * NACC);
}

// ---------------------------------------------------------------------------------------
static int spass_groups(const Engine &E, int nsites) {
    const int ntile = (nsites + SP_TS - 1) / SP_TS;
    const long per = (long)E.nchunk * E.kp.P;
    int g = (int)((152L * 8 + per - 1) / per);
    if (g < 1) g = 1;
    if (g > ntile) g = ntile;
    return g;
}

template <int OP>
static void run_spass(Engine &E, int s0, int nsites, int skipconv) {
    const int ng = spass_groups(E, nsites);
    const int ntile = (nsites + SP_TS - 1) / SP_TS;
    const int tsg = ((ntile + ng - 1) / ng) * SP_TS;
    const int ngr = (nsites + tsg - 1) / tsg;
    const int LZ = 2 * E.kp.lmax + 1;
    const size_t smem = (size_t)SP_TS * LZ * 16 + (size_t)SP_TS * E.max_runs_chunk * 16 +
                        (size_t)SP_TS * E.max_runs_chunk * 8 + (size_t)SP_TS * 4 * 8;
    static bool attr_set[3] = {false, false, false};
    if (!attr_set[OP]) {
        cudaFuncSetAttribute(k_spass<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set[OP] = true;
    }
    dim3 g(E.nchunk, ngr, E.kp.P);
    k_spass<OP><<<g, SP_NT, smem, E.stream>>>(E.kp, s0, nsites, tsg, ngr, skipconv); ++E.nlaunch;
    dim3 g2((E.kp.nk + 255) / 256, E.kp.P);
    k_sreduce<OP><<<g2, 256, 0, E.stream>>>(E.kp, ngr, skipconv); ++E.nlaunch;
}

template <int MODE>
static void run_field(Engine &E, int s0, int s1, int iter) {
    const int LZ = 2 * E.kp.lmax + 1;
    const size_t base = (size_t)KCH * (16 + 16 + 8);
    if ((size_t)LZ * 128 * 16 + base <= 96 * 1024) {
        constexpr int NT = 128;
        const size_t smem = (size_t)LZ * NT * 16 + base;
        static bool set = false;
        if (!set) {
            cudaFuncSetAttribute(k_field<MODE, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            set = true;
        }
        dim3 g((s1 - s0 + NT - 1) / NT, E.kp.P);
        k_field<MODE, NT><<<g, NT, smem, E.stream>>>(E.kp, s0, s1, iter); ++E.nlaunch;
    } else {
        constexpr int NT = 64;
        const size_t smem = (size_t)LZ * NT * 16 + base;
        static bool set = false;
        if (!set) {
            cudaFuncSetAttribute(k_field<MODE, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            set = true;
        }
        dim3 g((s1 - s0 + NT - 1) / NT, E.kp.P);
        k_field<MODE, NT><<<g, NT, smem, E.stream>>>(E.kp, s0, s1, iter); ++E.nlaunch;
    }
}

void launch_ewald_tables(Engine &E) {
    dim3 g((E.kp.S + 127) / 128, E.kp.P);
    k_ewald_tables<<<g, 128, 0, E.stream>>>(E.kp); ++E.nlaunch;
}

// ewald_std_qq: S(k) over the charged sites, then the field at the sites that need it
void launch_ewald_sq(Engine &E) {
    const int N = E.kp.N;
    run_spass<OP_Q>(E, N, E.kp.S - N, 0);
}
void launch_ewald_fq(Engine &E) {
    const int N = E.kp.N;
    // TTM3-F never reads the O-site field (no charge, no dipole); TTM2.1-F polarises O
    const int s0 = (E.kp.model == 2) ? 0 : N;
    run_field<F_Q>(E, s0, E.kp.S, 0);
}
// one induced-dipole iteration's reciprocal part (ewald_std_dd) fused with the update
void launch_ewald_smu(Engine &E) { run_spass<OP_MU>(E, E.kp.fd, E.kp.ld - E.kp.fd, 1); }
void launch_dd_update(Engine &E, int iter) { run_field<F_D>(E, E.kp.fd, E.kp.ld, iter); }
// ewald_std_qd
void launch_ewald_qd(Engine &E) {
    run_spass<OP_DIP>(E, E.kp.fd, E.kp.ld - E.kp.fd, 0);
    dim3 g((E.kp.nk + 127) / 128, E.kp.P);
    k_qd_virial<<<g, 128, 0, E.stream>>>(E.kp); ++E.nlaunch;
    const int s0 = (E.kp.model == 2) ? 0 : E.kp.N;
    run_field<F_QD>(E, s0, E.kp.S, 0);
}

}  // namespace pimd
