// Tensor-core (tcgen05) dipole structure factor of the mixed engine:
//   S(k) = sum_s (k.mu_s) e^{i k.r_s}            (ewald.f90:99-108, the per-iteration ewald_std_dd sum)
// over the dipole sites of every bead, as 3xTF32 GEMMs with FP32 accumulators in TMEM.
//
// Formulation. For a run (kx, ky) with kz in [kzlo, kzlo + nkz) and a site s, e^{ik.r} =
// exy(s) ez(s, kz) with exy = ex(kx) ey(ky) (ewald.f90:30-31). Writing
//   A0 = (kx mu_x + ky mu_y) exy,   A1 = mu_z exy,   S(kz) = G0(kz) + kz G1(kz),
//   Gi(kz) = sum_s Ai(s) ez(s, kz),
// and ez(-j) = conj ez(j) = c_j - i s_j, every Gi(+-j) follows from the four real sums
//   Ar.c_j, Ar.s_j, Ai.c_j, Ai.s_j   (j = |kz| >= 0):
//   G(+j) = (Ar.c - Ai.s) + i (Ar.s + Ai.c),   G(-j) = (Ar.c + Ai.s) + i (Ai.c - Ar.s).
// So one real GEMM per bead, D[(run, component)][(j, cos|sin)] = sum_s A[.][s] B[.][s], with four
// components (A0 re, A0 im, A1 re, A1 im) per run, gives every k-vector: half the products of
// the direct complex sum over kz in [-m, m]. Rows of an M = 128 tile hold 32 runs (runs sorted by
// kz extent, so a tile's N = 2 (max |kz| + 1), rounded up to 16, is tight); row = 32 component
// + run slot, so the A stores of a warp fill whole 128-byte lines.
//
// Pipeline of one CTA (a bead, a group of consecutive sites, a group of <= 8 tiles):
//   * TMA (cp.async.bulk.tensor.2d, two boxes of 16 sites x all ntab rows, 128-byte swizzle)
//     brings the FP32 tables of 32 sites into a double-buffered stage, completing on an mbarrier;
//   * per 8 sites (one kind::tf32 K step) all threads build A (the tiles' 4 x 32 rows) and B
//     (ez cos/sin rows) in the canonical no-swizzle K-major layout, split into TF32 hi + lo;
//   * one thread issues hi.hi + hi.lo + lo.hi per tile into the tile's TMEM columns and commits
//     to the buffer's mbarrier, so the MMAs of step i run while step i + 1 is built;
//   * the epilogue reads TMEM (tcgen05.ld), combines the four components of each run through
//     shared memory and writes the FP32 partial S of every k of its runs to Spart, which
//     k_sreduce adds in FP64 in a fixed order, as for the other structure-factor kernels.
// Every mbarrier wait is bounded (~0.13 s); after a timeout the CTA stops issuing work, waits
// (bounded) for its MMAs in flight, frees its TMEM and returns, and bit 8 of the context's error
// word is set.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <algorithm>
#include <vector>

#include "engine.h"
#include "umma.cuh"

namespace pimd {

constexpr int TC_NT = 256;     // threads per CTA (8 warps)
constexpr int TC_RUNS = 32;    // runs per M tile (4 rows each)
constexpr int TC_TGMAX = 8;    // M tiles per CTA
constexpr int TC_SS = 32;      // sites per table stage (two TMA boxes)
constexpr int TC_KS = 8;       // sites per MMA step
constexpr long long TC_WAIT = 1LL << 28;  // cycles before a wait gives up (~0.13 s)

struct TcArgs {
    const int4 *tile;  // coff, N, J, first slot in run
    const int *run;    // [tiles][32]
    const int4 *grp;   // t0, nt, ncols
    int ntg;           // tile groups
    int ngroups;       // site groups
    int sbase;         // first site of group 0 (multiple of 32, <= s_lo)
    int s_lo, s_hi;    // dipole sites [s_lo, s_hi)
    int tsg;           // sites per group (multiple of 32)
    int nrows;         // B rows (max N over tiles)
    int jmax;          // ez rows used (max J over tiles)
    int skipconv;
};

// Shared-memory carve-up (bytes from a 1024-aligned base), used by the kernel and the launcher.
// A table stage is two TMA boxes of 16 sites x ntab rows, each written with the 128-byte swizzle
// (16-byte chunk c of row r lands at chunk c ^ (r & 7)), so loads of the same sites from
// different rows fall in different banks.
struct TcSmem {
    int boxb, stage, A, B, mu, total, astride;
    __host__ __device__ TcSmem(int ntab, int tg, int nrows) {
        boxb = ((ntab * 128 + 1023) / 1024) * 1024;
        stage = 2 * boxb;
        A = 2 * stage;                     // [2 buffers][hi tiles | lo tiles][4 KB]
        astride = 2 * tg * 4096;
        B = A + 2 * astride;               // [2 buffers][hi | lo][nrows][32 B]
        mu = B + 2 * 2 * nrows * 32;       // [2][32] float4
        total = mu + 2 * TC_SS * 16 + 1024;  // + alignment slack of the dynamic base
    }
};

// 16-byte chunk holding sites (site, site + 1) of table row `row` in a swizzled stage
PIMD_D const float4 *tab_chunk(const unsigned char *stage, int boxb, int row, int site) {
    const int c = (site & 15) >> 1;
    return reinterpret_cast<const float4 *>(stage + (site >> 4) * boxb + row * 128 + ((c ^ (row & 7)) << 4));
}
PIMD_D float2 tab_elem(const unsigned char *stage, int boxb, int row, int site) {
    const float2 *p = reinterpret_cast<const float2 *>(tab_chunk(stage, boxb, row, site & ~1));
    return p[site & 1];
}

PIMD_D void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            umma::smem_u32(dst)),
        "l"((unsigned long long)map), "r"(x), "r"(y), "r"(umma::smem_u32(bar))
        : "memory");
}
PIMD_D void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(umma::smem_u32(bar)), "r"(bytes) : "memory");
}
// TF32 split by truncation: hi keeps the top 10 mantissa bits, lo = x - hi exactly
PIMD_D void split_t(float x, float &hi, float &lo) {
    hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
    lo = x - hi;
}

__global__ void __launch_bounds__(TC_NT, 1) k_sfac_tc(const __grid_constant__ CUtensorMap tmap, KP kp, TcArgs a) {
    const int b = blockIdx.y;
    if (a.skipconv && kp.acc[(size_t)b * NACC + ACC_CONV] != 0.0) return;
    const int tg = blockIdx.x % a.ntg, grp = blockIdx.x / a.ntg;
    const int4 gi = a.grp[tg];
    const int t0 = gi.x, nt = gi.y;
    const uint32_t ncols = (uint32_t)gi.z;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const TcSmem L(kp.ntab, TC_TGMAX, a.nrows);
    extern __shared__ __align__(1024) unsigned char sm_raw[];
    // the swizzle pattern follows shared-memory address bits 7-9: align the base to 1024 bytes
    unsigned char *sm = sm_raw + ((1024u - (umma::smem_u32(sm_raw) & 1023u)) & 1023u);
    __shared__ uint64_t tbar[2], mbar[2];
    __shared__ uint32_t tslot;
    __shared__ int4 stile[TC_TGMAX];
    float4 *smu = reinterpret_cast<float4 *>(sm + L.mu);

    const int g0 = a.sbase + grp * a.tsg;
    const int g1 = min(a.s_hi, g0 + a.tsg);
    const int nstage = (g1 - g0 + TC_SS - 1) / TC_SS;
    const int yrow = kp.hmax + 1;            // first ey row (ky = 0)
    const int zrow = yrow + kp.kmax + 1;     // first ez row (kz = 0)
    const uint32_t box_tx = (uint32_t)(kp.ntab * 128);

    // per-thread A items (tile, run slot q, site quad h), at most two: rows 32 c + q of the tile
    int it_n = 0;
    int it_off[2], it_xr[2], it_yr[2], it_h[2];
    float it_kx[2], it_ky[2], it_ys[2];
    bool it_ok[2];
#pragma unroll
    for (int u = 0; u < 2; u++) {
        const int it = tid + u * TC_NT;
        it_ok[u] = false;
        it_off[u] = it_xr[u] = it_yr[u] = it_h[u] = 0;
        it_kx[u] = it_ky[u] = 0.f;
        it_ys[u] = 1.f;
        if (it >= nt * 64) continue;
        it_n = u + 1;
        const int t = it >> 6, q = (it >> 1) & 31, h = it & 1;
        const int4 ti = a.tile[t0 + t];
        const int r = a.run[ti.w + q];
        // byte offset of (row q, K quad h) in tile t of the hi operand; component c adds 1024 c
        it_off[u] = t * 4096 + (((q >> 3) * 2 + h) << 7) + ((q & 7) << 4);
        it_h[u] = h;
        if (r >= 0) {
            const KRun run = kp.runs[r];
            const float2 kv = kp.runkf[r];
            it_ok[u] = true;
            it_xr[u] = run.kx;
            it_yr[u] = yrow + (run.ky < 0 ? -run.ky : run.ky);
            it_ys[u] = run.ky < 0 ? -1.f : 1.f;
            it_kx[u] = kv.x;
            it_ky[u] = kv.y;
        }
    }
    if (tid < nt) stile[tid] = a.tile[t0 + tid];

    if (warp == 0) umma::tmem_alloc(&tslot, ncols);
    if (tid == 0) {
        umma::mbar_init(&tbar[0], 1);
        umma::mbar_init(&tbar[1], 1);
        umma::mbar_init(&mbar[0], 1);
        umma::mbar_init(&mbar[1], 1);
    }
    {   // B rows n >= 2 jmax stay zero in both buffers (hi and lo)
        const int per = a.nrows * 8, pad0 = 2 * a.jmax;
        float *Bf = reinterpret_cast<float *>(sm + L.B);
        for (int i = tid; i < 4 * per; i += TC_NT) {
            const int f = i % per;
            const int n = ((f >> 5) >> 1) * 8 + ((f & 31) >> 2);
            if (n >= pad0) Bf[i] = 0.f;
        }
    }
    auto load_mu = [&](int stage, int buf) {
        if (tid < TC_SS) {
            const int s = g0 + stage * TC_SS + tid;
            float4 m = make_float4(0.f, 0.f, 0.f, 0.f);
            if (s >= a.s_lo && s < g1) m = kp.dipf[(size_t)b * kp.S + s];
            smu[buf * TC_SS + tid] = m;
        }
    };
    auto load_tab = [&](int stage, int buf) {  // thread 0
        uint64_t *bar = &tbar[buf];
        unsigned char *dst = sm + buf * L.stage;
        const int x = 2 * (g0 + stage * TC_SS);
        mbar_expect_tx(bar, 2 * box_tx);
        tma_load_2d(dst, &tmap, x, b * kp.ntab, bar);
        tma_load_2d(dst + L.boxb, &tmap, x + 2 * 16, b * kp.ntab, bar);
    };
    load_mu(0, 0);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tm = tslot;
    if (tid == 0) load_tab(0, 0);
    int issued = 1, landed = 0;  // table stages requested / seen complete
    uint32_t err = 0;
    bool bad = false;  // a wait timed out somewhere in the CTA: stop issuing, free TMEM, return
    int sub = 0;
    const uint32_t idesc_base = umma::idesc_tf32(128, 16) & ~(0x3Fu << 17);
    for (int ts = 0; ts < nstage && !bad; ts++) {
        const int tb = ts & 1;
        if (ts + 1 < nstage) {  // both buffers of stage ts - 1 were last read before the last barrier
            if (tid == 0) load_tab(ts + 1, tb ^ 1);
            load_mu(ts + 1, tb ^ 1);
            issued = ts + 2;
        }
        {
            const int to = umma::mbar_wait(&tbar[tb], (uint32_t)((ts >> 1) & 1), TC_WAIT);
            err |= (uint32_t)to;
            if (!to) landed = ts + 1;
        }
        const unsigned char *tab = sm + tb * L.stage;
        const float4 *mus = smu + tb * TC_SS;
        for (int ks = 0; ks < TC_SS / TC_KS; ks++, sub++) {
            const int ab = sub & 1;
            if (sub >= 2) err |= (uint32_t)umma::mbar_wait(&mbar[ab], (uint32_t)(((sub - 2) >> 1) & 1), TC_WAIT);
            unsigned char *Ab = sm + L.A + ab * L.astride;
            unsigned char *Bb = sm + L.B + ab * 2 * a.nrows * 32;
            const int so = ks * TC_KS;
#pragma unroll
            for (int u = 0; u < 2; u++) {
                if (u >= it_n) break;
                float4 c[4];
                if (it_ok[u]) {
                    const int sq = so + 4 * it_h[u];
                    const float4 x01 = *tab_chunk(tab, L.boxb, it_xr[u], sq);
                    const float4 x23 = *tab_chunk(tab, L.boxb, it_xr[u], sq + 2);
                    const float4 y01 = *tab_chunk(tab, L.boxb, it_yr[u], sq);
                    const float4 y23 = *tab_chunk(tab, L.boxb, it_yr[u], sq + 2);
                    const float ys = it_ys[u];
                    const float ex[4][2] = {{x01.x, x01.y}, {x01.z, x01.w}, {x23.x, x23.y}, {x23.z, x23.w}};
                    const float ey[4][2] = {{y01.x, ys * y01.y}, {y01.z, ys * y01.w}, {y23.x, ys * y23.y}, {y23.z, ys * y23.w}};
                    float v[4][4];
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const float4 m = mus[sq + i];
                        // ewald.f90:30-31: coskxky = cx cy - sx sy, sinkxky = sx cy + cx sy
                        const float er = ex[i][0] * ey[i][0] - ex[i][1] * ey[i][1];
                        const float ei = ex[i][1] * ey[i][0] + ex[i][0] * ey[i][1];
                        const float t = fmaf(it_kx[u], m.x, it_ky[u] * m.y);  // k.mu without k_z
                        v[0][i] = t * er;
                        v[1][i] = t * ei;
                        v[2][i] = m.z * er;
                        v[3][i] = m.z * ei;
                    }
#pragma unroll
                    for (int cc = 0; cc < 4; cc++) c[cc] = make_float4(v[cc][0], v[cc][1], v[cc][2], v[cc][3]);
                } else {
#pragma unroll
                    for (int cc = 0; cc < 4; cc++) c[cc] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int cc = 0; cc < 4; cc++) {
                    float4 hi, lo;
                    split_t(c[cc].x, hi.x, lo.x);
                    split_t(c[cc].y, hi.y, lo.y);
                    split_t(c[cc].z, hi.z, lo.z);
                    split_t(c[cc].w, hi.w, lo.w);
                    *reinterpret_cast<float4 *>(Ab + it_off[u] + cc * 1024) = hi;
                    *reinterpret_cast<float4 *>(Ab + nt * 4096 + it_off[u] + cc * 1024) = lo;
                }
            }
            // B rows 2j (cos) and 2j + 1 (sin) of ez, K = the step's 8 sites
            if (tid < a.jmax * TC_KS) {
                const int j = tid >> 3, k = tid & 7;
                const float2 z = tab_elem(tab, L.boxb, zrow + j, so + k);
                float *Bh = reinterpret_cast<float *>(Bb);
                float *Bl = Bh + a.nrows * 8;
                const int n0 = 2 * j, n1 = 2 * j + 1;
                const int o0 = (umma::kmajor_off(n0, k, 2)) >> 2;
                const int o1 = (umma::kmajor_off(n1, k, 2)) >> 2;
                float hi, lo;
                split_t(z.x, hi, lo);
                Bh[o0] = hi;
                Bl[o0] = lo;
                split_t(z.y, hi, lo);
                Bh[o1] = hi;
                Bl[o1] = lo;
            }
            umma::fence_smem_to_async();
            if (__syncthreads_or((int)err)) {
                bad = true;
                break;
            }
            if (tid == 0) {
                umma::fence_after_sync();
                const uint32_t aH = umma::smem_u32(Ab), aL = aH + nt * 4096;
                const uint32_t bH = umma::smem_u32(Bb), bL = bH + a.nrows * 32;
                const uint64_t db_h = umma::sdesc(bH, 128, 256), db_l = umma::sdesc(bL, 128, 256);
                for (int t = 0; t < nt; t++) {
                    const int4 ti = stile[t];
                    const uint32_t id = idesc_base | ((uint32_t)(ti.y >> 3) << 17);
                    const uint32_t d = tm + (uint32_t)ti.x;
                    const uint64_t da_h = umma::sdesc(aH + t * 4096, 128, 256), da_l = umma::sdesc(aL + t * 4096, 128, 256);
                    umma::mma_tf32(d, da_h, db_h, id, sub > 0);
                    umma::mma_tf32(d, da_h, db_l, id, 1);
                    umma::mma_tf32(d, da_l, db_h, id, 1);
                }
                umma::commit(&mbar[ab]);
            }
        }
    }
    // all MMAs done: the last commit tracks every earlier MMA of the issuing thread
    if (sub > 0) {
        const int last = sub - 1;
        int to = umma::mbar_wait(&mbar[last & 1], (uint32_t)((last >> 1) & 1), TC_WAIT);
        if (to) to = umma::mbar_wait(&mbar[last & 1], (uint32_t)((last >> 1) & 1), TC_WAIT);
        err |= (uint32_t)to;
    }
    // table copies still in flight after a timeout land before the CTA leaves
    for (int w = landed; w < issued && err; w++) umma::mbar_wait(&tbar[w & 1], (uint32_t)((w >> 1) & 1), TC_WAIT);
    umma::fence_after_sync();
    bad = __syncthreads_or((int)err) != 0;
    // epilogue, one tile at a time through shared memory (the A buffers are free now)
    float *stg = reinterpret_cast<float *>(sm + L.A);
    float2 *part = reinterpret_cast<float2 *>(kp.Spart) + ((size_t)b * a.ngroups + grp) * kp.nk;
    for (int t = 0; t < nt && !bad; t++) {
        const int4 ti = stile[t];
        const int N = ti.y, J = ti.z, ld = N + 4;
        const int lq = warp & 3, half = warp >> 2, ncol = N / 2;
        for (int c0 = half * ncol; c0 < (half + 1) * ncol; c0 += 8) {
            float v[8];
            if (sub > 0) {
                umma::tmem_ld8(tm + ((uint32_t)(32 * lq) << 16) + (uint32_t)(ti.x + c0), v);
            } else {
#pragma unroll
                for (int j = 0; j < 8; j++) v[j] = 0.f;
            }
            float *row = stg + (32 * lq + lane) * ld + c0;
            *reinterpret_cast<float4 *>(row) = make_float4(v[0], v[1], v[2], v[3]);
            *reinterpret_cast<float4 *>(row + 4) = make_float4(v[4], v[5], v[6], v[7]);
        }
        __syncthreads();
        for (int i = tid; i < TC_RUNS * J; i += TC_NT) {
            const int q = i / J, j = i - q * J;
            const int r = a.run[ti.w + q];
            if (r < 0) continue;
            const KRun run = kp.runs[r];
            // (x, y) = (A.c_j, A.s_j) of the four components
            const float2 p0r = *reinterpret_cast<const float2 *>(stg + (0 * 32 + q) * ld + 2 * j);
            const float2 p0i = *reinterpret_cast<const float2 *>(stg + (1 * 32 + q) * ld + 2 * j);
            const float2 p1r = *reinterpret_cast<const float2 *>(stg + (2 * 32 + q) * ld + 2 * j);
            const float2 p1i = *reinterpret_cast<const float2 *>(stg + (3 * 32 + q) * ld + 2 * j);
            if (j >= run.kzlo && j < run.kzlo + run.nkz) {
                const int k = run.kbeg + j - run.kzlo;
                const float kz = kp.kzf[k];
                const float g0r = p0r.x - p0i.y, g0i = p0r.y + p0i.x;
                const float g1r = p1r.x - p1i.y, g1i = p1r.y + p1i.x;
                part[k] = make_float2(fmaf(kz, g1r, g0r), fmaf(kz, g1i, g0i));
            }
            if (j > 0 && -j >= run.kzlo && -j < run.kzlo + run.nkz) {
                const int k = run.kbeg - j - run.kzlo;
                const float kz = kp.kzf[k];
                const float g0r = p0r.x + p0i.y, g0i = p0i.x - p0r.y;
                const float g1r = p1r.x + p1i.y, g1i = p1i.x - p1r.y;
                part[k] = make_float2(fmaf(kz, g1r, g0r), fmaf(kz, g1i, g0i));
            }
        }
        __syncthreads();
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after_sync();
        umma::tmem_dealloc(tm, ncols);
        umma::tmem_relinquish();
    }
    if (err && tid == 0) atomicOr(kp.err, 8u);
}

// ---------------------------------------------------------------------------------------
// host side

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

void tc_init(Engine &E) {
    E.tc_ready = false;
    KP &kp = E.kp;
    if (E.precision != PIMD_MIXED || kp.ld <= kp.fd || !kp.tabf || !kp.dipf) return;
    // TMA rules: row pitch S x 8 bytes a multiple of 16, box rows <= 256
    if ((kp.S & 1) || kp.ntab > 256) return;
    int major = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, E.device);
    if (major != 10) return;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return;
    // runs sorted by their largest |kz| (longest first), 32 per M tile
    std::vector<int> order(kp.nrun), jr(kp.nrun);
    for (int r = 0; r < kp.nrun; r++) {
        const KRun &run = E.h_runs[r];
        const int lo = run.kzlo, hi = run.kzlo + run.nkz - 1;
        jr[r] = std::max(std::abs(lo), std::abs(hi)) + 1;
        order[r] = r;
    }
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return jr[x] > jr[y]; });
    const int T = (kp.nrun + TC_RUNS - 1) / TC_RUNS;
    std::vector<int4> tiles(T), groups;
    std::vector<int> slots((size_t)T * TC_RUNS, -1);
    int jmax = 1, nrows = 16;
    for (int t = 0; t < T; t++) {
        int J = 1;
        for (int q = 0; q < TC_RUNS && t * TC_RUNS + q < kp.nrun; q++) {
            const int r = order[t * TC_RUNS + q];
            slots[(size_t)t * TC_RUNS + q] = r;
            J = std::max(J, jr[r]);
        }
        const int N = ((2 * J + 15) / 16) * 16;
        if (N > 256) return;
        tiles[t] = make_int4(0, N, J, t * TC_RUNS);
        jmax = std::max(jmax, J);
        nrows = std::max(nrows, N);
    }
    // tile groups of <= 8 tiles whose TMEM columns fit in 512
    for (int t = 0; t < T;) {
        int cols = 0, n = 0;
        while (t + n < T && n < TC_TGMAX && cols + tiles[t + n].y <= 512) {
            tiles[t + n].x = cols;
            cols += tiles[t + n].y;
            n++;
        }
        if (n == 0) return;
        int pw = 32;
        while (pw < cols) pw *= 2;
        groups.push_back(make_int4(t, n, pw, 0));
        t += n;
    }
    if (jmax * TC_KS > TC_NT) return;
    const TcSmem L(kp.ntab, TC_TGMAX, nrows);
    if (L.total > 200 * 1024) return;
    // one limit for every context (the attribute belongs to the function, not the context)
    if (cudaFuncSetAttribute(k_sfac_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    int4 *d_tiles = nullptr, *d_groups = nullptr;
    int *d_slots = nullptr;
    if (cudaMalloc((void **)&d_tiles, sizeof(int4) * T) != cudaSuccess ||
        cudaMalloc((void **)&d_groups, sizeof(int4) * groups.size()) != cudaSuccess ||
        cudaMalloc((void **)&d_slots, sizeof(int) * slots.size()) != cudaSuccess) {
        cudaGetLastError();
        if (d_tiles) cudaFree(d_tiles);
        if (d_groups) cudaFree(d_groups);
        return;
    }
    E.allocs.push_back(d_tiles);
    E.allocs.push_back(d_groups);
    E.allocs.push_back(d_slots);
    cudaMemcpy(d_tiles, tiles.data(), sizeof(int4) * T, cudaMemcpyHostToDevice);
    cudaMemcpy(d_groups, groups.data(), sizeof(int4) * groups.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(d_slots, slots.data(), sizeof(int) * slots.size(), cudaMemcpyHostToDevice);
    // tables [P][ntab][S] float2 as a 2-D FP32 tensor (x = 2 S values, y = P ntab rows); a box
    // is 16 sites (128 bytes) x ntab rows, written to shared memory with the 128-byte swizzle
    CUtensorMap *map = reinterpret_cast<CUtensorMap *>(E.tc_map);
    const cuuint64_t dims[2] = {(cuuint64_t)2 * kp.S, (cuuint64_t)kp.P * kp.ntab};
    const cuuint64_t strides[1] = {(cuuint64_t)kp.S * 8};
    const cuuint32_t box[2] = {32, (cuuint32_t)kp.ntab};
    const cuuint32_t es[2] = {1, 1};
    if (enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, kp.tabf, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return;
    E.d_tctile = d_tiles;
    E.d_tcgrp = d_groups;
    E.d_tcrun = d_slots;
    E.tc_ntile = T;
    E.tc_ntg = (int)groups.size();
    E.tc_nrows = nrows;
    E.tc_jmax = jmax;
    E.tc_tgmax = TC_TGMAX;
    E.tc_ready = true;
}

int launch_sfac_tc(Engine &E, int s0, int nsites, int skipconv) {
    if (!E.tc_ready || !E.sf_tc || nsites <= 0) return 0;
    const KP &kp = E.kp;
    TcArgs a;
    a.tile = E.d_tctile;
    a.run = E.d_tcrun;
    a.grp = E.d_tcgrp;
    a.ntg = E.tc_ntg;
    a.sbase = s0 & ~(TC_SS - 1);  // TMA x coordinate 2 sbase: 256-byte aligned
    a.s_lo = s0;
    a.s_hi = s0 + nsites;
    a.nrows = E.tc_nrows;
    a.jmax = E.tc_jmax;
    a.skipconv = skipconv;
    // one CTA per SM (shared memory), one wave: site groups of whole 32-site stages
    const int nst = (a.s_hi - a.sbase + TC_SS - 1) / TC_SS;
    const long per = (long)E.tc_ntg * kp.P;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, E.device);
    int ng = (int)std::max(1L, (long)std::max(nsm, 1) / per);
    ng = std::max(1, std::min(ng, std::min(nst, E.sp_cap)));
    const int spg = (nst + ng - 1) / ng;
    a.tsg = spg * TC_SS;
    a.ngroups = (nst + spg - 1) / spg;
    const TcSmem L(kp.ntab, TC_TGMAX, a.nrows);
    dim3 g(E.tc_ntg * a.ngroups, kp.P);
    const CUtensorMap *map = reinterpret_cast<const CUtensorMap *>(E.tc_map);
    k_sfac_tc<<<g, TC_NT, L.total, E.stream>>>(*map, kp, a);
    ++E.nlaunch;
    return a.ngroups;
}

}  // namespace pimd
