// Tensor-core (tcgen05) dipole structure factor of the mixed engine:
//   S(k) = sum_s (k.mu_s) e^{i k.r_s}            (ewald.f90:99-108, the per-iteration ewald_std_dd sum)
// over the dipole sites of every bead, as GEMMs on FP16 hi + lo splits (hi.hi + hi.lo + lo.hi,
// ~22-bit operands) with FP32 accumulators in TMEM, followed by the sum over site groups and the
// FP32 field weights (k_sreduce's job) in the same launch.
//
// Formulation. For a run (kx, ky) with kz in [kzlo, kzlo + nkz) and a site s, e^{ik.r} =
// exy(s) ez(s, kz) with exy = ex(kx) ey(ky) (ewald.f90:30-31), and
//   S(kz) = kx Gx(kz) + ky Gy(kz) + kz Gz(kz),   Gc(kz) = sum_s mu_c(s) exy(s) ez(s, kz).
// With ez(-j) = conj ez(j) = c_j - i s_j, every Gc(+-j) follows from four real sums over s,
//   Re.c = sum Re(exy) mu_c c_j,  Re.s,  Im.c,  Im.s :
//   Gc(+j) = (Re.c - Im.s) + i (Re.s + Im.c),   Gc(-j) = (Re.c + Im.s) + i (Im.c - Re.s),
// so one real GEMM per bead gives every k-vector:
//   D[(c, j, cos|sin)][(run, Re|Im)] = sum_s Z[(c, j, cos|sin)][s] X[(run, Re|Im)][s],
//   Z = mu_c(s) (c_j(s) | s_j(s)),   X = Re|Im exy(s, run).
// The M side holds 6 (max |kz| + 1) <= 128 rows, the N side two columns per run (<= 256 runs,
// two MMAs of N <= 256 per K step). A tcgen05 MMA costs about the same for any N <= 256 on this
// part (measured: ~200 cycles for M = 128 and 32 bytes of K), so the wide, run-dependent operand
// goes on N, and kind::f16 (16 sites per 32 bytes of K) halves the MMAs per site of kind::tf32;
// each K step of 16 sites is three MMAs per N half. Z is scaled by 2^6 (exact) so that small
// mu_c ez values keep normal FP16 lo parts; the epilogue takes the scale out.
//
// A CTA owns one bead, one group of <= 256 runs and one group of consecutive sites; the site
// groups of a (bead, run group) form a thread-block cluster. Warp roles:
//   * producer warp: per 32-site stage, TMA (cp.async.bulk.tensor.2d, two boxes of 16 sites x all
//     ntab table rows, 128-byte swizzle) plus a bulk copy of the 32 FP32 dipoles, completing on an
//     mbarrier; it then turns the dipoles into scaled, masked per-component rows and releases the
//     stage to the builders;
//   * 16 builder warps: per 16 sites build X (exy of every run, one item per thread) and Z
//     (mu_c ez, on the threads without an X item) in the canonical no-swizzle K-major layout,
//     split into FP16 hi + lo, into one of three buffers;
//   * MMA warp: one thread issues the MMAs into TMEM and commits to the buffer's mbarrier, which
//     releases the buffer to the builders.
// Only mbarriers connect the roles, so building, copying and MMAs overlap. The epilogue reads
// TMEM (tcgen05.ld) 64 runs at a time, combines each k-vector's 12 sums, and keeps the CTA's FP32
// partial S in shared memory; after a cluster barrier each CTA adds the partials of all CTAs of
// its cluster over a slice of the k-vectors (distributed shared memory, FP32, site groups in a
// fixed order) and writes Sm and the FP32 weights Wf.
// Every mbarrier wait is bounded (~0.13 s); after a timeout a role stops, the CTA waits (bounded)
// for its copies and MMAs in flight, frees its TMEM, still meets its cluster barriers, and bit 8
// of the context's error word is set.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <algorithm>
#include <vector>

#include <cuda_fp16.h>

#include "dipole_check.cuh"
#include "engine.h"
#include "umma.cuh"

namespace pimd {

constexpr int TC_NB = 16;                 // builder warps
constexpr int TC_MMA_WARP = TC_NB;        // MMA-issuing warp (then the producer warp)
constexpr int TC_NT = (TC_NB + 2) * 32;   // 576 threads
constexpr int TC_SS = 32;                 // sites per table stage
constexpr int TC_KS = 16;                 // sites per MMA step (kind::f16: 32 bytes of K)
constexpr float TC_ZS = 64.f;             // power-of-two scale of Z (keeps small mu_c ez normal in FP16)
constexpr int TC_NABUF_MAX = 4;           // operand buffers (4: 708 -> 712 graph steps/s over 3)
constexpr int TC_NST = 4;                 // table stage buffers (a CTA's 128 sites at 512 x 32)
constexpr int TC_ZMAX = 4;                // Z items per builder thread (6 (|kz|max + 1) x 2 <= 256)
constexpr int TC_CLMAX = 8;               // site groups per cluster (portable cluster size)
constexpr int TC_MAXRUN = 256;            // runs per group: 512 TMEM columns
constexpr int TC_CH = 64;                 // runs per epilogue chunk
constexpr int TC_LD = 2 * TC_CH + 4;      // staging row pitch (floats)
constexpr long long TC_WAIT = 1LL << 28;  // cycles before a wait gives up (~0.13 s)

// structure-factor sums (values as in ewald.cu): charge q e, dipole (k.mu) e, dipole components mu_c e
enum { TC_OP_Q = 0, TC_OP_MU = 1, TC_OP_DIP = 2 };
// field passes (values as in ewald.cu): charge field and potential, dipole field + SOR update,
// and the two halves of the force pass ewald_std_qd: TF_QG the charge force and potential from
// the dipole structure factor, TF_DG the dipole force from the total (charge + dipole) one
enum { TF_Q = 0, TF_D = 1, TF_QG = 2, TF_DG = 3 };

// A run group: slots [p0, p0 + nr), MMA columns, the |kz| rows j0 .. j0 + jm - 1 of its Z
// operand (6 jm <= 128: |kz| above 20 goes to band groups, j0 = 21, of the same runs), k-vectors
// (local indices; those of a run outside the group's |kz| rows are entries with k = -1)
struct TcGroup {
    int p0, nr, ncol, jm, nkl, kgoff, j0, pad1;
};

// k-vector of a local index and its 4 pi Ak / V
struct TcKW {
    int k;
    float w;
};

struct TcArgs {
    const int4 *slot;     // per slot: kx + 256 (ky + 128), local k offset, kzlo, nkz
    const float2 *skv;    // per slot: FP32 (k_x, k_y)
    const TcGroup *grp;
    const TcKW *kw;       // k-vector and weight of each local index
    const float *kzv;     // k_z by kz + lmax
    int sbase;            // first site of site group 0 (multiple of 32, <= s_lo)
    int s_lo, s_hi;       // dipole sites [s_lo, s_hi)
    int tsg;              // sites per group (multiple of 32)
    int ncolmax;          // max MMA columns over run groups
    int nabuf;            // operand buffers
    int skipconv;
    uint4 *xcache;        // X operand blocks of the dipole sites (null: no cache), see k_sfac_tc
    int xsub, xblock;     // 16-site blocks per bead and run group, bytes per block
    int xkeep;            // load the cached X blocks with the L2 evict-last policy
    int pdl;              // launched as a programmatic dependent of the previous iteration's field pass
};

// Shared-memory carve-up (bytes from a 1024-aligned base), used by the kernel and the launcher.
// A table stage holds two TMA boxes of 16 sites x ntab rows, each written with the 128-byte
// swizzle (16-byte chunk c of row r lands at chunk c ^ (r & 7), so loads of the same sites from
// different rows fall in different banks), followed by the stage's 32 dipoles (as copied, then
// as 3 rows of 2^6 mu_c with the sites outside the group zeroed). An operand
// buffer holds Z hi, Z lo (128 rows x 16 FP16 sites each) and X hi, X lo (ncolmax rows x 16 sites).
struct TcSmem {
    int boxb, mu, muz, stage, buf, xoff, bufstride, total;
    __host__ __device__ TcSmem(int ntab, int ncolmax, int nabuf) {
        boxb = ((ntab * 128 + 1023) / 1024) * 1024;
        mu = 2 * boxb;
        muz = mu + TC_SS * 16;
        stage = ((muz + 3 * TC_SS * 4 + 1023) / 1024) * 1024;
        buf = TC_NST * stage;
        xoff = 2 * 128 * 32;
        bufstride = xoff + 2 * ncolmax * 32;
        total = buf + nabuf * bufstride + 1024;  // + alignment slack of the dynamic base
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
// contiguous global -> shared copy (addresses 16-byte aligned, bytes a multiple of 16)
PIMD_D void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     umma::smem_u32(dst)),
                 "l"((unsigned long long)src), "r"(bytes), "r"(umma::smem_u32(bar))
                 : "memory");
}
// the same with an L2 eviction policy: evict-first (data read once per kernel that should not
// displace the working set of the other kernels) or, with keep, evict-last (data read again by
// every dipole iteration of the force call, kept in L2 across them)
PIMD_D void bulk_load_stream(void *dst, const void *src, uint32_t bytes, uint64_t *bar, bool keep = false) {
    uint64_t pol;
    if (keep)
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    else
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
                     umma::smem_u32(dst)),
                 "l"((unsigned long long)src), "r"(bytes), "r"(umma::smem_u32(bar)), "l"(pol)
                 : "memory");
}
// programmatic dependent launch: the next kernel of the stream may start (its CTAs wait with
// pdl_wait before they read what this grid writes); pdl_wait returns once the previous grid
// has completed and its writes are visible (a no-op without the launch attribute)
PIMD_D void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
PIMD_D void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
PIMD_D void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(umma::smem_u32(bar)), "r"(bytes) : "memory");
}
PIMD_D void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_u32(bar)) : "memory");
}
PIMD_D void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
PIMD_D uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
PIMD_D float2 ld_cluster_f2(uint32_t local_addr, uint32_t rank) {
    uint32_t ra;
    float2 v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(local_addr), "r"(rank));
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(ra));
    return v;
}
// Eight FP32 values as FP16 hi + lo (x = hi + lo to ~22 bits): two 16-byte rows of 8 halves
PIMD_D void split8_h(const float (&x)[8], uint4 &hi, uint4 &lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const __half2 hh = __floats2half2_rn(x[2 * i], x[2 * i + 1]);
        const float2 hf = __half22float2(hh);
        const __half2 ll = __floats2half2_rn(x[2 * i] - hf.x, x[2 * i + 1] - hf.y);
        h[i] = *reinterpret_cast<const uint32_t *>(&hh);
        l[i] = *reinterpret_cast<const uint32_t *>(&ll);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}
// byte offset of the 16-byte chunk c (sites 8 c .. 8 c + 7) of row n in a K-major operand of 16
// FP16 sites (two core matrices along K)
PIMD_D int rowchunk(int n, int c) { return (((n >> 3) * 2 + c) << 7) + ((n & 7) << 4); }

// 64 registers a thread (a few bytes spill): one CTA of 576 threads then leaves 28 K registers
// of the SM to the real-space dipole field running beside it on the second stream (4 blocks
// instead of 1 at 95 registers); the graph step at 512 x 32 measured 677 -> 702 steps/s
// (72 registers: 695, 56: 697, 48: 680)
template <int OP>
__global__ void __maxnreg__(64) k_sfac_tc(const __grid_constant__ CUtensorMap tmap, KP kp, TcArgs a) {
    // Z components: q (charges) or mu_x, mu_y, mu_z; partial sums per k: S, or the three G_c
    constexpr int NCZ = (OP == TC_OP_Q) ? 1 : 3;
    constexpr int NPT = (OP == TC_OP_DIP) ? 3 : 1;
    const int grp = blockIdx.x, tg = blockIdx.y, b = blockIdx.z;
    // a programmatic launch starts under the previous field pass: the convergence flags, the
    // dipoles and the weights are that grid's output
    if (a.pdl) pdl_wait();
    // the whole cluster (same bead) leaves together
    if (a.skipconv && bead_converged(kp, b)) return;
    const TcGroup G = a.grp[tg];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const TcSmem L(kp.ntab, a.ncolmax, a.nabuf);
    extern __shared__ __align__(1024) unsigned char sm_raw[];
    // the swizzle pattern follows shared-memory address bits 7-9: align the base to 1024 bytes
    unsigned char *sm = sm_raw + ((1024u - (umma::smem_u32(sm_raw) & 1023u)) & 1023u);
    __shared__ uint64_t tfull[TC_NST], mfull[TC_NST], tempty[TC_NST], afull[TC_NABUF_MAX], aempty[TC_NABUF_MAX];
    __shared__ uint64_t xfull[TC_NABUF_MAX];  // a cached X block has landed in the buffer
    __shared__ uint32_t tslot;
    __shared__ int4 sslot[TC_MAXRUN];
    __shared__ float2 sskv[TC_MAXRUN];
    __shared__ float skz[256];

    const int g0 = a.sbase + grp * a.tsg;
    const int g1 = min(a.s_hi, g0 + a.tsg);
    const int nstage = max(0, (g1 - g0 + TC_SS - 1) / TC_SS);
    const int nsub = nstage * (TC_SS / TC_KS);
    const int yrow = kp.hmax + 1;            // first ey row (ky = 0); ez rows follow the ky rows
    const int nab = a.nabuf, jm = G.jm, nr = G.nr;
    const int xlo = a.ncolmax * 32;          // X lo after X hi
    // X = exy(site, run) depends on the positions only, so the dipole structure factor of the
    // iterations builds it once per force call: the first iteration (no iteration done yet)
    // builds and stores it (xm 1), later ones load it by bulk copies (xm 2) and build only Z.
    // A block holds the X rows [0, 2 nr) rounded to 8-row groups, hi then lo, in the operand
    // layout; the cache is zeroed once, so the rows past 2 nr stay zero.
    const int xm = (OP == TC_OP_MU && a.xcache) ? (kp.dstep[1] == 0 ? 1 : 2) : 0;
    const int xbytes = ((2 * nr + 7) / 8) * 256;
    uint4 *xc = xm ? a.xcache + ((size_t)(b * gridDim.y + tg) * a.xsub + (g0 - a.sbase) / TC_KS) * (a.xblock / 16)
                   : nullptr;

    if (tid < nr) {
        sslot[tid] = a.slot[G.p0 + tid];
        sskv[tid] = a.skv[G.p0 + tid];
    }
    if (tid < 2 * kp.lmax + 1) skz[tid] = a.kzv[tid];
    if (warp == 0) umma::tmem_alloc(&tslot, 512);
    // table stage ts of this group: TMA boxes of the tables and a bulk copy of the dipoles
    const uint32_t box_tx = (uint32_t)(kp.ntab * 128);
    auto issue_stage = [&](int ts) {
        const int sfirst = g0 + ts * TC_SS, tb = ts % TC_NST;
        unsigned char *dst = sm + tb * L.stage;
        const int nmu = min(TC_SS, kp.S - sfirst);  // dipoles inside this bead's rows
        const uint32_t mub = (uint32_t)nmu * 16u;
        mbar_expect_tx(&tfull[tb], 2 * box_tx + mub);
        tma_load_2d(dst, &tmap, 2 * sfirst, b * kp.ntab, &tfull[tb]);
        tma_load_2d(dst + L.boxb, &tmap, 2 * sfirst + 32, b * kp.ntab, &tfull[tb]);
        const float4 *wsrc = (OP == TC_OP_Q) ? kp.posf : dipf_cur(kp);  // (offset, q) or (mu, 0)
        bulk_load(dst + L.mu, wsrc + (size_t)b * kp.S + sfirst, mub, &tfull[tb]);
    };
    if (tid == 0) {
        for (int i = 0; i < TC_NST; i++) {
            umma::mbar_init(&tfull[i], 1);
            umma::mbar_init(&mfull[i], 1);
            umma::mbar_init(&tempty[i], TC_NB);
        }
        for (int i = 0; i < nab; i++) {
            umma::mbar_init(&afull[i], TC_NB);
            umma::mbar_init(&aempty[i], 1);
            umma::mbar_init(&xfull[i], 1);
        }
        // the first stages go out now, under the rest of the set-up
        for (int ts = 0; ts < min(nstage, TC_NST); ts++) issue_stage(ts);
    }
    {   // padding stays zero in every buffer (hi and lo): Z rows >= 6 jm, X rows >= 2 nr
        const int zp = 128 - 2 * NCZ * jm, xp = G.ncol - 2 * nr;
        for (int i = tid; i < nab * 2 * (zp + xp) * 2; i += TC_NT) {
            const int q = i & 1, rr = i >> 1;
            const int row = rr % (zp + xp), hl = (rr / (zp + xp)) & 1, bi = rr / (2 * (zp + xp));
            unsigned char *B0 = sm + L.buf + bi * L.bufstride;
            unsigned char *dst = row < zp ? B0 + hl * 128 * 32 + rowchunk(2 * NCZ * jm + row, q)
                                          : B0 + L.xoff + hl * a.ncolmax * 32 + rowchunk(2 * nr + row - zp, q);
            *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    // the iteration's field pass may start its set-up (tables, Q) on the SMs this grid leaves free
    pdl_launch_dependents();
    const uint32_t tm = tslot;
    uint32_t err = 0;

    if (warp < TC_NB) {
        // ---------------- builders: X = exy of every run (8 sites per item), Z = mu_c ez
        const int bt = tid;  // 0 .. 32 TC_NB - 1
        int it_n = 0, it_off[2], it_xr[2], it_yr[2], it_o[2];
        float it_ys[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int it = bt + u * 32 * TC_NB;
            it_off[u] = it_xr[u] = it_yr[u] = it_o[u] = 0;
            it_ys[u] = 1.f;
            if (it >= 2 * nr || xm == 2) continue;
            it_n = u + 1;
            const int p = it >> 1, o = it & 1;
            const int kxy = sslot[p].x, kx = kxy & 255, ky = (kxy >> 8) - 128;
            it_off[u] = rowchunk(2 * p, o);  // Re row; the Im row 2 p + 1 is 16 bytes further
            it_o[u] = o;
            it_xr[u] = kx;
            it_yr[u] = yrow + (ky < 0 ? -ky : ky);
            it_ys[u] = ky < 0 ? -1.f : 1.f;
        }
        // Z items: one row (c, j, cos|sin) x 8 sites each, on the whole warps after the X items
        // (else on the last warp), at most TC_ZMAX per thread; row decoded once here
        const int nzi = 2 * NCZ * jm * 2;
        const int zwarps = xm == 2 ? TC_NB : max(1, TC_NB - (2 * nr + 31) / 32);
        const int zthreads = 32 * zwarps, zbase = 32 * TC_NB - zthreads;
        int zn = 0, zoff[TC_ZMAX], zmo[TC_ZMAX], zer[TC_ZMAX], zcs[TC_ZMAX], zq[TC_ZMAX];
#pragma unroll
        for (int u = 0; u < TC_ZMAX; u++) {
            const int zi = bt - zbase + u * zthreads;
            zoff[u] = zmo[u] = zer[u] = zcs[u] = zq[u] = 0;
            if (bt < zbase || zi >= nzi) continue;
            zn = u + 1;
            const int zr = zi >> 1, c = zr / (2 * jm);
            zoff[u] = rowchunk(zr, zi & 1);
            zmo[u] = c * TC_SS + 8 * (zi & 1);         // component row of muz, first site
            zer[u] = yrow + kp.kmax + 1 + G.j0 + ((zr >> 1) % jm);  // ez row of |kz| = j0 + j
            zcs[u] = zr & 1;
            zq[u] = 8 * (zi & 1);
        }
        for (int ts = 0; ts < nstage && !err; ts++) {
            const int tb = ts % TC_NST;
            err |= (uint32_t)umma::mbar_wait(&mfull[tb], (uint32_t)((ts / TC_NST) & 1), TC_WAIT);
            const unsigned char *tab = sm + tb * L.stage;
            const float *muz = reinterpret_cast<const float *>(tab + L.muz);
            for (int ks = 0; ks < TC_SS / TC_KS && !err; ks++) {
                const int sub = ts * (TC_SS / TC_KS) + ks, ab = sub % nab, use = sub / nab;
                if (use > 0) err |= (uint32_t)umma::mbar_wait(&aempty[ab], (uint32_t)((use - 1) & 1), TC_WAIT);
                unsigned char *Bf = sm + L.buf + ab * L.bufstride;
                const int so = ks * TC_KS;
                uint4 *xb = xm ? xc + (size_t)sub * (a.xblock / 16) : nullptr;  // this block in the cache
                if (xm == 2 && bt == 0) {
                    mbar_expect_tx(&xfull[ab], 2u * (uint32_t)xbytes);
                    bulk_load_stream(Bf + L.xoff, xb, (uint32_t)xbytes, &xfull[ab], a.xkeep);
                    bulk_load_stream(Bf + L.xoff + xlo, xb + xbytes / 16, (uint32_t)xbytes, &xfull[ab], a.xkeep);
                }
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    if (u >= it_n) break;
                    const int sq = so + 8 * it_o[u];
                    const float ys = it_ys[u];
                    float re[8], im[8];
#pragma unroll
                    for (int h = 0; h < 4; h++) {
                        const float4 xx = *tab_chunk(tab, L.boxb, it_xr[u], sq + 2 * h);
                        const float4 yy = *tab_chunk(tab, L.boxb, it_yr[u], sq + 2 * h);
                        // ewald.f90:30-31: coskxky = cx cy - sx sy, sinkxky = sx cy + cx sy
                        re[2 * h] = xx.x * yy.x - xx.y * (ys * yy.y);
                        im[2 * h] = xx.y * yy.x + xx.x * (ys * yy.y);
                        re[2 * h + 1] = xx.z * yy.z - xx.w * (ys * yy.w);
                        im[2 * h + 1] = xx.w * yy.z + xx.z * (ys * yy.w);
                    }
                    uint4 rh, rl, ih, il;
                    split8_h(re, rh, rl);
                    split8_h(im, ih, il);
                    unsigned char *xp = Bf + L.xoff + it_off[u];
                    *reinterpret_cast<uint4 *>(xp) = rh;
                    *reinterpret_cast<uint4 *>(xp + 16) = ih;
                    *reinterpret_cast<uint4 *>(xp + xlo) = rl;
                    *reinterpret_cast<uint4 *>(xp + xlo + 16) = il;
                    if (xm == 1) {
                        uint4 *g = xb + it_off[u] / 16;
                        g[0] = rh;
                        g[1] = ih;
                        g[xbytes / 16] = rl;
                        g[xbytes / 16 + 1] = il;
                    }
                }
#pragma unroll
                for (int u = 0; u < TC_ZMAX; u++) {
                    if (u >= zn) break;
                    const int sq = so + zq[u];
                    const float4 m0 = *reinterpret_cast<const float4 *>(muz + zmo[u] + so);
                    const float4 m1 = *reinterpret_cast<const float4 *>(muz + zmo[u] + so + 4);
                    const float mc[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
                    float v[8];
#pragma unroll
                    for (int h = 0; h < 4; h++) {
                        const float4 zz = *tab_chunk(tab, L.boxb, zer[u], sq + 2 * h);
                        v[2 * h] = mc[2 * h] * (zcs[u] ? zz.y : zz.x);
                        v[2 * h + 1] = mc[2 * h + 1] * (zcs[u] ? zz.w : zz.z);
                    }
                    uint4 hi, lo;
                    split8_h(v, hi, lo);
                    *reinterpret_cast<uint4 *>(Bf + zoff[u]) = hi;
                    *reinterpret_cast<uint4 *>(Bf + 128 * 32 + zoff[u]) = lo;
                }
                umma::fence_smem_to_async();
                __syncwarp();
                if (lane == 0) mbar_arrive(&afull[ab]);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[tb]);
        }
    } else if (warp == TC_MMA_WARP) {
        // ---------------- MMA issue (one thread): D[128][ncol] += Z X^T, two N halves
        if (lane == 0) {
            const uint32_t idesc_base = umma::idesc_f16(128, 16) & ~(0x3Fu << 17);
            for (int sub = 0; sub < nsub && !err; sub++) {
                const int ab = sub % nab, use = sub / nab;
                err |= (uint32_t)umma::mbar_wait(&afull[ab], (uint32_t)(use & 1), TC_WAIT);
                if (xm == 2) err |= (uint32_t)umma::mbar_wait(&xfull[ab], (uint32_t)(use & 1), TC_WAIT);
                if (err) break;
                umma::fence_after_sync();
                const uint32_t zH = umma::smem_u32(sm + L.buf + ab * L.bufstride), zL = zH + 128 * 32;
                const uint32_t xH = zH + L.xoff, xL = xH + xlo;
                const uint64_t dz_h = umma::sdesc(zH, 128, 256), dz_l = umma::sdesc(zL, 128, 256);
                for (int nt = 0; nt * 256 < G.ncol; nt++) {
                    const int N = min(256, G.ncol - nt * 256);
                    const uint32_t id = idesc_base | ((uint32_t)(N >> 3) << 17);
                    const uint32_t d = tm + (uint32_t)(nt * 256);
                    // rows 256 nt.. of X: 32 row groups of 256 bytes per half
                    const uint64_t dx_h = umma::sdesc(xH + nt * 8192, 128, 256), dx_l = umma::sdesc(xL + nt * 8192, 128, 256);
                    umma::mma_f16(d, dz_h, dx_h, id, sub > 0);
                    umma::mma_f16(d, dz_h, dx_l, id, 1);
                    umma::mma_f16(d, dz_l, dx_h, id, 1);
                }
                umma::commit(&aempty[ab]);
            }
        }
    } else {
        // ---------------- producer: as each table stage lands, the dipoles as 3 component rows
        // (2^6 mu_c, zero outside [s_lo, g1)) for the builders; stages beyond the first TC_NST are
        // copied into a buffer once all builder warps are done with its previous stage
        int issued = min(nstage, TC_NST), landed = 0;
        for (int ts = 0; ts < nstage && !err; ts++) {
            const int tb = ts % TC_NST;
            err |= (uint32_t)umma::mbar_wait(&tfull[tb], (uint32_t)((ts / TC_NST) & 1), TC_WAIT);
            if (err) break;
            landed = ts + 1;
            unsigned char *dst = sm + tb * L.stage;
            {
                const int s = g0 + ts * TC_SS + lane;
                const float4 m = reinterpret_cast<const float4 *>(dst + L.mu)[lane];
                const bool in = s >= a.s_lo && s < g1;
                float *muz = reinterpret_cast<float *>(dst + L.muz);
                if (OP == TC_OP_Q) {
                    muz[lane] = in ? TC_ZS * m.w : 0.f;
                } else {
                    muz[lane] = in ? TC_ZS * m.x : 0.f;
                    muz[TC_SS + lane] = in ? TC_ZS * m.y : 0.f;
                    muz[2 * TC_SS + lane] = in ? TC_ZS * m.z : 0.f;
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&mfull[tb]);
            const int tr = ts + TC_NST - 1;  // refill the buffer of stage ts - 1
            if (ts >= 1 && tr < nstage) {
                err |= (uint32_t)umma::mbar_wait(&tempty[tr % TC_NST], (uint32_t)(((ts - 1) / TC_NST) & 1), TC_WAIT);
                if (err) break;
                if (lane == 0) issue_stage(tr);
                issued = tr + 1;
                __syncwarp();
            }
        }
        // copies still in flight after a timeout land before the CTA leaves
        for (int w = landed; w < issued && err; w++)
            umma::mbar_wait(&tfull[w % TC_NST], (uint32_t)((w / TC_NST) & 1), TC_WAIT);
    }

    // ---------------- all MMAs done: the last commit tracks every earlier MMA of the issuing thread
    if (nsub > 0) {
        const int last = nsub - 1;
        int to = umma::mbar_wait(&aempty[last % nab], (uint32_t)((last / nab) & 1), TC_WAIT);
        if (to) to = umma::mbar_wait(&aempty[last % nab], (uint32_t)((last / nab) & 1), TC_WAIT);
        err |= (uint32_t)to;
    }
    umma::fence_after_sync();
    const bool bad = __syncthreads_or((int)err) != 0;

    // this CTA's slice of the cluster reduction; its (k, w) pairs are fetched now, under the epilogue
    const int cr = (int)cluster_rank(), cn = gridDim.x;
    const int i0 = (int)((long)cr * G.nkl / cn), i1 = (int)((long)(cr + 1) * G.nkl / cn);
    constexpr int TC_PF = 4;
    TcKW pf[TC_PF];
#pragma unroll
    for (int u = 0; u < TC_PF; u++) {
        const int i = i0 + tid + u * TC_NT;
        pf[u] = i < i1 ? a.kw[G.kgoff + i] : TcKW{0, 0.f};
    }
    // epilogue: TMEM -> shared, 64 runs (128 columns) at a time -> partial S of every k of the group
    float *stg = reinterpret_cast<float *>(sm);                       // [128][TC_LD]
    float2 *pt = reinterpret_cast<float2 *>(sm + 128 * TC_LD * 4);    // [nkl]
    for (int ch = 0; ch * TC_CH < nr && !bad; ch++) {
        if (warp < 16) {
            const int lq = warp & 3, part = warp >> 2;  // 4 lane quarters x 4 column quarters
            const int c0 = ch * 2 * TC_CH + 32 * part;
            float v[8];
            float *row = stg + (32 * lq + lane) * TC_LD + 32 * part;
#pragma unroll
            for (int hh = 0; hh < 4; hh++) {
                if (nsub > 0) {
                    umma::tmem_ld8(tm + ((uint32_t)(32 * lq) << 16) + (uint32_t)(c0 + 8 * hh), v);
                } else {
#pragma unroll
                    for (int j = 0; j < 8; j++) v[j] = 0.f;
                }
                *reinterpret_cast<float4 *>(row + 8 * hh) = make_float4(v[0], v[1], v[2], v[3]);
                *reinterpret_cast<float4 *>(row + 8 * hh + 4) = make_float4(v[4], v[5], v[6], v[7]);
            }
        }
        __syncthreads();
        for (int i = tid; i < TC_CH * jm; i += TC_NT) {
            const int q = i % TC_CH, jj = i / TC_CH, p = ch * TC_CH + q, j = G.j0 + jj;  // row jj: |kz| = j
            if (p >= nr) continue;
            const int4 sl = sslot[p];  // run, local offset, kzlo, nkz
            const bool plus = j >= sl.z && j < sl.z + sl.w;
            const bool minus = j > 0 && -j >= sl.z && -j < sl.z + sl.w;
            if (!plus && !minus) continue;
            float2 gp[NCZ], gm[NCZ];
#pragma unroll
            for (int c = 0; c < NCZ; c++) {
                const int rc = (c * jm + jj) * 2;
                // (x, y) = (Re exy, Im exy) against mu_c c_j (row rc) and mu_c s_j (row rc + 1)
                const float2 dc = *reinterpret_cast<const float2 *>(stg + rc * TC_LD + 2 * q);
                const float2 ds = *reinterpret_cast<const float2 *>(stg + (rc + 1) * TC_LD + 2 * q);
                gp[c] = make_float2(dc.x - ds.y, ds.x + dc.y);
                gm[c] = make_float2(dc.x + ds.y, dc.y - ds.x);
            }
            const float zs = 1.f / TC_ZS;
            if (OP == TC_OP_MU) {
                const float2 kv = make_float2(sskv[p].x * zs, sskv[p].y * zs);
                if (plus) {
                    const float kz = skz[kp.lmax + j] * zs;
                    pt[sl.y + j - sl.z] = make_float2(fmaf(kz, gp[NCZ - 1].x, fmaf(kv.y, gp[1 % NCZ].x, kv.x * gp[0].x)),
                                                      fmaf(kz, gp[NCZ - 1].y, fmaf(kv.y, gp[1 % NCZ].y, kv.x * gp[0].y)));
                }
                if (minus) {
                    const float kz = skz[kp.lmax - j] * zs;
                    pt[sl.y - j - sl.z] = make_float2(fmaf(kz, gm[NCZ - 1].x, fmaf(kv.y, gm[1 % NCZ].x, kv.x * gm[0].x)),
                                                      fmaf(kz, gm[NCZ - 1].y, fmaf(kv.y, gm[1 % NCZ].y, kv.x * gm[0].y)));
                }
            } else {
                // charges: S itself; dipole components: the three G_c
#pragma unroll
                for (int c = 0; c < NPT; c++) {
                    if (plus) pt[NPT * (sl.y + j - sl.z) + c] = make_float2(zs * gp[c].x, zs * gp[c].y);
                    if (minus) pt[NPT * (sl.y - j - sl.z) + c] = make_float2(zs * gm[c].x, zs * gm[c].y);
                }
            }
        }
        __syncthreads();
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after_sync();
        umma::tmem_dealloc(tm, 512);
        umma::tmem_relinquish();
    }
    // cluster: add the partials of all site groups over this CTA's slice of the k-vectors
    // (groups in order), then Sm = (-Im, Re) and the FP32 weights 4 pi Ak / V conj(S)
    cluster_sync();
    if (!bad) {
        const uint32_t pbase = umma::smem_u32(pt);
        auto reduce_one = [&](int i, const TcKW &kw) {
            if (kw.k < 0) return;  // a k-vector of the run that another (band) group sums
#pragma unroll
            for (int e = 0; e < NPT; e++) {
                float2 v[TC_CLMAX];
#pragma unroll
                for (int c = 0; c < TC_CLMAX; c++)
                    if (c < cn) v[c] = ld_cluster_f2(pbase + 8u * (uint32_t)(NPT * i + e), (uint32_t)c);
                // FP32 in a fixed order: FP64 arithmetic is slow on this part, and the partials
                // carry only the split operands' ~2^-21 anyway
                float sx = 0.f, sy = 0.f;
#pragma unroll
                for (int c = 0; c < TC_CLMAX; c++)
                    if (c < cn) {
                        sx += v[c].x;
                        sy += v[c].y;
                    }
                if (OP == TC_OP_MU) {  // (-Im, Re) as the reference's rQm, iQm (ewald.f90:106-107)
                    kp.Sm[(size_t)b * kp.nk + kw.k] = make_double2(-(double)sy, (double)sx);
                    kp.Wf[((size_t)b * 2 + 1) * kp.nk + kw.k] = make_float2(-kw.w * sy, -kw.w * sx);
                } else if (OP == TC_OP_Q) {
                    kp.Sq[(size_t)b * kp.nk + kw.k] = make_double2((double)sx, (double)sy);
                    kp.Wf[((size_t)b * 2) * kp.nk + kw.k] = make_float2(kw.w * sx, -kw.w * sy);
                } else {
                    kp.Sdip[((size_t)b * kp.nk + kw.k) * 3 + e] = make_double2((double)sx, (double)sy);
                }
            }
        };
#pragma unroll
        for (int u = 0; u < TC_PF; u++) {
            const int i = i0 + tid + u * TC_NT;
            if (i < i1) reduce_one(i, pf[u]);
        }
        for (int i = i0 + tid + TC_PF * TC_NT; i < i1; i += TC_NT) reduce_one(i, a.kw[G.kgoff + i]);
    }
    cluster_sync();  // remote reads done before any CTA of the cluster leaves
    if (bad && tid == 0) atomicOr(kp.err, 8u);
}

// ---------------------------------------------------------------------------------------
// Tensor-core dipole field of the mixed engine (the per-iteration k_field_f<F_D> sum,
// ewald.f90:114-117): at every dipole site s of a bead,
//   E_x,y(s) = sum_run k_x,y Im(exy(s) T0(s)),   E_z(s) = sum_run Im(exy(s) T1(s)),
//   T0(s) = sum_kz W(kz) ez(s, kz),   T1(s) = sum_kz k_z W(kz) ez(s, kz),
// with W the FP32 weights 4 pi Ak / V conj(S) of the run's k-vectors. Folding +-j as in the
// structure factor (W+ = W(+j), W- = W(-j), Wp = W+ + W-, Wm = W+ - W-):
//   T0 = sum_j (Wp.x c_j - Wm.y s_j) + i (Wp.y c_j + Wm.x s_j)
//   T1 = sum_j k_z(j) [(Wm.x c_j - Wp.y s_j) + i (Wm.y c_j + Wp.x s_j)]
// so T0, T1 of every run at every site are one GEMM per bead,
//   D[s][(run, comp)] = sum_q Q[s][q] V[(run, comp)][q],  comp = T0re|T0im|T1re|T1im,  q = (j, cos|sin),
// with the sites on M (128 per CTA), runs x components on N (two passes of half the runs, each
// component-major in <= 512 TMEM columns) and only 2 (max |kz| + 1) terms on K (FP16 hi + lo
// split, three MMAs per 16-term K step). V is built by every CTA of a bead from
// the bead's weights Wf (one bulk copy into shared memory; scaled by 2^10, exact, to keep small
// weights normal in FP16). The epilogue contracts each TMEM row with exy(s, run) from the
// TMA-staged tables (16 warps = 4 lane quarters x 4 run quarters, 16 runs x 4 components per
// TMEM wait), then applies the iteration's
// FP64 SOR update at the CTA's dipole sites and the convergence test in the last CTA
// (dipole_check.cuh, as k_field_finish<F_D> does).
constexpr int TF_NT = 512;
constexpr int TF_SITES = 128;             // sites per CTA (M)
constexpr float TF_WS = 1024.f;           // power-of-two scale of V

struct TfArgs {
    const int4 *slot;     // per run slot: packed kx/ky, local k offset, kzlo, nkz
    const float2 *skv;    // per run slot: FP32 (k_x, k_y)
    const int2 *kpm;      // per (slot, j): k-vector of kz = +j and of kz = -j (-1: none)
    const float *kzv;     // k_z by kz + lmax
    int nr, nph, ncol, kq, jm;  // runs, runs per pass (rounded up to 8), V rows (8 nph), K terms (x16), kz rows
    int sbase, s_lo, s_hi;
    int pdl;  // launched as a programmatic dependent of the structure factor (pdl_wait before W)
    int vpp;    // more than two passes: V of each pass built before it (4 nph rows), as TF_DG does
    int wglob;  // the bead's weights read from global memory (too many k-vectors for shared memory)
};

struct TfSmem {
    int boxb, A, B, W, total;
    __host__ __device__ TfSmem(int ntab, int ncol, int kq, int nk, int nslot = 1) {
        boxb = ((ntab * 128 + 1023) / 1024) * 1024;
        A = 8 * boxb;                      // tables of 128 sites: 8 TMA boxes of 16 sites
        B = A + 2 * TF_SITES * kq * 2;     // Q hi, lo: 128 rows x kq halves
        W = B + 2 * ncol * kq * 2;         // V hi, lo: ncol rows x kq halves
        total = W + ((nslot * nk * 8 + 127) / 128) * 128 + 1024;  // the bead's weights Wf (1 or 2 slots)
    }
};

// byte offset of the 16-byte chunk jc (halves 8 jc .. 8 jc + 7) of row n in a K-major operand
// with kcm core matrices along K
PIMD_D int rowchunk_k(int n, int jc, int kcm) { return (((n >> 3) * kcm + jc) << 7) + ((n & 7) << 4); }

// VPP: V built before each pass (more than two passes); a template argument so that the
// two-pass form keeps its registers (118 against 127 with a run-time choice)
template <int MODE, bool VPP>
__global__ void __launch_bounds__(TF_NT, 1) k_field_tc(const __grid_constant__ CUtensorMap tmap, KP kp, TfArgs a) {
    // TF_DG: 6 components per run (T0, T1 and T2 = sum kz^2 W ez, complex), V rebuilt for each
    // pass of nph runs; the other modes: 4 components, V of both passes built once (or, with
    // a.vpp, V of each pass before it, for more than two passes)
    constexpr bool DG = MODE == TF_DG;
    constexpr int NC = DG ? 6 : 4;
    constexpr bool vpp = DG || VPP;
    const int t = blockIdx.x, b = blockIdx.y;
    // the next iteration's structure factor may be scheduled now; it waits for this grid
    if (MODE == TF_D) pdl_launch_dependents();
    if (MODE == TF_D && bead_converged(kp, b)) {
        // converged bead: no update, but the block still counts towards the convergence test
        const double zero[2] = {0.0, 0.0};
        if (kp.dd_async) {  // (a unit's arrivals still complete it)
            const float z[3] = {0.f, 0.f, 0.f};
            if (dd_unit_arrive(kp, b, t)) dd_unit_sor<TF_NT>(kp, b, t, false, z);
            return;
        }
        dd_block_end<TF_NT>(kp, b, zero, false);
        return;
    }
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const TfSmem L(kp.ntab, a.ncol, a.kq, kp.nk, a.wglob ? 0 : (DG ? 2 : 1));
    extern __shared__ __align__(1024) unsigned char sm_raw[];
    unsigned char *sm = sm_raw + ((1024u - (umma::smem_u32(sm_raw) & 1023u)) & 1023u);
    __shared__ uint64_t tbar, wbar, mbar;
    __shared__ uint32_t tslot;
    // per run of the current pass: byte offsets of the ex and ey table rows in a stage and their
    // swizzle keys (16 x (row & 7)); bit 0 of the ey key: ky < 0 (conjugate ey)
    __shared__ int4 sroff[TC_MAXRUN];
    __shared__ float2 sskv[TC_MAXRUN];
    const int sb = a.sbase + t * TF_SITES;
    // the copies go out first: the bead's weights (one bulk copy) and the tables of 128 sites
    if (tid == 0) {
        umma::mbar_init(&tbar, 1);
        umma::mbar_init(&wbar, 1);
        umma::mbar_init(&mbar, 1);
        // weight slots: charge (0), dipole (1); TF_DG takes both (adjacent in Wf)
        if (!a.pdl && !a.wglob) {
            const int slot = (MODE == TF_D || MODE == TF_QG) ? 1 : 0;
            const uint32_t wbytes = (uint32_t)kp.nk * 8u * (DG ? 2u : 1u);
            mbar_expect_tx(&wbar, wbytes);
            bulk_load(sm + L.W, kp.Wf + ((size_t)b * 2 + slot) * kp.nk, wbytes, &wbar);
        }
        const uint32_t box_tx = (uint32_t)(kp.ntab * 128);
        mbar_expect_tx(&tbar, 8 * box_tx);
        for (int i = 0; i < 8; i++) tma_load_2d(sm + i * L.boxb, &tmap, 2 * (sb + 16 * i), b * kp.ntab, &tbar);
    }
    const int iter = kp.dstep[1] + 1;  // dipole iteration of this update
    const int kcm = a.kq / 8, nr = a.nr, nph = a.nph, jm = a.jm;
    const int npass = vpp ? (nr + nph - 1) / nph : 2;
    const int yrow = kp.hmax + 1, zrow = yrow + kp.kmax + 1;
    // the runs' table offsets: all of them once when they fit the arrays, else those of each
    // pass before it (index p - rbase; the caller syncs before the epilogue reads them)
    const bool rall = nr <= TC_MAXRUN;
    auto load_runs = [&](int pass) {
        const int p = (rall ? 0 : pass * nph) + tid;
        if (tid < (rall ? nr : nph) && p < nr) {
            const int kxy = a.slot[p].x, kx = kxy & 255, ky = (kxy >> 8) - 128;
            const int ry = yrow + (ky < 0 ? -ky : ky);
            sroff[tid] = make_int4(kx * 128, (kx & 7) << 4, ry * 128, ((ry & 7) << 4) | (ky < 0 ? 1 : 0));
            const float ws = DG ? 1.f : 1.f / TF_WS;  // TF_DG scales its sums once at the end
            sskv[tid] = make_float2(a.skv[p].x * ws, a.skv[p].y * ws);
        }
    };
    load_runs(0);
    if (warp == 0) umma::tmem_alloc(&tslot, 512);
    // the (k(+j), k(-j)) pairs and k_z of a V item (run p0 + it % nrow, j = 4 (it / nrow) + e):
    // this thread's first item of each early V build is fetched now, before the weights land
    auto fetch_km = [&](int p0, int nrow, int it, int2 (&km)[4], float (&kz)[4]) {
        const int p = p0 + it % nrow, jc = it / nrow;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int j = 4 * jc + e;
            const bool ok = it < nrow * kcm && p < nr && j < jm;
            km[e] = ok ? a.kpm[p * jm + j] : make_int2(-1, -1);
            kz[e] = ok ? a.kzv[kp.lmax + j] : 0.f;
        }
    };
    int2 km0[4], km1[4];
    float kz0[4], kz1[4];
    fetch_km(0, nph, tid, km0, kz0);
    fetch_km(vpp ? 0 : nph, nph, tid, km1, kz1);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tm = tslot;
    unsigned char *Vh = sm + L.B, *Vl = Vh + a.ncol * a.kq * 2;
    unsigned char *Qh = sm + L.A, *Ql = Qh + TF_SITES * a.kq * 2;
    // Q = ez rows of the CTA's sites, 8 halves (4 j: c_j, s_j) per item, zero for j >= jm
    uint32_t err = (uint32_t)umma::mbar_wait(&tbar, 0, TC_WAIT);
    for (int it = tid; it < TF_SITES * kcm; it += TF_NT) {
        const int s = it % TF_SITES, jc = it / TF_SITES;
        float v[8];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int j = 4 * jc + e;
            const float2 z = j < jm ? tab_elem(sm, L.boxb, zrow + j, s) : make_float2(0.f, 0.f);
            v[2 * e] = z.x;
            v[2 * e + 1] = z.y;
        }
        uint4 hi, lo;
        split8_h(v, hi, lo);
        const int o = rowchunk_k(s, jc, kcm);
        *reinterpret_cast<uint4 *>(Qh + o) = hi;
        *reinterpret_cast<uint4 *>(Ql + o) = lo;
    }
    // everything above reads only the positions; from here on the structure factor's weights
    // and the iteration's dipoles and fields (a programmatic launch waits for them here)
    if (a.pdl) {
        pdl_wait();
        if (tid == 0 && !a.wglob) {
            const int slot = (MODE == TF_D || MODE == TF_QG) ? 1 : 0;
            const uint32_t wbytes = (uint32_t)kp.nk * 8u * (DG ? 2u : 1u);
            mbar_expect_tx(&wbar, wbytes);
            bulk_load(sm + L.W, kp.Wf + ((size_t)b * 2 + slot) * kp.nk, wbytes, &wbar);
        }
    }
    // the SOR inputs of the CTA's dipole sites
    const int s_own = sb + tid;
    const bool own = tid < TF_SITES && s_own >= a.s_lo && s_own < a.s_hi;
    DdSite din;
    if (MODE == TF_D && own && !kp.dd_async) dd_sor_load(kp, b, s_own, din);
    if (!a.wglob) err |= (uint32_t)umma::mbar_wait(&wbar, 0, TC_WAIT);
    const float2 *W = a.wglob ? kp.Wf + ((size_t)b * 2 + ((MODE == TF_D || MODE == TF_QG) ? 1 : 0)) * kp.nk
                              : reinterpret_cast<const float2 *>(sm + L.W);
    // V of runs [p0, p0 + nrow): run p0 + pl, component c at row vrow0 + c nrow + pl; 8 halves
    // (4 j) per item, zero for runs >= nr and j >= jm
    auto build_v = [&](int p0, int nrow, int vrow0, const int2 (&kmf)[4], const float (&kzf)[4]) {
        for (int it = tid; it < nrow * kcm; it += TF_NT) {
            const int pl = it % nrow, jc = it / nrow;
            int2 km[4];
            float kzz[4];
            if (it == tid) {
#pragma unroll
                for (int e = 0; e < 4; e++) km[e] = kmf[e], kzz[e] = kzf[e];
            } else {
                fetch_km(p0, nrow, it, km, kzz);
            }
            float v[NC][8];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                float2 wp = make_float2(0.f, 0.f), wm = wp;
                const float kz = kzz[e];
                {
                    float2 wpl = km[e].x >= 0 ? W[km[e].x] : make_float2(0.f, 0.f);
                    float2 wmi = km[e].y >= 0 ? W[km[e].y] : make_float2(0.f, 0.f);
                    if (DG) {  // total weights W_q + W_mu
                        if (km[e].x >= 0) wpl = make_float2(wpl.x + W[kp.nk + km[e].x].x, wpl.y + W[kp.nk + km[e].x].y);
                        if (km[e].y >= 0) wmi = make_float2(wmi.x + W[kp.nk + km[e].y].x, wmi.y + W[kp.nk + km[e].y].y);
                    }
                    wp = make_float2(TF_WS * (wpl.x + wmi.x), TF_WS * (wpl.y + wmi.y));
                    wm = make_float2(TF_WS * (wpl.x - wmi.x), TF_WS * (wpl.y - wmi.y));
                }
                // (cos, sin) coefficients of T0re, T0im, T1re, T1im (, T2re, T2im)
                v[0][2 * e] = wp.x;
                v[0][2 * e + 1] = -wm.y;
                v[1][2 * e] = wp.y;
                v[1][2 * e + 1] = wm.x;
                v[2][2 * e] = kz * wm.x;
                v[2][2 * e + 1] = -kz * wp.y;
                v[3][2 * e] = kz * wm.y;
                v[3][2 * e + 1] = kz * wp.x;
                if constexpr (DG) {
                    const float k2 = kz * kz;
                    v[4][2 * e] = k2 * wp.x;
                    v[4][2 * e + 1] = -k2 * wm.y;
                    v[5][2 * e] = k2 * wp.y;
                    v[5][2 * e + 1] = k2 * wm.x;
                }
            }
#pragma unroll
            for (int c = 0; c < NC; c++) {
                uint4 hi, lo;
                split8_h(v[c], hi, lo);
                const int o = rowchunk_k(vrow0 + c * nrow + pl, jc, kcm);
                *reinterpret_cast<uint4 *>(Vh + o) = hi;
                *reinterpret_cast<uint4 *>(Vl + o) = lo;
            }
        }
    };
    if (!vpp) {  // both passes: pass q's rows from q 4 nph
        build_v(0, nph, 0, km0, kz0);
        build_v(nph, nph, 4 * nph, km1, kz1);
    }
    // passes of nph runs, NC nph <= 512 TMEM columns each: column c nph + pl for component c
    // of the pass's run pl
    float Ex = 0.f, Ey = 0.f, Ez = 0.f, phi = 0.f;
    const int lq = warp & 3, part = warp >> 2, sl = 32 * lq + lane;
    const int q4 = nph / 4;  // runs per run quarter
    // the epilogue lane's site in the staged tables: its box and float2 slot, and its 16-byte
    // chunk (before the swizzle) times 16
    const unsigned char *tsite = sm + (sl >> 4) * L.boxb + (sl & 1) * 8;
    const int cs4 = ((sl & 15) >> 1) << 4;
    // TF_DG: the dipole of the epilogue lane's site (scaled by nothing; zero outside the range)
    float mu[3] = {0.f, 0.f, 0.f};
    if (DG && sb + sl >= a.s_lo && sb + sl < a.s_hi) {
        const float4 m = kp.dipf[(size_t)b * kp.S + sb + sl];
        mu[0] = m.x, mu[1] = m.y, mu[2] = m.z;
    }
    bool bad = err != 0;
    for (int pass = 0; pass < npass; pass++) {
        if (pass > 0 && !rall) load_runs(pass);  // (the previous pass's epilogue is past its last sync)
        const int rbase = rall ? 0 : pass * nph;
        if (vpp) {
            if (pass == 0) {
                build_v(0, nph, 0, km0, kz0);
            } else {
                fetch_km(pass * nph, nph, tid, km1, kz1);
                build_v(pass * nph, nph, 0, km1, kz1);
            }
        }
        umma::fence_smem_to_async();
        umma::fence_before_sync();
        bad = __syncthreads_or((int)bad) != 0;
        umma::fence_after_sync();
        if (bad) break;
        if (tid == 0) {
            const uint32_t idesc_base = umma::idesc_f16(128, 16) & ~(0x3Fu << 17);
            const uint32_t qh = umma::smem_u32(Qh), ql = umma::smem_u32(Ql);
            const uint32_t vh = umma::smem_u32(Vh), vl = umma::smem_u32(Vl);
            for (int c0 = 0; c0 < NC * nph; c0 += 256) {
                const int N = min(256, NC * nph - c0);
                const uint32_t id = idesc_base | ((uint32_t)(N >> 3) << 17);
                const uint32_t d = tm + (uint32_t)c0;
                const int vr = (vpp ? 0 : pass * 4 * nph) + c0;  // first V row of the MMA
                const uint32_t vo = (uint32_t)((vr >> 3) * kcm * 128);
                for (int ks = 0; ks < a.kq / 16; ks++) {
                    const uint64_t dq_h = umma::sdesc(qh + ks * 256, 128, kcm * 128), dq_l = umma::sdesc(ql + ks * 256, 128, kcm * 128);
                    const uint64_t dv_h = umma::sdesc(vh + vo + ks * 256, 128, kcm * 128), dv_l = umma::sdesc(vl + vo + ks * 256, 128, kcm * 128);
                    umma::mma_f16(d, dq_h, dv_h, id, ks > 0);
                    umma::mma_f16(d, dq_h, dv_l, id, 1);
                    umma::mma_f16(d, dq_l, dv_h, id, 1);
                }
            }
            umma::commit(&mbar);
        }
        __syncwarp();
        int to = umma::mbar_wait(&mbar, (uint32_t)(pass & 1), TC_WAIT);
        if (to) to = umma::mbar_wait(&mbar, (uint32_t)(pass & 1), TC_WAIT);
        umma::fence_after_sync();
        bad = __syncthreads_or(to) != 0;
        if (bad) break;
        // this warp's run quarter in groups of 16 runs x 4 (6) components (one TMEM wait each)
        for (int pl0 = part * q4; pl0 < (part + 1) * q4; pl0 += 16) {
            if (pass * nph + pl0 >= nr) break;
            float v[64];
            const uint32_t tl = tm + ((uint32_t)(32 * lq) << 16) + (uint32_t)pl0;
            umma::tmem_ld16x4(tl, tl + (uint32_t)nph, tl + (uint32_t)(2 * nph), tl + (uint32_t)(3 * nph), v);
            float w[32];
            if constexpr (DG) umma::tmem_ld16x2(tl + (uint32_t)(4 * nph), tl + (uint32_t)(5 * nph), w);
#pragma unroll
            for (int e = 0; e < 16; e++) {
                const int pl = pl0 + e, p = pass * nph + pl;
                if (pl >= (part + 1) * q4 || p >= nr) break;
                // tab_elem(sm, boxb, row, sl) with the run's row offsets and keys precomputed
                const int4 ro = sroff[p - rbase];
                const float2 ex = *reinterpret_cast<const float2 *>(tsite + ro.x + (cs4 ^ ro.y));
                float2 ey = *reinterpret_cast<const float2 *>(tsite + ro.z + (cs4 ^ (ro.w & ~1)));
                if (ro.w & 1) ey.y = -ey.y;
                // ewald.f90:30-31: coskxky = cx cy - sx sy, sinkxky = sx cy + cx sy
                const float er = ex.x * ey.x - ex.y * ey.y, ei = ex.y * ey.x + ex.x * ey.y;
                const float2 kv = sskv[p - rbase];
                if constexpr (DG) {
                    // sum_k k (k . mu) Re(e W) with the run's kz sums (ewald.f90:146-187)
                    const float R0 = fmaf(er, v[e], -ei * v[16 + e]);       // Re(exy T0)
                    const float R1 = fmaf(er, v[32 + e], -ei * v[48 + e]);  // Re(exy T1)
                    const float R2 = fmaf(er, w[e], -ei * w[16 + e]);       // Re(exy T2)
                    const float aa = kv.x * mu[0] + kv.y * mu[1];
                    const float tt = fmaf(aa, R0, mu[2] * R1);
                    Ex = fmaf(-kv.x, tt, Ex);
                    Ey = fmaf(-kv.y, tt, Ey);
                    Ez -= fmaf(aa, R1, mu[2] * R2);
                } else {
                    const float t0 = fmaf(er, v[16 + e], ei * v[e]);       // Im(exy T0)
                    const float t1 = fmaf(er, v[48 + e], ei * v[32 + e]);  // Im(exy T1)
                    Ex = fmaf(kv.x, t0, Ex);
                    Ey = fmaf(kv.y, t0, Ey);
                    Ez = fmaf(1.f / TF_WS, t1, Ez);
                    if (MODE == TF_Q || MODE == TF_QG) phi = fmaf(1.f / TF_WS, fmaf(er, v[e], -ei * v[16 + e]), phi);  // Re(exy T0)
                }
            }
        }
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
    }
    if (DG) {
        Ex *= 1.f / TF_WS;
        Ey *= 1.f / TF_WS;
        Ez *= 1.f / TF_WS;
    }
    // the four run quarters of each site, in order
    float *red = reinterpret_cast<float *>(Qh);  // [4][128][4]
    red[(part * TF_SITES + sl) * 4 + 0] = Ex;
    red[(part * TF_SITES + sl) * 4 + 1] = Ey;
    red[(part * TF_SITES + sl) * 4 + 2] = Ez;
    red[(part * TF_SITES + sl) * 4 + 3] = phi;
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after_sync();
        umma::tmem_dealloc(tm, 512);
        umma::tmem_relinquish();
    }
    float e[4] = {0.f, 0.f, 0.f, 0.f};
    if (own && !bad) {
#pragma unroll
        for (int rq = 0; rq < 4; rq++)
#pragma unroll
            for (int c = 0; c < 4; c++) e[c] += red[(rq * TF_SITES + tid) * 4 + c];
    }
    if (bad && tid == 0) atomicOr(kp.err, 8u);
    if (MODE == TF_Q && (kp.fx_mode & 1)) {  // into the scratch (this pass runs beside the pair kernels)
        if (own && !bad)
            kp.Fx[(size_t)b * kp.S + s_own] =
                make_double4_32a((double)e[0], (double)e[1], (double)e[2], s_own >= kp.fq ? (double)e[3] : 0.0);
        return;
    }
    if ((MODE == TF_QG || MODE == TF_DG) && (kp.fx_mode & 2)) {
        if (own && !bad) {
            const size_t gs = (size_t)b * kp.S + s_own;
            if (MODE == TF_QG) {
                const double q = kp.pos[gs].w;
                kp.Fx[gs] = make_double4_32a(-q * (double)e[0], -q * (double)e[1], -q * (double)e[2],
                                             s_own >= kp.fq ? (double)e[3] : 0.0);
            } else {
                double4_32a f = kp.Fx[gs];
                f.x += (double)e[0];
                f.y += (double)e[1];
                f.z += (double)e[2];
                kp.Fx[gs] = f;
            }
        }
        return;
    }
    if (MODE == TF_Q) {
        // ewald.f90:45-49 as k_field_finish<F_Q>: Efq += E, phi += (charged sites)
        if (own && !bad) {
            const size_t gs = (size_t)b * kp.S + s_own;
            double4_32a f = kp.F[gs];
            f.x += (double)e[0];
            f.y += (double)e[1];
            f.z += (double)e[2];
            if (s_own >= kp.fq) f.w += (double)e[3];
            kp.F[gs] = f;
        }
        return;
    }
    if (MODE == TF_QG || MODE == TF_DG) {
        // as k_field_finish<F_QD>: dR += -q E (charge part) or the dipole force; phi of the
        // dipole structure factor at the charged sites
        if (own && !bad) {
            const size_t gs = (size_t)b * kp.S + s_own;
            const double q = MODE == TF_QG ? kp.pos[gs].w : -1.0;
            kp.dR[3 * gs + 0] -= q * (double)e[0];
            kp.dR[3 * gs + 1] -= q * (double)e[1];
            kp.dR[3 * gs + 2] -= q * (double)e[2];
            if (MODE == TF_QG && s_own >= kp.fq) kp.F[gs].w += (double)e[3];
        }
        return;
    }
    if (kp.dd_async) {
        // the real-space field runs beside this pass: store the reciprocal field, arrive, and
        // run the unit's SOR update if the real-space blocks of its molecules are done
        if (own && !bad) kp.Erec[(size_t)b * kp.S + s_own] = make_float4(e[0], e[1], e[2], 0.f);
        const float er[3] = {e[0], e[1], e[2]};
        if (dd_unit_arrive(kp, b, t)) dd_unit_sor<TF_NT>(kp, b, t, own && !bad, er);
        return;
    }
    // the iteration's FP64 SOR update at the CTA's dipole sites, then the block's end
    double av[2] = {0.0, 0.0};
    if (own && !bad) {
        const double E[3] = {(double)e[0], (double)e[1], (double)e[2]};
        dd_sor_apply(kp, b, s_own, din, E, iter, av);
    }
    dd_block_end<TF_NT, TF_SITES / 32>(kp, b, av, !bad);  // own sites: threads < TF_SITES
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
    if (E.precision != PIMD_MIXED || kp.ld <= kp.fd || !kp.tabf || !kp.dipf || !kp.Wf) return;
    // TMA rules: row pitch S x 8 bytes a multiple of 16, box rows <= 256; kz table <= 256
    if ((kp.S & 1) || kp.ntab > 256 || 2 * kp.lmax + 1 > 256) return;
    int major = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, E.device);
    if (major != 10) return;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return;
    // the FP32 k_z of a k-vector depends on kz alone
    std::vector<float> kzv(2 * kp.lmax + 1, 0.f);
    std::vector<int> kzseen(2 * kp.lmax + 1, 0);
    for (int r = 0; r < kp.nrun; r++) {
        const KRun &run = E.h_runs[r];
        for (int j = 0; j < run.nkz; j++) {
            const int kz = run.kzlo + j, k = run.kbeg + j;
            const float v = (float)E.h_kvec[3 * k + 2];
            if (kzseen[kz + kp.lmax] && kzv[kz + kp.lmax] != v) return;
            kzseen[kz + kp.lmax] = 1;
            kzv[kz + kp.lmax] = v;
        }
    }
    // runs sorted by their largest |kz| (longest first), groups of <= 256 runs, 6 (max |kz| + 1)
    // Z rows per group <= 128
    std::vector<int> order(kp.nrun), jr(kp.nrun);
    for (int r = 0; r < kp.nrun; r++) {
        const KRun &run = E.h_runs[r];
        jr[r] = std::max(std::abs(run.kzlo), std::abs(run.kzlo + run.nkz - 1)) + 1;
        order[r] = r;
    }
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return jr[x] > jr[y]; });
    // slots: every run once with its |kz| rows below TC_JB, then the runs reaching beyond once
    // per further band of TC_JB rows (j0 = TC_JB, 2 TC_JB, ...), each band in groups of <= 256
    // slots; a slot's k-vectors outside its group's rows are local entries with k = -1
    constexpr int TC_JB = 21;  // 6 TC_JB <= 128 Z rows
    std::vector<int2> src;     // (run, j0)
    for (int q = 0; q < kp.nrun; q++) src.push_back(make_int2(order[q], 0));
    for (int j0 = TC_JB;; j0 += TC_JB) {
        const size_t n0 = src.size();
        for (int q = 0; q < kp.nrun; q++)
            if (jr[order[q]] > j0) src.push_back(make_int2(order[q], j0));
        if (src.size() == n0) break;
    }
    const int nslot = (int)src.size();
    std::vector<int4> slots(nslot);
    std::vector<float2> skv(nslot);
    std::vector<TcGroup> groups;
    std::vector<TcKW> kloc;
    std::vector<float2> runkf(kp.nrun);
    for (int r = 0; r < kp.nrun; r++)
        runkf[r] = make_float2((float)E.h_kvec[3 * E.h_runs[r].kbeg], (float)E.h_kvec[3 * E.h_runs[r].kbeg + 1]);
    int ncolmax = 16, nklmax = 0, nvalid = 0;
    // while a group's X is built, its 2 nr X items take whole builder warps first and the Z items
    // (12 jm at most) the warps left over, TC_ZMAX per thread: the most runs a group of jm rows holds
    auto zfit = [](int nr, int jm) {
        const int zw = std::max(1, TC_NB - (2 * nr + 31) / 32);
        return (12 * jm + 32 * zw - 1) / (32 * zw) <= TC_ZMAX;
    };
    for (int p0 = 0; p0 < nslot;) {
        const int j0 = src[p0].y, jmg = std::min(TC_JB, jr[src[p0].x] - j0);
        int nr = 0;
        while (p0 + nr < nslot && nr < TC_MAXRUN && src[p0 + nr].y == j0 && zfit(nr + 1, jmg)) nr++;
        if (nr == 0) return;
        TcGroup g{p0, nr, 0, jmg, 0, (int)kloc.size(), j0, 0};
        g.ncol = ((2 * g.nr + 15) / 16) * 16;
        for (int p = p0; p < p0 + g.nr; p++) {
            const int r = src[p].x;
            const KRun &run = E.h_runs[r];
            slots[p] = make_int4(run.kx + 256 * (run.ky + 128), g.nkl, run.kzlo, run.nkz);
            skv[p] = runkf[r];
            for (int j = 0; j < run.nkz; j++) {
                const int akz = std::abs(run.kzlo + j);
                const bool mine = akz >= j0 && akz < j0 + g.jm;
                nvalid += mine;
                kloc.push_back(TcKW{mine ? run.kbeg + j : -1, (float)(FOURPI * E.h_Ak[run.kbeg + j] / kp.volume)});
            }
            g.nkl += run.nkz;
        }
        groups.push_back(g);
        ncolmax = std::max(ncolmax, g.ncol);
        nklmax = std::max(nklmax, g.nkl);
        p0 += nr;
    }
    if (nvalid != kp.nk) return;  // every k-vector in exactly one group
    // dynamic shared memory available: the opt-in limit minus the kernel's static part
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, E.device);
    cudaFuncAttributes fa, fq, fd;
    if (cudaFuncGetAttributes(&fa, k_sfac_tc<TC_OP_MU>) != cudaSuccess ||
        cudaFuncGetAttributes(&fq, k_sfac_tc<TC_OP_Q>) != cudaSuccess ||
        cudaFuncGetAttributes(&fd, k_sfac_tc<TC_OP_DIP>) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    const int dmax = optin - (int)std::max(fa.sharedSizeBytes, std::max(fq.sharedSizeBytes, fd.sharedSizeBytes));
    // operand buffers: three when they fit, else two
    int nabuf = TC_NABUF_MAX;
    while (nabuf > 2 && TcSmem(kp.ntab, ncolmax, nabuf).total > dmax) nabuf--;
    const TcSmem L(kp.ntab, ncolmax, nabuf);
    if (L.total > dmax) return;
    // the epilogue's staging tile and partial S reuse the table and operand regions
    if (128 * TC_LD * 4 + 8 * nklmax > L.total - 1024) return;
    if (cudaFuncSetAttribute(k_sfac_tc<TC_OP_MU>, cudaFuncAttributeMaxDynamicSharedMemorySize, dmax) != cudaSuccess ||
        cudaFuncSetAttribute(k_sfac_tc<TC_OP_Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, dmax) != cudaSuccess ||
        cudaFuncSetAttribute(k_sfac_tc<TC_OP_DIP>, cudaFuncAttributeMaxDynamicSharedMemorySize, dmax) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    // the component sums keep three partials per k-vector
    E.tc_dip_ok = 128 * TC_LD * 4 + 3 * 8 * nklmax <= L.total - 1024;
    int4 *d_slots = nullptr;
    float2 *d_skv = nullptr;
    TcGroup *d_groups = nullptr;
    TcKW *d_kloc = nullptr;
    float *d_kzv = nullptr;
    if (cudaMalloc((void **)&d_slots, sizeof(int4) * slots.size()) != cudaSuccess ||
        cudaMalloc((void **)&d_skv, sizeof(float2) * skv.size()) != cudaSuccess ||
        cudaMalloc((void **)&d_groups, sizeof(TcGroup) * groups.size()) != cudaSuccess ||
        cudaMalloc((void **)&d_kloc, sizeof(TcKW) * kloc.size()) != cudaSuccess ||
        cudaMalloc((void **)&d_kzv, sizeof(float) * kzv.size()) != cudaSuccess) {
        cudaGetLastError();
        for (void *p : {(void *)d_slots, (void *)d_skv, (void *)d_groups, (void *)d_kloc, (void *)d_kzv})
            if (p) cudaFree(p);
        return;
    }
    for (void *p : {(void *)d_slots, (void *)d_skv, (void *)d_groups, (void *)d_kloc, (void *)d_kzv}) E.allocs.push_back(p);
    cudaMemcpy(d_slots, slots.data(), sizeof(int4) * slots.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(d_skv, skv.data(), sizeof(float2) * skv.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(d_groups, groups.data(), sizeof(TcGroup) * groups.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(d_kloc, kloc.data(), sizeof(TcKW) * kloc.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(d_kzv, kzv.data(), sizeof(float) * kzv.size(), cudaMemcpyHostToDevice);
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
    E.d_tcslot = d_slots;
    E.d_tcskv = d_skv;
    E.d_tcgrp = d_groups;
    E.d_tckloc = d_kloc;
    E.d_tckzv = d_kzv;
    // X-operand cache of the dipole sites (k_sfac_tc, TC_OP_MU): per bead and run group, one
    // block per 16 sites from the first site group's base, hi and lo rows [0, 2 nr) rounded to
    // 8-row groups; zero-filled once (the padding rows are never written)
    E.d_tcx = nullptr;
    if (kp.ld > kp.fd) {
        int xb = 0;
        for (const TcGroup &g : groups) xb = std::max(xb, ((2 * g.nr + 7) / 8) * 256);
        const int sbase = kp.fd & ~(TC_SS - 1);
        const int xsub = (kp.ld - sbase + TC_SS - 1) / TC_SS * (TC_SS / TC_KS);  // whole table stages
        const size_t bytes = (size_t)kp.P * groups.size() * xsub * 2 * xb;
        void *d_x = nullptr;
        if (cudaMalloc(&d_x, bytes) == cudaSuccess) {
            E.allocs.push_back(d_x);
            cudaMemset(d_x, 0, bytes);
            E.d_tcx = d_x;
            E.tc_xsub = xsub;
            E.tc_xblock = 2 * xb;
        } else {
            cudaGetLastError();
        }
    }
    E.tc_ntg = (int)groups.size();
    E.tc_ncolmax = ncolmax;
    E.tc_nabuf = nabuf;
    E.tc_ready = true;
    // field kernel: every run once (the first kp.nrun slots, in the same order), K over its
    // whole |kz| range; per (run, j) the k-vectors of kz = +j and -j
    E.tf_ready = false;
    const int nr = kp.nrun, jm = jr[order[0]], kq = ((2 * jm + 15) / 16) * 16;
    const void *fk[7] = {(const void *)k_field_tc<TF_Q, false>, (const void *)k_field_tc<TF_D, false>,
                         (const void *)k_field_tc<TF_QG, false>, (const void *)k_field_tc<TF_Q, true>,
                         (const void *)k_field_tc<TF_D, true>, (const void *)k_field_tc<TF_QG, true>,
                         (const void *)k_field_tc<TF_DG, true>};
    size_t fstat = 0;
    for (const void *f : fk) {
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, f) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        fstat = std::max(fstat, fa.sharedSizeBytes);
    }
    const int dmaxf = optin - (int)fstat;
    for (const void *f : fk)
        if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, dmaxf) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
    // passes: two passes of nph runs (a multiple of 8) x 4 components in TMEM with V of both built
    // once, when that fits (plus the 16 columns the last 16-run load of a run quarter reaches past
    // a pass); else passes of nph runs with V of each built before it. The bead's weights sit in
    // shared memory (one bulk copy: 8 nk bytes, a multiple of 16) when they fit, else the V
    // builders read them from global memory.
    auto fits = [&](int nph_, int vpp_, int wglob_, int ncomp, int nslot_) {
        return ncomp * nph_ + 16 <= 512 && TfSmem(kp.ntab, (vpp_ ? ncomp : 2 * ncomp) * nph_, kq, kp.nk, wglob_ ? 0 : nslot_).total <= dmaxf;
    };
    const bool w_ok = (kp.nk & 1) == 0;
    int nph = ((nr + 1) / 2 + 7) / 8 * 8, vpp = 0, wglob = w_ok ? 0 : 1;
    if (!fits(nph, 0, wglob, 4, 1)) {
        vpp = 1;
        for (wglob = w_ok ? 0 : 1; wglob < 2; wglob++) {
            for (nph = std::min(120, (nr + 7) / 8 * 8); nph > 8 && !fits(nph, 1, wglob, 4, 1); nph -= 8) {
            }
            if (fits(nph, 1, wglob, 4, 1)) break;
        }
        if (wglob == 2) return;
    }
    const int ncolf = (vpp ? 4 : 8) * nph;
    if (kp.ntab > 128) return;
    std::vector<int2> kpm((size_t)nr * jm, make_int2(-1, -1));
    for (int p = 0; p < nr; p++) {
        const KRun &run = E.h_runs[order[p]];
        for (int j = 0; j < jm; j++) {
            int2 v = make_int2(-1, -1);
            if (j >= run.kzlo && j < run.kzlo + run.nkz) v.x = run.kbeg + j - run.kzlo;
            if (j > 0 && -j >= run.kzlo && -j < run.kzlo + run.nkz) v.y = run.kbeg - j - run.kzlo;
            kpm[(size_t)p * jm + j] = v;
        }
    }
    int2 *d_kpm = nullptr;
    if (cudaMalloc((void **)&d_kpm, sizeof(int2) * kpm.size()) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    E.allocs.push_back(d_kpm);
    cudaMemcpy(d_kpm, kpm.data(), sizeof(int2) * kpm.size(), cudaMemcpyHostToDevice);
    E.d_tfkpm = d_kpm;
    E.tf_nr = nr;
    E.tf_nph = nph;
    E.tf_jm = jm;
    E.tf_ncol = ncolf;
    E.tf_kq = kq;
    E.tf_vpp = vpp;
    E.tf_wglob = wglob;
    E.tf_ready = true;
    // dipole-force mode: 6 components per run, passes of nphd runs (a multiple of 8) with
    // 6 nphd + 16 <= 512 TMEM columns, V of one pass at a time, both weight slots in shared
    // memory when they fit
    const int npd = (nr + 79) / 80;
    int nphd = ((nr + npd - 1) / npd + 7) / 8 * 8, wgd = w_ok ? 0 : 1;
    for (; wgd < 2; wgd++) {
        for (nphd = ((nr + npd - 1) / npd + 7) / 8 * 8; nphd > 8 && !fits(nphd, 1, wgd, 6, 2); nphd -= 8) {
        }
        if (fits(nphd, 1, wgd, 6, 2)) break;
    }
    E.tf_qd_ready = wgd < 2;
    E.tf_nphd = nphd;
    E.tf_ncold = 6 * nphd;
    E.tf_wglob_d = wgd;
}

// whether the iterations' field pass is launched as a programmatic dependent (griddepcontrol.wait
// before it reads the iteration's fields)
bool field_pdl_ok(const Engine &E) { return E.tc_ready && E.tf_ready && E.ff_tc && E.tc_pdl && E.sf_tc; }

// mode TF_D: dipole field, SOR update and convergence test of one iteration at the dipole sites
// [s0, s1) (k_field_f<F_D> + k_field_finish<F_D>); TF_Q: charge field and potential added to F at
// [s0, s1) (k_field_f<F_Q> + k_field_finish<F_Q>); TF_QG, TF_DG: the halves of the force pass
// (launch_field_qd_tc). 1 when launched, else 0.
int launch_field_tc(Engine &E, int mode, int s0, int s1) {
    if (!E.tc_ready || !E.tf_ready || !E.ff_tc || s1 <= s0) return 0;
    const KP &kp = E.kp;
    TfArgs a;
    a.slot = E.d_tcslot;
    a.skv = E.d_tcskv;
    a.kpm = E.d_tfkpm;
    a.kzv = E.d_tckzv;
    a.nr = E.tf_nr;
    a.nph = E.tf_nph;
    a.ncol = E.tf_ncol;
    a.kq = E.tf_kq;
    a.jm = E.tf_jm;
    a.sbase = s0 & ~(TC_SS - 1);  // TMA x coordinates 2 (sbase + 16 i): 128-byte aligned
    a.s_lo = s0;
    a.s_hi = s1;
    a.vpp = E.tf_vpp;
    a.wglob = E.tf_wglob;
    if (mode == TF_DG) {
        a.nph = E.tf_nphd;
        a.ncol = E.tf_ncold;
        a.vpp = 1;
        a.wglob = E.tf_wglob_d;
    }
    const TfSmem L(kp.ntab, a.ncol, a.kq, kp.nk, a.wglob ? 0 : (mode == TF_DG ? 2 : 1));
    dim3 g((s1 - a.sbase + TF_SITES - 1) / TF_SITES, kp.P);
    const CUtensorMap *map = reinterpret_cast<const CUtensorMap *>(E.tc_map);
    a.pdl = 0;
    if (mode == TF_D && E.tc_pdl && E.sf_tc) {
        // a programmatic dependent of the iteration's structure factor: its set-up (tables,
        // Q) runs while that grid finishes; it waits (pdl_wait) before reading the weights
        a.pdl = 1;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = g;
        cfg.blockDim = dim3(TF_NT);
        cfg.dynamicSmemBytes = L.total;
        cfg.stream = E.stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        const cudaError_t le = a.vpp ? cudaLaunchKernelEx(&cfg, k_field_tc<TF_D, true>, *map, kp, a)
                                     : cudaLaunchKernelEx(&cfg, k_field_tc<TF_D, false>, *map, kp, a);
        if (le == cudaSuccess) {
            ++E.nlaunch;
            return 1;
        }
        cudaGetLastError();
        a.pdl = 0;
        E.tc_pdl = false;  // not available: plain launches from now on
        if (E.field_needs_join) cudaStreamWaitEvent(E.stream, E.loop_join, 0);
    }
    if (mode == TF_D)
        a.vpp ? k_field_tc<TF_D, true><<<g, TF_NT, L.total, E.stream>>>(*map, kp, a)
              : k_field_tc<TF_D, false><<<g, TF_NT, L.total, E.stream>>>(*map, kp, a);
    else if (mode == TF_Q)
        a.vpp ? k_field_tc<TF_Q, true><<<g, TF_NT, L.total, E.stream>>>(*map, kp, a)
              : k_field_tc<TF_Q, false><<<g, TF_NT, L.total, E.stream>>>(*map, kp, a);
    else if (mode == TF_QG)
        a.vpp ? k_field_tc<TF_QG, true><<<g, TF_NT, L.total, E.stream>>>(*map, kp, a)
              : k_field_tc<TF_QG, false><<<g, TF_NT, L.total, E.stream>>>(*map, kp, a);
    else
        k_field_tc<TF_DG, true><<<g, TF_NT, L.total, E.stream>>>(*map, kp, a);
    ++E.nlaunch;
    return 1;
}

// The differentiation form's reverse sweep on the mixed engine: the reciprocal field at the
// dipole sites from the charge weight slot (TF_Q: into kp.Fx with fx_mode 1), and the dipole
// force of kp.dipf from the two weight slots (TF_DG: into kp.dR, or kp.Fx with fx_mode 2), at
// [fd, ld). 1 when launched, else 0.
int launch_adj_field_tc(Engine &E) {
    if (!E.tf_qd_ready || E.kp.ld <= E.kp.fd) return 0;
    return launch_field_tc(E, TF_Q, E.kp.fd, E.kp.ld);
}
int launch_adj_dforce_tc(Engine &E) {
    if (!E.tf_qd_ready || E.kp.ld <= E.kp.fd) return 0;
    return launch_field_tc(E, TF_DG, E.kp.fd, E.kp.ld);
}
// the charge half of the force pass (TF_QG: -q E and phi of the dipole slot's weights) at the
// charged sites from N on (TTM3-F: H1, H2, M), into kp.Fx with fx_mode 2
int launch_adj_qforce_tc(Engine &E) {
    if (!E.tf_qd_ready) return 0;
    return launch_field_tc(E, TF_QG, E.kp.N, E.kp.S);
}

// ewald_std_qd's force pass (k_field_f<F_QD> + k_field_finish<F_QD>) as two tensor-core passes:
// the charge force -q E and potential from the dipole structure factor at [s0, s1), then the
// dipole force at the dipole sites from the total structure factor. 1 when launched, else 0.
int launch_field_qd_tc(Engine &E, int s0, int s1) {
    if (!E.tc_ready || !E.tf_ready || !E.tf_qd_ready || !E.ff_tc || s1 <= s0) return 0;
    launch_field_tc(E, TF_QG, s0, s1);
    if (E.kp.ld > E.kp.fd) launch_field_tc(E, TF_DG, E.kp.fd, E.kp.ld);
    return 1;
}

// Returns 1 when the launch wrote the structure factor of `op` (Sq and the charge weights, Sm
// and the dipole weights, or Sdip; no k_sreduce needed), else 0.
int launch_sfac_tc(Engine &E, int op, int s0, int nsites, int skipconv) {
    if (!E.tc_ready || !E.sf_tc || nsites <= 0 || (op == TC_OP_DIP && !E.tc_dip_ok)) return 0;
    const KP &kp = E.kp;
    TcArgs a;
    a.slot = E.d_tcslot;
    a.skv = E.d_tcskv;
    a.grp = reinterpret_cast<const TcGroup *>(E.d_tcgrp);
    a.kw = reinterpret_cast<const TcKW *>(E.d_tckloc);
    a.kzv = E.d_tckzv;
    a.sbase = s0 & ~(TC_SS - 1);  // TMA x coordinate 2 sbase: 256-byte aligned
    a.s_lo = s0;
    a.s_hi = s0 + nsites;
    a.ncolmax = E.tc_ncolmax;
    a.nabuf = E.tc_nabuf;
    a.skipconv = skipconv;
    // the iterations' dipole structure factor caches X (its site range is the cached one)
    const bool xok = op == TC_OP_MU && E.d_tcx && E.tc_xcache && s0 == kp.fd && nsites == kp.ld - kp.fd;
    a.xcache = xok ? reinterpret_cast<uint4 *>(E.d_tcx) : nullptr;
    a.xsub = E.tc_xsub;
    a.xblock = E.tc_xblock;
    a.xkeep = E.l2_keep ? 1 : 0;
    // the iterations' structure factor follows the previous iteration's field pass on the stream
    // (or the charge passes, which need no overlap): its CTAs are scheduled as that grid drains
    a.pdl = (op == TC_OP_MU && skipconv && E.tc_pdl && E.tf_ready && E.ff_tc) ? 1 : 0;
    // one CTA per SM (shared memory); site groups (= cluster size) so that one wave fills the GPU
    static int nsm_cache[64] = {0};
    int &nsm = nsm_cache[E.device & 63];
    if (!nsm) {
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, E.device);
        if (nsm <= 0) nsm = 152;
    }
    const int nst = (a.s_hi - a.sbase + TC_SS - 1) / TC_SS;
    const long per = (long)E.tc_ntg * kp.P;
    int ng = (int)std::max(1L, (long)nsm / per);
    ng = std::max(1, std::min(ng, std::min(nst, TC_CLMAX)));
    const int spg = (nst + ng - 1) / ng;
    a.tsg = spg * TC_SS;
    ng = (nst + spg - 1) / spg;
    const TcSmem L(kp.ntab, a.ncolmax, a.nabuf);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ng, E.tc_ntg, kp.P);
    cfg.blockDim = dim3(TC_NT);
    cfg.dynamicSmemBytes = L.total;
    cfg.stream = E.stream;
    // the highest stream priority: the mixed engine's real-space dipole field runs beside this
    // kernel on a second stream and must not hold the SMs its clusters wait for
    static int prio_cache[64] = {0}, prio_set[64] = {0};
    if (!prio_set[E.device & 63]) {
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess) prio_cache[E.device & 63] = greatest;
        prio_set[E.device & 63] = 1;
    }
    cudaLaunchAttribute at[4];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = ng;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributePriority;
    at[1].val.priority = prio_cache[E.device & 63];
    int na = 2;
    if (a.pdl) {
        at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[na].val.programmaticStreamSerializationAllowed = 1;
        na++;
    }
    // the caller's programmatic event: recorded once every CTA has passed its set-up
    // (griddepcontrol.launch_dependents) or left
    const bool pev = E.sfac_pev_req && op == TC_OP_MU && E.loop_pev;
    if (pev) {
        at[na].id = cudaLaunchAttributeProgrammaticEvent;
        at[na].val.programmaticEvent.event = E.loop_pev;
        at[na].val.programmaticEvent.flags = 0;
        at[na].val.programmaticEvent.triggerAtBlockStart = 0;
        na++;
    }
    cfg.attrs = at;
    cfg.numAttrs = na;
    const CUtensorMap *map = reinterpret_cast<const CUtensorMap *>(E.tc_map);
    cudaError_t e = cudaErrorInvalidValue;
    if (op == TC_OP_MU)
        e = cudaLaunchKernelEx(&cfg, k_sfac_tc<TC_OP_MU>, *map, kp, a);
    else if (op == TC_OP_Q)
        e = cudaLaunchKernelEx(&cfg, k_sfac_tc<TC_OP_Q>, *map, kp, a);
    else
        e = cudaLaunchKernelEx(&cfg, k_sfac_tc<TC_OP_DIP>, *map, kp, a);
    if (e == cudaSuccess && pev) E.sfac_pev_armed = true;
    if (e != cudaSuccess && na > 2) {  // an attribute refused: a plain cluster launch
        cudaGetLastError();
        a.pdl = 0;
        cfg.numAttrs = 2;
        e = cudaLaunchKernelEx(&cfg, k_sfac_tc<TC_OP_MU>, *map, kp, a);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        E.sf_tc = false;  // e.g. no room for the cluster: the FP32-pipe kernel from now on
        return 0;
    }
    ++E.nlaunch;
    return 1;
}

}  // namespace pimd
