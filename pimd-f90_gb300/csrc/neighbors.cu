// neighbors.cu -- O-O neighbour lists of all beads (find_neigh.f90:14-120).
//
// For molecule i the reference keeps every j > i with |R_Oi - R_Oj|^2 < Rc^2 under the anint
// minimum image, in ascending j. Here one warp owns one (molecule, bead): its lanes test 32
// consecutive j at a time, a ballot orders the hits, and the pairs are written in ascending j,
// so the list is the reference's list bit for bit and independent of scheduling. A count pass
// and a fill pass bracket a per-bead exclusive scan. The test is the reference's FP64
// arithmetic with every product and difference rounded separately; the mixed engine first
// tests in FP32 and repeats the FP64 test only within 1e-4 of the cutoff, which gives the same
// decisions. The mixed engine also builds the full list (all j != i) for its dipole gather.
#include "engine.h"
#include "umma.cuh"

namespace pimd {

PIMD_D float wrapf_n(float v, float L, float Li) { return v - L * rint_small(__fmul_rn(v, Li)); }

template <bool PRE>
PIMD_D bool oo_test(const double4_32a &a, const double4_32a &b, const KP &kp) {
    if (PRE) {
        const float rc2f = (float)kp.rc2;
        const float dx = wrapf_n((float)(a.x - b.x), (float)kp.box[0], (float)kp.boxi[0]);
        const float dy = wrapf_n((float)(a.y - b.y), (float)kp.box[1], (float)kp.boxi[1]);
        const float dz = wrapf_n((float)(a.z - b.z), (float)kp.box[2], (float)kp.boxi[2]);
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (fabsf(d2 - rc2f) > 1e-4f * rc2f + 1e-3f) return d2 < rc2f;
    }
    const double x = min_image_rn(__dsub_rn(a.x, b.x), kp.box[0], kp.boxi[0]);
    const double y = min_image_rn(__dsub_rn(a.y, b.y), kp.box[1], kp.boxi[1]);
    const double z = min_image_rn(__dsub_rn(a.z, b.z), kp.box[2], kp.boxi[2]);
    return dot3_rn(x, y, z) < kp.rc2;
}

// FILL = false: cnt[b][i] = number of neighbours; FILL = true: write them at off[b][i]
template <bool FULL, bool PRE, bool FILL>
__global__ void __launch_bounds__(128) k_nbr_warp(KP kp, int *cnt_or_off) {
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, b = blockIdx.y;
    if (i >= kp.N) return;
    const double4_32a *O = kp.pos + (size_t)b * kp.S;
    const double4_32a oi = O[i];
    const int cap = FULL ? kp.fcap : kp.cap;
    int2 *out = (FULL ? reinterpret_cast<int2 *>(kp.fnbr) : kp.pairs) + (size_t)b * cap;
    int o = FILL ? cnt_or_off[(size_t)b * kp.N + i] : 0;
    for (int j0 = FULL ? 0 : i + 1; j0 < kp.N; j0 += 32) {
        const int j = j0 + lane;
        const bool hit = j < kp.N && j != i && oo_test<PRE>(oi, O[j], kp);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (FILL && hit) {
            const int slot = o + __popc(m & ((1u << lane) - 1u));
            if (slot < cap) out[slot] = make_int2(i, j);
        }
        o += __popc(m);
    }
    if (!FILL && lane == 0) cnt_or_off[(size_t)b * kp.N + i] = o;
}

// exclusive scan of per-molecule counts (in place allowed), one block per bead
__global__ void __launch_bounds__(1024) k_scan_counts(int *cnt, int *tot, int N, int cap, unsigned *err) {
    __shared__ int part[1024];
    const int b = blockIdx.x, nt = blockDim.x;
    const int per = (N + nt - 1) / nt, i0 = threadIdx.x * per, i1 = min(N, i0 + per);
    int *c = cnt + (size_t)b * N;
    int s = 0;
    for (int i = i0; i < i1; i++) s += c[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int d = 1; d < nt; d <<= 1) {
        const int v = (threadIdx.x >= d) ? part[threadIdx.x - d] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int base = part[threadIdx.x] - s;
    for (int i = i0; i < i1; i++) {
        const int v = c[i];
        c[i] = base;
        base += v;
    }
    if (threadIdx.x == nt - 1) {
        tot[b] = min(part[nt - 1], cap);
        if (part[nt - 1] > cap) atomicOr(err, 1u);
    }
}

// Boxes of at most NB_MAXN molecules: one block per bead builds the half list (and, with FULL,
// the full list of the mixed engine) in one launch. The bead's O sites are staged in shared
// memory in FP64 and FP32; each warp owns rows, counts both lists with ballots, a block-wide
// exclusive scan turns the counts into row offsets, and a second sweep writes the pairs in the
// reference's order. The FP32 prefilter decides every pair farther than 1e-4 relative from the
// cutoff; the rest are decided by the reference's FP64 arithmetic, so both engines get the
// reference's list bit for bit.
constexpr int NB_MAXN = 1024;

PIMD_D bool oo_test_sm(const float4 &af, const float4 &bf, const double4_32a &a, const double4_32a &b, const KP &kp,
                       float rc2f, const float3 &Lf, const float3 &Lif) {
    const float dx = wrapf_n(af.x - bf.x, Lf.x, Lif.x);
    const float dy = wrapf_n(af.y - bf.y, Lf.y, Lif.y);
    const float dz = wrapf_n(af.z - bf.z, Lf.z, Lif.z);
    const float d2 = dx * dx + dy * dy + dz * dz;
    if (fabsf(d2 - rc2f) > 1e-4f * rc2f + 1e-3f) return d2 < rc2f;
    const double x = min_image_rn(__dsub_rn(a.x, b.x), kp.box[0], kp.boxi[0]);
    const double y = min_image_rn(__dsub_rn(a.y, b.y), kp.box[1], kp.boxi[1]);
    const double z = min_image_rn(__dsub_rn(a.z, b.z), kp.box[2], kp.boxi[2]);
    return dot3_rn(x, y, z) < kp.rc2;
}

// block-wide exclusive scan of v over blockDim.x (a multiple of 32) threads; returns the block total
PIMD_D int block_exscan(int v, int *ex, int *wsum) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < nw ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        wsum[lane] = t;  // inclusive prefix of warp totals
    }
    __syncthreads();
    *ex = x - v + (w > 0 ? wsum[w - 1] : 0);
    const int total = wsum[nw - 1];
    __syncthreads();
    return total;
}

// One bead per thread-block cluster: CTA r of the cluster owns rows [r N / n, (r + 1) N / n) and
// every CTA holds all N O sites in shared memory. Row offsets are the exclusive scan over the
// bead's rows: within a CTA a block scan, across the cluster the totals of the lower-ranked CTAs
// read from their shared memory, so the lists are the same whatever the cluster size.
template <bool FULL>
__global__ void __launch_bounds__(NB_MAXN) k_nbr_block(KP kp) {
    extern __shared__ double4_32a sO[];
    const int ncl = (int)umma::cluster_size(), cr = (int)umma::cluster_rank();
    const int N = kp.N, b = blockIdx.x / ncl;
    const int r0 = cr * N / ncl, r1 = (cr + 1) * N / ncl;
    __shared__ int ctot[2];
    float4 *sf = reinterpret_cast<float4 *>(sO + N);
    int *oh = reinterpret_cast<int *>(sf + N), *of = oh + N;
    // the count pass keeps each row's hit masks (one word per 32 candidates) for the fill pass
    const int nch = (N + 31) / 32;
    unsigned *mk = reinterpret_cast<unsigned *>(of + N);
    __shared__ int wsum[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // the O sites straight from the input positions (atom 3 i; the same values k_sites copies into
    // pos), so that the lists can be built beside k_sites
    const double *Rb = kp.RRt + (size_t)b * kp.natoms * 3;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double4_32a o = make_double4_32a(Rb[9 * i], Rb[9 * i + 1], Rb[9 * i + 2], 0.0);
        sO[i] = o;
        // the FP32 copy is wrapped into the primary box first (in FP64), so its rounding error
        // stays ~1e-7 of the box whatever the magnitude of the input coordinates
        sf[i] = make_float4((float)(o.x - kp.box[0] * round(o.x * kp.boxi[0])), (float)(o.y - kp.box[1] * round(o.y * kp.boxi[1])),
                            (float)(o.z - kp.box[2] * round(o.z * kp.boxi[2])), 0.f);
    }
    const float rc2f = (float)kp.rc2;
    const float3 Lf = make_float3((float)kp.box[0], (float)kp.box[1], (float)kp.box[2]);
    const float3 Lif = make_float3((float)kp.boxi[0], (float)kp.boxi[1], (float)kp.boxi[2]);
    __syncthreads();
    for (int i = r0 + w; i < r1; i += nw) {
        const float4 fi = sf[i];
        const double4_32a di = sO[i];
        int nh = 0, nf = 0;
        for (int j0 = FULL ? 0 : ((i + 1) & ~31); j0 < N; j0 += 32) {
            const int j = j0 + lane;
            const bool hit = j < N && j != i && (FULL || j > i) && oo_test_sm(fi, sf[j], di, sO[j], kp, rc2f, Lf, Lif);
            const unsigned m = __ballot_sync(0xffffffffu, hit), mh = __ballot_sync(0xffffffffu, hit && j > i);
            nf += __popc(m);
            nh += __popc(mh);
            if (lane == 0) mk[(i - r0) * nch + (j0 >> 5)] = m;
        }
        if (lane == 0) {
            oh[i] = nh;
            of[i] = nf;
        }
    }
    __syncthreads();
    // row offsets (this CTA's rows <= blockDim.x: one row per thread), then the lower CTAs' totals
    const int t = threadIdx.x, nrow = r1 - r0;
    int ch = (t < nrow) ? oh[r0 + t] : 0, cf = (t < nrow) ? of[r0 + t] : 0, eh, ef = 0;
    const int toth = block_exscan(ch, &eh, wsum);
    const int totf = FULL ? block_exscan(cf, &ef, wsum) : 0;
    if (t == 0) {
        ctot[0] = toth;
        ctot[1] = totf;
    }
    umma::cluster_barrier();
    int bh = 0, bf = 0;
    for (int c = 0; c < cr; c++) {
        bh += umma::ld_cluster_s32(&ctot[0], (uint32_t)c);
        if (FULL) bf += umma::ld_cluster_s32(&ctot[1], (uint32_t)c);
    }
    umma::cluster_barrier();  // the totals are read before any CTA of the cluster leaves
    if (t < nrow) {
        oh[r0 + t] = bh + eh;
        kp.nbrtmp[(size_t)b * N + r0 + t] = bh + eh;
        if (FULL) {
            of[r0 + t] = bf + ef;
            kp.foff[(size_t)b * N + r0 + t] = bf + ef;
        }
    }
    if (t == 0 && cr == ncl - 1) {
        kp.npair[b] = min(bh + toth, kp.cap);
        if (bh + toth > kp.cap) atomicOr(kp.err, 1u);
        if (FULL) {
            kp.fntot[b] = min(bf + totf, kp.fcap);
            if (bf + totf > kp.fcap) atomicOr(kp.err, 1u);
        }
    }
    __syncthreads();
    int2 *ph = kp.pairs + (size_t)b * kp.cap;
    int2 *pf = reinterpret_cast<int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    for (int i = r0 + w; i < r1; i += nw) {
        int h = oh[i], f = FULL ? of[i] : 0;
        for (int j0 = FULL ? 0 : ((i + 1) & ~31); j0 < N; j0 += 32) {
            const int j = j0 + lane;
            const unsigned m = mk[(i - r0) * nch + (j0 >> 5)];  // the count pass's tests
            const bool hit = (m >> lane) & 1u;
            const int d = i - j0;  // lanes above d have j > i
            const unsigned mh = m & (d < 0 ? 0xffffffffu : (d >= 31 ? 0u : (0xffffffffu << (d + 1))));
            const unsigned below = (1u << lane) - 1u;
            if (hit && j > i) {
                const int slot = h + __popc(mh & below);
                if (slot < kp.cap) ph[slot] = make_int2(i, j);
            }
            if (FULL && hit) {
                const int slot = f + __popc(m & below);
                if (slot < kp.fcap) pf[slot] = make_int2(i, j);
            }
            h += __popc(mh);
            f += __popc(m);
        }
    }
}

// ---------------------------------------------------------------------------------------
// Boxes of more than NB_MAXN molecules with at least 4 cells of width >= Rc per edge: cell lists.
// The O sites of a bead are binned into cells; a warp owns row i, tests the members of the 27
// surrounding cells (FP32 prefilter, FP64 near the cutoff: the same decisions as above), collects
// the hits of the full row in shared memory and sorts them by j (bitonic), so the half and full
// lists written afterwards are the reference's lists bit for bit.
constexpr int CL_ROWCAP = 256;  // neighbours of one molecule in the full list (about 100 at water density and 9 A)

__global__ void __launch_bounds__(128) k_cell_bin(KP kp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (i >= kp.N) return;
    const double4_32a o = kp.pos[(size_t)b * kp.S + i];
    const double x[3] = {o.x, o.y, o.z};
    int c[3];
    float w[3];
    for (int d = 0; d < 3; d++) {
        const double xw = x[d] - kp.box[d] * round(x[d] * kp.boxi[d]);  // in [-L/2, L/2]
        w[d] = (float)xw;
        int ci = (int)floor((xw * kp.boxi[d] + 0.5) * kp.cl_n[d]);
        c[d] = min(max(ci, 0), kp.cl_n[d] - 1);
    }
    const int cell = (c[2] * kp.cl_n[1] + c[1]) * kp.cl_n[0] + c[0];
    kp.cl_mol[(size_t)b * kp.N + i] = cell;
    kp.cl_posf[(size_t)b * kp.N + i] = make_float4(w[0], w[1], w[2], 0.f);
    atomicAdd(kp.cl_cnt + (size_t)b * kp.cl_ncell + cell, 1);
}

// exclusive scan of the cell counts into cell starts, one block per bead; resets the counts
__global__ void __launch_bounds__(1024) k_cell_scan(KP kp) {
    __shared__ int part[1024];
    const int b = blockIdx.x, nt = blockDim.x, nc = kp.cl_ncell;
    const int per = (nc + nt - 1) / nt, c0 = threadIdx.x * per, c1 = min(nc, c0 + per);
    int *cnt = kp.cl_cnt + (size_t)b * nc, *start = kp.cl_start + (size_t)b * (nc + 1);
    int s = 0;
    for (int c = c0; c < c1; c++) s += cnt[c];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int d = 1; d < nt; d <<= 1) {
        const int v = (threadIdx.x >= d) ? part[threadIdx.x - d] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int base = part[threadIdx.x] - s;
    for (int c = c0; c < c1; c++) {
        start[c] = base;
        base += cnt[c];
        cnt[c] = 0;
    }
    if (threadIdx.x == nt - 1) start[nc] = part[nt - 1];
}

__global__ void __launch_bounds__(128) k_cell_fill(KP kp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (i >= kp.N) return;
    const int cell = kp.cl_mol[(size_t)b * kp.N + i];
    const int slot = atomicAdd(kp.cl_cnt + (size_t)b * kp.cl_ncell + cell, 1);
    kp.cl_list[(size_t)b * kp.N + kp.cl_start[(size_t)b * (kp.cl_ncell + 1) + cell] + slot] = i;
}

// warp per (row, bead): sorted full row into cl_row, counts of the half / full rows
template <bool FULL>
__global__ void __launch_bounds__(128) k_cell_rows(KP kp) {
    __shared__ int buf[4][CL_ROWCAP];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, b = blockIdx.y;
    if (i >= kp.N) return;
    int *row = buf[wib];
    const float4 *pf = kp.cl_posf + (size_t)b * kp.N;
    const double4_32a *O = kp.pos + (size_t)b * kp.S;
    const float4 fi = pf[i];
    const double4_32a di = O[i];
    const float rc2f = (float)kp.rc2;
    const float3 Lf = make_float3((float)kp.box[0], (float)kp.box[1], (float)kp.box[2]);
    const float3 Lif = make_float3((float)kp.boxi[0], (float)kp.boxi[1], (float)kp.boxi[2]);
    const int ci = kp.cl_mol[(size_t)b * kp.N + i];
    const int c0 = ci % kp.cl_n[0], c1 = (ci / kp.cl_n[0]) % kp.cl_n[1], c2 = ci / (kp.cl_n[0] * kp.cl_n[1]);
    const int *start = kp.cl_start + (size_t)b * (kp.cl_ncell + 1);
    const int *list = kp.cl_list + (size_t)b * kp.N;
    int n = 0;
    for (int d = 0; d < 27; d++) {
        const int x = (c0 + d % 3 - 1 + kp.cl_n[0]) % kp.cl_n[0];
        const int y = (c1 + (d / 3) % 3 - 1 + kp.cl_n[1]) % kp.cl_n[1];
        const int z = (c2 + d / 9 - 1 + kp.cl_n[2]) % kp.cl_n[2];
        const int cell = (z * kp.cl_n[1] + y) * kp.cl_n[0] + x;
        const int m0 = start[cell], m1 = start[cell + 1];
        for (int m = m0; m < m1; m += 32) {
            const int mm = m + lane;
            const int j = mm < m1 ? list[mm] : -1;
            const bool hit = j >= 0 && j != i && oo_test_sm(fi, pf[max(j, 0)], di, O[max(j, 0)], kp, rc2f, Lf, Lif);
            const unsigned msk = __ballot_sync(0xffffffffu, hit);
            if (hit) {
                const int slot = n + __popc(msk & ((1u << lane) - 1u));
                if (slot < CL_ROWCAP) row[slot] = j;
            }
            n += __popc(msk);
        }
    }
    if (n > CL_ROWCAP) {
        if (lane == 0) atomicOr(kp.err, 1u);
        n = CL_ROWCAP;
    }
    for (int s = n + lane; s < CL_ROWCAP; s += 32) row[s] = 0x7fffffff;
    __syncwarp();
    // bitonic sort of the row (ascending j)
    for (int k = 2; k <= CL_ROWCAP; k <<= 1)
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int t = lane; t < CL_ROWCAP; t += 32) {
                const int p = t ^ jj;
                if (p > t) {
                    const int a = row[t], c = row[p];
                    const bool up = (t & k) == 0;
                    if ((a > c) == up) {
                        row[t] = c;
                        row[p] = a;
                    }
                }
            }
            __syncwarp();
        }
    int nh = 0;
    int *out = kp.cl_row + ((size_t)b * kp.N + i) * CL_ROWCAP;
    for (int s = lane; s < n; s += 32) {
        out[s] = row[s];
        nh += row[s] > i;
    }
    for (int o = 16; o > 0; o >>= 1) nh += __shfl_xor_sync(0xffffffffu, nh, o);
    if (lane == 0) {
        kp.cl_rowlen[(size_t)b * kp.N + i] = n;
        kp.nbrtmp[(size_t)b * kp.N + i] = nh;  // scanned into half-list offsets
        if (FULL) kp.foff[(size_t)b * kp.N + i] = n;
    }
}

// copy the sorted rows into the compact half list (and full list) at the scanned offsets
template <bool FULL>
__global__ void __launch_bounds__(128) k_cell_copy(KP kp) {
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, b = blockIdx.y;
    if (i >= kp.N) return;
    const int *row = kp.cl_row + ((size_t)b * kp.N + i) * CL_ROWCAP;
    const int oh = kp.nbrtmp[(size_t)b * kp.N + i];
    const int of = FULL ? kp.foff[(size_t)b * kp.N + i] : 0;
    const int nf = FULL ? ((i + 1 < kp.N) ? kp.foff[(size_t)b * kp.N + i + 1] : kp.fntot[b]) - of : 0;
    const int nh_end = (i + 1 < kp.N) ? kp.nbrtmp[(size_t)b * kp.N + i + 1] : kp.npair[b];
    const int nh = nh_end - oh;
    // the row's first entry with j > i: the full row minus the half row
    const int n = kp.cl_rowlen[(size_t)b * kp.N + i];
    int2 *ph = kp.pairs + (size_t)b * kp.cap;
    int2 *pfl = reinterpret_cast<int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    for (int s = lane; s < n; s += 32) {
        const int j = row[s];
        const int sh = s - (n - nh);  // the j > i entries are the last nh of the sorted row
        if (sh >= 0 && oh + sh < kp.cap) ph[oh + sh] = make_int2(i, j);
        if (FULL && s < nf && of + s < kp.fcap) pfl[of + s] = make_int2(i, j);
    }
}

template <bool FULL, bool PRE>
static void build_list(Engine &E, int *cnt, int *tot, int cap) {
    KP &kp = E.kp;
    dim3 g((kp.N * 32 + 127) / 128, kp.P);
    k_nbr_warp<FULL, PRE, false><<<g, 128, 0, E.stream>>>(kp, cnt);
    k_scan_counts<<<kp.P, 1024, 0, E.stream>>>(cnt, tot, kp.N, cap, kp.err);
    k_nbr_warp<FULL, PRE, true><<<g, 128, 0, E.stream>>>(kp, cnt);
    E.nlaunch += 3;
}

// half list for every engine; the mixed engine adds the full list (row offsets in foff)
// whether launch_neighbors builds the lists from the input positions alone (the one-launch
// block path; the cell-list path reads the site array k_sites writes)
bool nbr_from_inputs(const Engine &E) {
    return !(E.kp.N > NB_MAXN && E.kp.cl_ncell > 0 && E.nbr_cells) && E.kp.N <= NB_MAXN && E.nbr_block;
}

void launch_neighbors(Engine &E) {
    KP &kp = E.kp;
    if (kp.N > NB_MAXN && kp.cl_ncell > 0 && E.nbr_cells) {
        const bool full = E.precision == PIMD_PREC_MIXED;
        cudaMemsetAsync(kp.cl_cnt, 0, sizeof(int) * (size_t)kp.P * kp.cl_ncell, E.stream);
        dim3 g1((kp.N + 127) / 128, kp.P), gw((kp.N * 32 + 127) / 128, kp.P);
        k_cell_bin<<<g1, 128, 0, E.stream>>>(kp);
        k_cell_scan<<<kp.P, 1024, 0, E.stream>>>(kp);
        k_cell_fill<<<g1, 128, 0, E.stream>>>(kp);
        if (full)
            k_cell_rows<true><<<gw, 128, 0, E.stream>>>(kp);
        else
            k_cell_rows<false><<<gw, 128, 0, E.stream>>>(kp);
        k_scan_counts<<<kp.P, 1024, 0, E.stream>>>(kp.nbrtmp, kp.npair, kp.N, kp.cap, kp.err);
        if (full) k_scan_counts<<<kp.P, 1024, 0, E.stream>>>(kp.foff, kp.fntot, kp.N, kp.fcap, kp.err);
        if (full)
            k_cell_copy<true><<<gw, 128, 0, E.stream>>>(kp);
        else
            k_cell_copy<false><<<gw, 128, 0, E.stream>>>(kp);
        E.nlaunch += full ? 7 : 6;
        return;
    }
    if (kp.N <= NB_MAXN && E.nbr_block) {
        const int nt = ((kp.N + 31) / 32) * 32 < 256 ? 256 : ((kp.N + 31) / 32) * 32;
        size_t smem = (sizeof(double4_32a) + sizeof(float4) + 2 * sizeof(int)) * (size_t)kp.N;
        // a cluster of up to 4 CTAs per bead so that the beads cover the GPU
        static int nsm_cache[64] = {0};
        int &nsm = nsm_cache[E.device & 63];
        if (!nsm) {
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, E.device);
            if (nsm <= 0) nsm = 152;
        }
        const int ncl = std::max(1, std::min(4, std::min(nsm / std::max(kp.P, 1), kp.N / 32)));
        // + the hit masks of a CTA's rows (at most 128 KB at N = 1024 in one CTA)
        smem += sizeof(unsigned) * (size_t)((kp.N + ncl - 1) / ncl + 1) * ((kp.N + 31) / 32);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(ncl * kp.P);
        cfg.blockDim = dim3(nt);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = E.stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = ncl;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (E.precision == PIMD_PREC_MIXED)
            cudaLaunchKernelEx(&cfg, k_nbr_block<true>, kp);
        else
            cudaLaunchKernelEx(&cfg, k_nbr_block<false>, kp);
        ++E.nlaunch;
        return;
    }
    if (E.precision == PIMD_PREC_MIXED) {
        build_list<false, true>(E, kp.nbrtmp, kp.npair, kp.cap);
        build_list<true, true>(E, kp.foff, kp.fntot, kp.fcap);
    } else {
        build_list<false, false>(E, kp.nbrtmp, kp.npair, kp.cap);
    }
}

}  // namespace pimd

namespace pimd {
void neighbors_init(Engine &E) {
    (void)E;
    cudaFuncSetAttribute(k_nbr_block<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_nbr_block<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}
}  // namespace pimd
