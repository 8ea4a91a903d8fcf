// neighbors.cu -- O-O neighbour lists of all beads (find_neigh.f90:171-277).
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

namespace pimd {

PIMD_D float wrapf_n(float v, float L, float Li) { return v - L * rintf(v * Li); }

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

template <bool FULL>
__global__ void __launch_bounds__(NB_MAXN) k_nbr_block(KP kp) {
    extern __shared__ double4_32a sO[];
    const int N = kp.N, b = blockIdx.x;
    float4 *sf = reinterpret_cast<float4 *>(sO + N);
    int *oh = reinterpret_cast<int *>(sf + N), *of = oh + N;
    __shared__ int wsum[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const double4_32a *O = kp.pos + (size_t)b * kp.S;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double4_32a o = O[i];
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
    for (int i = w; i < N; i += nw) {
        const float4 fi = sf[i];
        const double4_32a di = sO[i];
        int nh = 0, nf = 0;
        for (int j0 = FULL ? 0 : ((i + 1) & ~31); j0 < N; j0 += 32) {
            const int j = j0 + lane;
            const bool hit = j < N && j != i && (FULL || j > i) && oo_test_sm(fi, sf[j], di, sO[j], kp, rc2f, Lf, Lif);
            const unsigned m = __ballot_sync(0xffffffffu, hit), mh = __ballot_sync(0xffffffffu, hit && j > i);
            nf += __popc(m);
            nh += __popc(mh);
        }
        if (lane == 0) {
            oh[i] = nh;
            of[i] = nf;
        }
    }
    __syncthreads();
    // row offsets (N <= blockDim.x: one row per thread)
    const int t = threadIdx.x;
    int ch = (t < N) ? oh[t] : 0, cf = (t < N) ? of[t] : 0, eh, ef;
    const int toth = block_exscan(ch, &eh, wsum);
    const int totf = FULL ? block_exscan(cf, &ef, wsum) : 0;
    if (t < N) {
        oh[t] = eh;
        kp.nbrtmp[(size_t)b * N + t] = eh;
        if (FULL) {
            of[t] = ef;
            kp.foff[(size_t)b * N + t] = ef;
        }
    }
    if (t == 0) {
        kp.npair[b] = min(toth, kp.cap);
        if (toth > kp.cap) atomicOr(kp.err, 1u);
        if (FULL) {
            kp.fntot[b] = min(totf, kp.fcap);
            if (totf > kp.fcap) atomicOr(kp.err, 1u);
        }
    }
    __syncthreads();
    int2 *ph = kp.pairs + (size_t)b * kp.cap;
    int2 *pf = reinterpret_cast<int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
    for (int i = w; i < N; i += nw) {
        const float4 fi = sf[i];
        const double4_32a di = sO[i];
        int h = oh[i], f = FULL ? of[i] : 0;
        for (int j0 = FULL ? 0 : ((i + 1) & ~31); j0 < N; j0 += 32) {
            const int j = j0 + lane;
            const bool hit = j < N && j != i && (FULL || j > i) && oo_test_sm(fi, sf[j], di, sO[j], kp, rc2f, Lf, Lif);
            const unsigned m = __ballot_sync(0xffffffffu, hit), mh = __ballot_sync(0xffffffffu, hit && j > i);
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
void launch_neighbors(Engine &E) {
    KP &kp = E.kp;
    if (kp.N <= NB_MAXN && E.nbr_block) {
        const int nt = ((kp.N + 31) / 32) * 32 < 256 ? 256 : ((kp.N + 31) / 32) * 32;
        const size_t smem = (sizeof(double4_32a) + sizeof(float4) + 2 * sizeof(int)) * (size_t)kp.N;
        if (E.precision == PIMD_PREC_MIXED)
            k_nbr_block<true><<<kp.P, nt, smem, E.stream>>>(kp);
        else
            k_nbr_block<false><<<kp.P, nt, smem, E.stream>>>(kp);
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
    cudaFuncSetAttribute(k_nbr_block<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    cudaFuncSetAttribute(k_nbr_block<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
}
}  // namespace pimd
