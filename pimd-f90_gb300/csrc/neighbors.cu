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

template <bool FULL, bool PRE>
static void build_list(Engine &E, int *cnt, int *tot, int cap) {
    KP &kp = E.kp;
    dim3 g((kp.N * 32 + 127) / 128, kp.P);
    k_nbr_warp<FULL, PRE, false><<<g, 128, 0, E.stream>>>(kp, cnt);
    k_scan_counts<<<kp.P, 1024, 0, E.stream>>>(cnt, tot, kp.N, cap, kp.err);
    k_nbr_warp<FULL, PRE, true><<<g, 128, 0, E.stream>>>(kp, cnt);
    E.nlaunch += 3;
}

// half list for every engine; the mixed engine adds the full list (counts kept in fcnt,
// offsets in foff)
void launch_neighbors(Engine &E) {
    KP &kp = E.kp;
    if (E.precision == PIMD_PREC_MIXED) {
        build_list<false, true>(E, kp.nbrtmp, kp.npair, kp.cap);
        build_list<true, true>(E, kp.foff, kp.fntot, kp.fcap);
    } else {
        build_list<false, false>(E, kp.nbrtmp, kp.npair, kp.cap);
    }
}

}  // namespace pimd
