// dipole_check.cuh -- the induced-dipole convergence test of one iteration, for all beads, run
// by one thread block (pot_ttm.f90:379-385).
#pragma once
#include "engine.h"

namespace pimd {

// Per bead: stath * |dmu| against polar_eps, Uind = -1/2 sum mu . Efq, iteration count; a bead
// is done at convergence (1) or at polar_maxiter (2). The iteration number comes from the
// device step word, which this advances; inside a CUDA graph it also sets the conditional of
// the dipole loop (continue while some bead is not done).
PIMD_D void dd_check_block(const KP &kp, double eps) {
    __shared__ int nconv;
    const int iter = kp.dstep[1] + 1;
    if (threadIdx.x == 0) nconv = 0;
    __syncthreads();
    for (int b = threadIdx.x; b < kp.P; b += blockDim.x) {
        // the sums arrived by atomics from other blocks: read through L2
        double *a = kp.acc + (size_t)b * NACC;
        if (__ldcg(a + ACC_CONV) == 0.0) {
            const double dd = kp.stath * sqrt(__ldcg(a + ACC_DSQ));
            a[ACC_UIND] = -0.5 * __ldcg(a + ACC_MUEFQ);
            a[ACC_NITER] = (double)iter;
            a[ACC_DELTADIP] = dd;
            if (dd < eps || iter >= kp.polar_maxiter) a[ACC_CONV] = (dd < eps) ? 1.0 : 2.0;
            a[ACC_DSQ] = 0.0;
            a[ACC_MUEFQ] = 0.0;
        }
        if (__ldcg(a + ACC_CONV) != 0.0) atomicAdd(&nconv, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *kp.allconv = (nconv == kp.P) ? 1 : 0;
        kp.dstep[1] = iter;
        if (kp.cond) cudaGraphSetConditional(kp.cond, nconv == kp.P ? 0u : 1u);
    }
}

// The FP64 inputs of one dipole site's SOR update (fetched early by callers that can hide the
// latency).
struct DdSite {
    double mu[3], efq[3], efdr[3], pol;
};
PIMD_D void dd_sor_load(const KP &kp, int b, int s, DdSite &d) {
    const size_t gs = (size_t)b * kp.S + s;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        d.mu[c] = kp.dip[3 * gs + c];
        // written by another kernel of the iteration when the real-space field is asynchronous:
        // read through L2 (the L1 of this SM may hold an older line)
        d.efdr[c] = kp.dd_async ? __ldcg(kp.Efdr + 3 * gs + c) : kp.Efdr[3 * gs + c];
    }
    const double4_32a f = kp.F[gs];
    d.efq[0] = f.x;
    d.efq[1] = f.y;
    d.efq[2] = f.z;
    d.pol = kp.polar_sor * kp.polar[s / kp.N + 1];
}
// pot_ttm.f90:371-381: Efd = Efd_real + Efd_rec + Efq + factor mu and the SOR update (FP64) of
// the dipole at site s of bead b, with E this iteration's reciprocal field at the site;
// av += (|mu_new - mu|^2 (|mu_new|^2 on the first iteration), mu_new . Efq).
PIMD_D void dd_sor_apply(const KP &kp, int b, int s, const DdSite &d, const double (&E)[3], int iter, double (&av)[2]) {
    const size_t gs = (size_t)b * kp.S + s;
    double mn[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const double efd = (d.efdr[c] + E[c]) + d.efq[c] + kp.factor * d.mu[c];
        mn[c] = (1.0 - kp.polar_sor) * d.mu[c] + d.pol * efd;
        const double dd = (iter == 1) ? mn[c] : mn[c] - d.mu[c];
        av[0] += dd * dd;
        av[1] += mn[c] * d.efq[c];
        kp.dip[3 * gs + c] = mn[c];
        kp.Efdr[3 * gs + c] = 0.0;
    }
    const float4 mf = make_float4((float)mn[0], (float)mn[1], (float)mn[2], 0.f);
    if (kp.dipf) dipf_next(kp)[gs] = mf;
    if (!kp.dd_async) mrec_dipole(kp, b, s, mf);  // (the asynchronous gather reads the buffers)
}
PIMD_D void dd_sor_site(const KP &kp, int b, int s, const double (&E)[3], int iter, double (&av)[2]) {
    DdSite d;
    dd_sor_load(kp, b, s, d);
    dd_sor_apply(kp, b, s, d, E, iter, av);
}

// End of a dipole-update block: its sums go into the bead's acc[ACC_DSQ], acc[ACC_MUEFQ] (when
// add), then the block counts itself and the last block of the launch runs the convergence
// test (a device counter, reset by that block). With total, the count to reach is total (units
// of the asynchronous protocol below) instead of the launch's blocks. Every thread of every
// block of the launch calls this exactly once; blocks of converged beads call it with add =
// false. Only the first NWA warps may hold nonzero sums (the others skip the FP64 shuffles; the
// totals are unchanged).
template <int NT, int NWA = NT / 32>
PIMD_D void dd_block_end(const KP &kp, int b, const double (&av)[2], bool add, unsigned total = 0u) {
    if (add) {
        __shared__ double red[NWA][2];
        const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
        if (wp < NWA) {
#pragma unroll
            for (int i = 0; i < 2; i++) {
                double x = av[i];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                if (lane == 0) red[wp][i] = x;
            }
        }
        __syncthreads();
        if (threadIdx.x < 2) {
            double t = 0;
            for (int w = 0; w < NWA; w++) t += red[w][threadIdx.x];
            atomicAdd(kp.acc + (size_t)b * NACC + ACC_DSQ + threadIdx.x, t);
        }
    }
    if (kp.fin_counter) {
        __shared__ bool last;
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();  // this block's sums are visible before it counts
            last = atomicAdd(kp.fin_counter, 1u) == (total ? total : gridDim.x * gridDim.y) - 1;
        }
        __syncthreads();
        if (last) {
            __threadfence();
            dd_check_block(kp, kp.polar_eps);
            if (threadIdx.x == 0) *kp.fin_counter = 0u;
        }
    }
}

// ---------------------------------------------------------------------------------------
// The asynchronous real-space field (kp.dd_async; TTM3-F, whose dipole sites are the M sites
// fd + i of the molecules i): the tensor-core field pass (one CTA per unit of 128 sites from
// kp.unit_sbase) and k_dd_real_m (blocks of 4 molecules) run at the same time. Each stores its
// field (kp.Erec, kp.Efdr), then arrives at the counters of the units it covers; the one that
// arrives last at a unit runs that unit's SOR update and block end. Nothing waits: an arrival
// is one atomic add, and the protocol is the classic last-block pattern.

// arrivals a unit expects: its field-pass CTA and every k_dd_real_m block of its molecules
PIMD_D unsigned dd_unit_expected(const KP &kp, int t) {
    const int s0 = kp.unit_sbase + 128 * t;
    const int lo = max(0, s0 - kp.fd), hi = min(kp.N, s0 + 128 - kp.fd);
    return 1u + (hi > lo ? (unsigned)((hi - 1) / 4 - lo / 4 + 1) : 0u);
}

// Block-wide (every thread calls): count this block's arrival at unit (b, t); true in every
// thread when it was the last, after which the other arrivals' stores are visible.
PIMD_D bool dd_unit_arrive(const KP &kp, int b, int t) {
    __shared__ int last_sh;
    __threadfence();  // this thread's field stores are visible before the block counts
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned *c = kp.unit_cnt + (size_t)b * kp.nunits + t;
        const bool last = atomicAdd(c, 1u) == dd_unit_expected(kp, t) - 1u;
        if (last) atomicExch(c, 0u);  // every arrival of this iteration is counted
        last_sh = last;
    }
    __syncthreads();
    const bool last = last_sh != 0;
    if (last) __threadfence();
    return last;
}

// The SOR update of unit (b, t) by its last arrival, NT threads, then the unit's block end.
// Sites without a value in Ereg (the field pass's own sites hold theirs in registers) read the
// reciprocal field from kp.Erec.
template <int NT>
PIMD_D void dd_unit_sor(const KP &kp, int b, int t, bool have_reg, const float (&Ereg)[3]) {
    const bool conv = bead_converged(kp, b);
    const int iter = kp.dstep[1] + 1;
    double av[2] = {0.0, 0.0};
    if (!conv) {
        for (int u = threadIdx.x; u < 128; u += NT) {
            const int s = kp.unit_sbase + 128 * t + u;
            if (s < kp.fd || s >= kp.ld) continue;
            DdSite d;
            dd_sor_load(kp, b, s, d);
            double E[3];
            if (have_reg && u == (int)threadIdx.x) {
                E[0] = (double)Ereg[0], E[1] = (double)Ereg[1], E[2] = (double)Ereg[2];
            } else {
                const float4 e = __ldcg(kp.Erec + (size_t)b * kp.S + s);
                E[0] = (double)e.x, E[1] = (double)e.y, E[2] = (double)e.z;
            }
            dd_sor_apply(kp, b, s, d, E, iter, av);
        }
    }
    dd_block_end<NT, (NT < 128 ? NT : 128) / 32>(kp, b, av, !conv, (unsigned)(kp.P * kp.nunits));
}

}  // namespace pimd
