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
        double *a = kp.acc + (size_t)b * NACC;
        if (a[ACC_CONV] == 0.0) {
            const double dd = kp.stath * sqrt(a[ACC_DSQ]);
            a[ACC_UIND] = -0.5 * a[ACC_MUEFQ];
            a[ACC_NITER] = (double)iter;
            a[ACC_DELTADIP] = dd;
            if (dd < eps || iter >= kp.polar_maxiter) a[ACC_CONV] = (dd < eps) ? 1.0 : 2.0;
            a[ACC_DSQ] = 0.0;
            a[ACC_MUEFQ] = 0.0;
        }
        if (a[ACC_CONV] != 0.0) atomicAdd(&nconv, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *kp.allconv = (nconv == kp.P) ? 1 : 0;
        kp.dstep[1] = iter;
        if (kp.cond) cudaGraphSetConditional(kp.cond, nconv == kp.P ? 0u : 1u);
    }
}

}  // namespace pimd
