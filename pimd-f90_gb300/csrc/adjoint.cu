// adjoint.cu -- differentiation form of the TTM3-F force call (FP64 and mixed engines).
//
// The energy of bead b as the forward computes it (pot_ttm.f90:3-630) is
//   E = Umon(theta) + Uvdw(theta) + Uelec + Uind + Uvdw_lrc,   Uind = -1/2 mu_K . E_q
// with mu_K the dipoles after K_b Jacobi-SOR iterations (pot_ttm.f90:298-390):
//   mu_0 = alpha E_q,   mu_k = (1 - w) mu_{k-1} + w alpha (D mu_{k-1} + E_q),   k = 1..K_b,
// D = T_real + T_recip + f I the symmetric dipole-field operator. The backward differentiates
// exactly this computation: g_K = dE/dmu_K = -1/2 E_q, then for k = K..1 the transposed
// iteration g_{k-1} = (1 - w) g_k + w D(alpha g_k) -- the same operator D, applied by the
// forward's own field kernels -- while collecting
//   d/dx    w (alpha g_k)^T (dD/dx) mu_{k-1}           (bilinear real and reciprocal terms)
//   d/dE_q  nu = -1/2 mu_K + alpha (w sum_k g_k + g_0)   (the adjoint of the charge field)
//   d/dalpha, d/da_dd from the same terms.
// nu then enters like a dipole set in the charge-field derivative (real, intramolecular and
// reciprocal), and its potential at the charge sites joins the charge potential in the chain
// through the DMS charges (grdq) and the M-site construction. Pair geometry is recomputed from
// the site positions, never stored. The forward records mu_0..mu_K and the structure factor of
// each iteration's dipoles (the tape) and the charge-only potential; nothing else is kept beyond
// the forward's own buffers.
// On the mixed engine the reverse sweep's operators are the forward's: D_real from its per-entry
// smear scalars with alpha g_k in the molecule records; the reciprocal passes on the tensor cores
// (structure factor, charge-field pass on moved weights, and the force pass's dipole half for the
// bilinear term), or on the FP32 pipe without them; the bilinear real-space term and the
// charge-field pair terms as full-list FP32 gathers (no atomics); sums in FP64 as in the forward.
// The monomer chain runs once, in FP64, on the forward's FP64 sites.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "engine.h"
#include "nasa.cuh"

namespace pimd {
int run_forces(Engine &E, int t, int check_every, double *Upott, double *virialt, double *virialct, double *virt9);

__constant__ double c_nasa4[4][245];  // C5ZA, CBASIS, CCORE, CREST (nasa_mod.f90)

// ---------------------------------------------------------------------------------------
// theta -> the derived parameters of the context (potential.f90:97-113, 152-160)
int apply_theta(Engine &E) {
    KP &kp = E.kp;
    const double *th = E.theta;
    kp.polar[4] = th[PIMD_TH_POLAR_M];
    for (int i = 1; i <= 4; i++)
        for (int j = 1; j <= 4; j++) {
            kp.pt.apol_qq[i][j] = (th[PIMD_TH_A_CC] * E.polfac[i]) * E.polfac[j];
            kp.pt.ra_qq[i][j] = std::pow(kp.pt.apol_qq[i][j], 1.0 / 3.0);
            kp.pt.apol_dd[i][j] = (th[PIMD_TH_A_DD] * E.polfac[i]) * E.polfac[j];
            kp.pt.apol_cd[i][j] = (th[PIMD_TH_A_CC] * E.polfac[i]) * E.polfac[j];
        }
    kp.same_acd = std::fabs(th[PIMD_TH_A_CC] - th[PIMD_TH_A_DD]) < 1.e-12 ? 1 : 0;
    kp.vdwC = th[PIMD_TH_VDW_C];
    kp.vdwD = th[PIMD_TH_VDW_D];
    kp.vdwE = th[PIMD_TH_VDW_E];
    kp_float_tables(kp);
    kp.dms1 = th[PIMD_TH_DMS1];
    kp.dms2 = th[PIMD_TH_DMS2];
    kp.dms3 = th[PIMD_TH_DMS3];
    kp.gammaM = th[PIMD_TH_GAMMA_M];
    {
        const double Rc = E.rc, r3 = Rc * Rc * Rc, r7 = r3 * r3 * Rc, r9 = r7 * Rc * Rc;
        kp.Uvdw_lrc = TWOPI * (double)(kp.N * kp.N) / kp.volume *
                      (E.vdwA_model / (9.0 * r9) + E.vdwB_model / (7.0 * r7) + kp.vdwC / (3.0 * r3));
    }
    const bool published = th[PIMD_TH_F5Z] == PIMD_NASA_F5Z && th[PIMD_TH_FBASIS] == PIMD_NASA_FBASIS &&
                           th[PIMD_TH_FCORE] == PIMD_NASA_FCORE && th[PIMD_TH_FREST] == PIMD_NASA_FREST;
    kp.nasa_f5z = th[PIMD_TH_F5Z];
    if (published) {
        kp.c5z = nullptr;
    } else {
        if (!E.d_c5z) {
            if (cudaMalloc((void **)&E.d_c5z, sizeof(double) * 245) != cudaSuccess) return PIMD_ERR_NOMEM;
            E.allocs.push_back(E.d_c5z);
        }
        double c5z[245];
        for (int j = 0; j < 245; j++)
            c5z[j] = th[PIMD_TH_F5Z] * PIMD_NASA_C5ZA[j] + th[PIMD_TH_FBASIS] * PIMD_NASA_CBASIS[j] +
                     th[PIMD_TH_FCORE] * PIMD_NASA_CCORE[j] + th[PIMD_TH_FREST] * PIMD_NASA_CREST[j];
        cudaMemcpy(E.d_c5z, c5z, sizeof(c5z), cudaMemcpyHostToDevice);
        kp.c5z = E.d_c5z;
    }
    return cudaGetLastError() == cudaSuccess ? PIMD_OK : PIMD_ERR_CUDA;
}

// ---------------------------------------------------------------------------------------
// tape: mu_iter of the dipole sites, (iteration 0) the charge-only potential, and (iteration
// iter >= 1) the structure factor that iteration formed from mu_{iter-1} (kp.Sm, unchanged in
// beads already converged, which the backward does not read at that iteration)
__global__ void k_tape(KP kp, double *tape, double *phiq, double2 *tapeS, int iter) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    const int nd = kp.ld - kp.fd;
    if (t < nd)
        for (int c = 0; c < 3; c++)
            tape[(((size_t)iter * kp.P + b) * nd + t) * 3 + c] = kp.dip[3 * ((size_t)b * kp.S + kp.fd + t) + c];
    if (iter == 0 && t < kp.S) phiq[(size_t)b * kp.S + t] = kp.F[(size_t)b * kp.S + t].w;
    if (iter >= 1)
        for (int k = t; k < kp.nk; k += gridDim.x * blockDim.x)
            tapeS[((size_t)(iter - 1) * kp.P + b) * kp.nk + k] = kp.Sm[(size_t)b * kp.nk + k];
}

void tape_record(Engine &E, int iter) {
    if (!E.d_tape || iter > E.tape_kmax) return;
    dim3 g((E.kp.S + 127) / 128, E.kp.P);
    k_tape<<<g, 128, 0, E.stream>>>(E.kp, E.d_tape, E.d_phiq, E.d_tapeS, iter);
    ++E.nlaunch;
}

// ---------------------------------------------------------------------------------------
// backward kernels; nd = dipole sites per bead, dipole site s = fd + i

__global__ void __launch_bounds__(128) k_adj_init(KP kp, const double *ebar, double *g, double *nu) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, nd = kp.ld - kp.fd;
    if (i >= nd) return;
    const size_t gs = (size_t)b * kp.S + kp.fd + i;
    const double4_32a F = kp.F[gs];
    const double eq[3] = {F.x, F.y, F.z};
    for (int c = 0; c < 3; c++) {
        g[((size_t)b * nd + i) * 3 + c] = -0.5 * ebar[b] * eq[c];  // dE/dmu_K of -1/2 mu_K . E_q
        nu[3 * gs + c] = -0.5 * ebar[b] * kp.dip[3 * gs + c];       // dE/dE_q of the same term
    }
}

// iteration k of the reverse sweep, first half: u = alpha g_k, v = mu_{k-1}, nu += w u, and
// d/dalpha of mu_k = (1-w) mu_{k-1} + w alpha F_k, with w alpha F_k = mu_k - (1-w) mu_{k-1}.
// Mixed engine (uf, vf given, float4 [P][S]; TTM3-F, dipole site fd + i of molecule i): FP32
// copies of u and v, and u in the molecule records, where the real-space field reads its dipoles.
__global__ void __launch_bounds__(128) k_adj_u(KP kp, int k, const int *iters, const double *tape, const double *g,
                                               double *u, double *v, double *nu, double *bacc, double *bw,
                                               double *thacc, double omega, float4 *uf, float4 *vf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, nd = kp.ld - kp.fd;
    const bool active = k <= iters[b];
    const double alpha = kp.polar[4];
    if (i == 0) {
        bacc[(size_t)b * NACC + ACC_CONV] = active ? 0.0 : 1.0;
        bw[b] = active ? omega : 0.0;
    }
    double th[1] = {0.0};
    if (i < nd) {
        const size_t gs = (size_t)b * kp.S + kp.fd + i;
        double uu[3] = {0.0, 0.0, 0.0}, vv[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < 3; c++) {
            const double gi = g[((size_t)b * nd + i) * 3 + c];
            if (active) {
                const double mk = tape[(((size_t)k * kp.P + b) * nd + i) * 3 + c];
                const double mp = tape[(((size_t)(k - 1) * kp.P + b) * nd + i) * 3 + c];
                uu[c] = alpha * gi;
                vv[c] = mp;
                nu[3 * gs + c] += omega * alpha * gi;
                th[0] += gi * (mk - (1.0 - omega) * mp) / alpha;
            }
            u[3 * gs + c] = uu[c];
            v[3 * gs + c] = vv[c];
        }
        if (uf) {
            const float4 u4 = make_float4((float)uu[0], (float)uu[1], (float)uu[2], 0.f);
            uf[gs] = u4;
            vf[gs] = make_float4((float)vv[0], (float)vv[1], (float)vv[2], 0.f);
            mrec_dipole(kp, b, kp.fd + i, u4);
        }
    }
    block_reduce_add<1, 128>(th, thacc + PIMD_TH_POLAR_M);
}

// second half: g_{k-1} = (1-w) g_k + w (D u + f u), D u accumulated in Dr by the field kernels.
// Mixed engine with the tensor-core sweep (Erec given): the reciprocal part of D u is in Erec
// (kp.Fx, x y z), and dDg (kp.dR) holds the two dipole-force passes of the reciprocal bilinear
// term, grad -= w_b dDg at the dipole sites.
__global__ void __launch_bounds__(128) k_adj_g(KP kp, int k, const int *iters, double *g, const double *u,
                                               const double *Dr, double omega, const double4_32a *Erec,
                                               const double *dDg, const double *bw, double *grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, nd = kp.ld - kp.fd;
    if (i >= nd || k > iters[b]) return;
    const size_t gs = (size_t)b * kp.S + kp.fd + i;
    double er[3] = {0.0, 0.0, 0.0};
    if (Erec) {
        const double4_32a x = Erec[gs];
        er[0] = x.x, er[1] = x.y, er[2] = x.z;
    }
    for (int c = 0; c < 3; c++) {
        double &gi = g[((size_t)b * nd + i) * 3 + c];
        gi = (1.0 - omega) * gi + omega * ((Dr[3 * gs + c] + er[c]) + kp.factor * u[3 * gs + c]);
    }
    if (dDg)
        for (int c = 0; c < 3; c++) grad[3 * gs + c] -= bw[b] * dDg[3 * gs + c];
}

// Weight slots of the tensor-core sweep (FP32 4 pi A_k / V conj(S) in the field passes' form):
// MODE 0: slot 0 <- slot 1 (the structure factor just formed), slot 1 <- 0; MODE 1: slot 0 <-
// the weights of Sm (the forward's structure factor of mu_{k-1}, from the tape), slot 1 stays 0.
// MODE 2: slot 0 <- the weights of S (the raw charge structure factor), slot 1 <- 0.
template <int MODE>
__global__ void __launch_bounds__(256) k_adj_wslots(KP kp, const double2 *Sm) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (k >= kp.nk) return;
    float2 *w0 = kp.Wf + (size_t)b * 2 * kp.nk, *w1 = w0 + kp.nk;
    if (MODE == 0) {
        w0[k] = w1[k];
        w1[k] = make_float2(0.f, 0.f);
    } else {
        const double w = kp.kinfo[k].w;
        const double2 a = Sm[(size_t)b * kp.nk + k];
        w0[k] = make_float2((float)(w * a.x), (float)(-w * a.y));
        if (MODE == 2) w1[k] = make_float2(0.f, 0.f);
    }
}

// mu_0 = alpha E_q: nu += alpha g_0, d/dalpha += g_0 . E_q
// (nuf given: an FP32 copy of nu at the dipole sites, for the tensor-core cross term)
__global__ void __launch_bounds__(128) k_adj_final(KP kp, const double *g, double *nu, double *thacc, float4 *nuf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, nd = kp.ld - kp.fd;
    double th[1] = {0.0};
    if (i < nd) {
        const size_t gs = (size_t)b * kp.S + kp.fd + i;
        const double4_32a F = kp.F[gs];
        const double eq[3] = {F.x, F.y, F.z};
        double n[3];
        for (int c = 0; c < 3; c++) {
            const double gi = g[((size_t)b * nd + i) * 3 + c];
            n[c] = nu[3 * gs + c] + kp.polar[4] * gi;
            nu[3 * gs + c] = n[c];
            th[0] += gi * eq[c];
        }
        if (nuf) nuf[gs] = make_float4((float)n[0], (float)n[1], (float)n[2], 0.f);
    }
    block_reduce_add<1, 128>(th, thacc + PIMD_TH_POLAR_M);
}

// The reciprocal cross term of the charge-field adjoint from the tensor-core passes:
// d/dx [nu^T E_q,rec] is q_s E_nu(s) at the charged sites (E_nu, phi_nu: the force pass's charge
// half on the weights of S_nu, Fx = (-q E_nu, phi_nu)) with -phi_nu(s) its derivative in q_s,
// plus the derivative at the dipole sites of nu . E_q at fixed S_q, minus the force pass's
// dipole half of nu on the charge weights (in dR).
__global__ void __launch_bounds__(128) k_adj_cross_fold(KP kp, int s0, double *grad, double *phin) {
    const int s = s0 + blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (s >= kp.S) return;
    const size_t gs = (size_t)b * kp.S + s;
    const double4_32a x = kp.Fx[gs];
    grad[3 * gs + 0] -= x.x;
    grad[3 * gs + 1] -= x.y;
    grad[3 * gs + 2] -= x.z;
    phin[gs] -= x.w;
    if (s >= kp.fd && s < kp.ld)
        for (int c = 0; c < 3; c++) grad[3 * gs + c] -= kp.dR[3 * gs + c];
}

// the forward's site-pair vector between site kinds isp of i and jsp of j (pot_ttm.f90:318-319)
PIMD_D void pair_vec(const KP &kp, const double4_32a &Oi, const double4_32a &Oj, const double4_32a &a,
                     const double4_32a &c, double Rs[3]) {
    const double Rij[3] = {min_image_rn(__dsub_rn(Oi.x, Oj.x), kp.box[0], kp.boxi[0]),
                           min_image_rn(__dsub_rn(Oi.y, Oj.y), kp.box[1], kp.boxi[1]),
                           min_image_rn(__dsub_rn(Oi.z, Oj.z), kp.box[2], kp.boxi[2])};
    const double Rij0[3] = {__dadd_rn(__dsub_rn(Rij[0], Oi.x), Oj.x), __dadd_rn(__dsub_rn(Rij[1], Oi.y), Oj.y),
                            __dadd_rn(__dsub_rn(Rij[2], Oi.z), Oj.z)};
    Rs[0] = min_image_rn(__dsub_rn(__dadd_rn(a.x, Rij0[0]), c.x), kp.box[0], kp.boxi[0]);
    Rs[1] = min_image_rn(__dsub_rn(__dadd_rn(a.y, Rij0[1]), c.y), kp.box[1], kp.boxi[1]);
    Rs[2] = min_image_rn(__dsub_rn(__dadd_rn(a.z, Rij0[2]), c.z), kp.box[2], kp.boxi[2]);
}

PIMD_D void atomic3(double *p, const double v[3], double s) {
    atomicAdd(p, s * v[0]);
    atomicAdd(p + 1, s * v[1]);
    atomicAdd(p + 2, s * v[2]);
}

struct Polfac {
    double v[5];  // polfac per site kind 1..4 (the Thole a12 = a polfac_i polfac_j)
};

// bilinear real-space term w u^T (dT/dx) v over the M-M pairs (Thole dipole tensor, smear3),
// and its d/da_dd (dT/da12 = 3 a12 r e^{-a12 r^3} R R^T - e^{-a12 r^3} I for r^2 < 25)
__global__ void __launch_bounds__(128) k_adj_ddbil(KP kp, Polfac pf, const double *u, const double *v,
                                                   const double *bw, double *grad, double *thacc) {
    const int b = blockIdx.y, N = kp.N;
    double th[1] = {0.0};
    const double w = bw[b];
    if (w != 0.0) {
        const int np = kp.npair[b];
        const double4_32a *pos = kp.pos + (size_t)b * kp.S;
        const double a12 = kp.pt.apol_dd[4][4];
        for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
            const int2 ij = kp.pairs[(size_t)b * kp.cap + p];
            const int i = ij.x, j = ij.y;
            double Rs[3];
            pair_vec(kp, pos[i], pos[j], pos[3 * N + i], pos[3 * N + j], Rs);
            const double d2 = dot3_rn(Rs[0], Rs[1], Rs[2]);
            double t1, t2, t3;
            smear3<double>(d2, a12, kp.ew, &t1, &t2, &t3);
            const size_t si = 3 * ((size_t)b * kp.S + 3 * N + i), sj = 3 * ((size_t)b * kp.S + 3 * N + j);
            const double ui[3] = {u[si], u[si + 1], u[si + 2]}, uj[3] = {u[sj], u[sj + 1], u[sj + 2]};
            const double vi[3] = {v[si], v[si + 1], v[si + 2]}, vj[3] = {v[sj], v[sj + 1], v[sj + 2]};
            double dij[3] = {0, 0, 0};
            dd_force(Rs, ui, vj, t2, t3, dij);  // -grad_R (u_i T v_j)
            dd_force(Rs, vi, uj, t2, t3, dij);  // -grad_R (v_i T u_j)
            atomic3(grad + si, dij, -w);
            atomic3(grad + sj, dij, w);
            if (d2 < 25.0) {
                const double r = sqrt(d2), e1 = exp(-a12 * d2 * r);
                const double rui = Rs[0] * ui[0] + Rs[1] * ui[1] + Rs[2] * ui[2];
                const double ruj = Rs[0] * uj[0] + Rs[1] * uj[1] + Rs[2] * uj[2];
                const double rvi = Rs[0] * vi[0] + Rs[1] * vi[1] + Rs[2] * vi[2];
                const double rvj = Rs[0] * vj[0] + Rs[1] * vj[1] + Rs[2] * vj[2];
                const double uv = ui[0] * vj[0] + ui[1] * vj[1] + ui[2] * vj[2];
                const double vu = vi[0] * uj[0] + vi[1] * uj[1] + vi[2] * uj[2];
                const double dT = 3.0 * a12 * r * e1 * (rui * rvj + rvi * ruj) - e1 * (uv + vu);
                th[0] += w * dT * pf.v[4] * pf.v[4];  // d a12 / d a_dd = polfac_M^2
            }
        }
    }
    block_reduce_add<1, 128>(th, thacc + PIMD_TH_A_DD);
}

// The same bilinear term on the mixed engine (TTM3-F), as a gather over the full list like its
// real-space field: one warp per molecule i, lanes over its entries (i, j); the M-M separation
// from the molecule records (fixed-point M sites, the forward's own R), smear3 and the rank-3
// contraction in FP32, and only i's side accumulated (j's side when j gathers i), so each site
// has one writer; the d/da_dd sum, which sees every pair twice, at weight 1/2.
__global__ void __launch_bounds__(128) k_adj_ddbil_m(KP kp, double pfm2, const float4 *uf, const float4 *vf,
                                                     const double *bw, double *grad, double *thacc) {
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, b = blockIdx.y, N = kp.N;
    const double w = bw[b];
    float gi[3] = {0.f, 0.f, 0.f}, th = 0.f;
    if (i < N && w != 0.0) {
        const float4 *rec = kp.mrec + (size_t)b * N * 2;
        const float4 *ub = uf + (size_t)b * kp.S + kp.fd, *vb = vf + (size_t)b * kp.S + kp.fd;
        const int2 *fl = reinterpret_cast<const int2 *>(kp.fnbr) + (size_t)b * kp.fcap;
        const int ne = kp.fntot[b];
        const int e0 = min(kp.foff[(size_t)b * N + i], ne);
        const int e1 = (i + 1 < N) ? min(kp.foff[(size_t)b * N + i + 1], ne) : ne;
        const float4 ri = rec[2 * i], u4 = ub[i], v4 = vb[i];
        const unsigned mi[3] = {__float_as_uint(ri.x), __float_as_uint(ri.y), __float_as_uint(ri.z)};
        const float ui[3] = {u4.x, u4.y, u4.z}, vi[3] = {v4.x, v4.y, v4.z};
        const float a12 = kp.ptf.apol_dd[4][4];
        for (int e = e0 + lane; e < e1; e += 32) {
            const int j = fl[e].y;
            const float4 rj = rec[2 * j], uj4 = ub[j], vj4 = vb[j];
            const float R[3] = {(float)(int)(mi[0] - __float_as_uint(rj.x)) * kp.boxq[0],
                                (float)(int)(mi[1] - __float_as_uint(rj.y)) * kp.boxq[1],
                                (float)(int)(mi[2] - __float_as_uint(rj.z)) * kp.boxq[2]};
            const float uj[3] = {uj4.x, uj4.y, uj4.z}, vj[3] = {vj4.x, vj4.y, vj4.z};
            const float d2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
            float t1, t2, t3;
            smear3<float>(d2, a12, kp.ewf, &t1, &t2, &t3);
            float dij[3] = {0.f, 0.f, 0.f};
            dd_force_f(R, ui, vj, t2, t3, dij);
            dd_force_f(R, vi, uj, t2, t3, dij);
            gi[0] -= dij[0];
            gi[1] -= dij[1];
            gi[2] -= dij[2];
            if (d2 < 25.f) {
                const float r = sqrtf(d2), e1x = __expf(-a12 * d2 * r);
                const float rui = R[0] * ui[0] + R[1] * ui[1] + R[2] * ui[2];
                const float ruj = R[0] * uj[0] + R[1] * uj[1] + R[2] * uj[2];
                const float rvi = R[0] * vi[0] + R[1] * vi[1] + R[2] * vi[2];
                const float rvj = R[0] * vj[0] + R[1] * vj[1] + R[2] * vj[2];
                const float uv = ui[0] * vj[0] + ui[1] * vj[1] + ui[2] * vj[2];
                const float vu = vi[0] * uj[0] + vi[1] * uj[1] + vi[2] * uj[2];
                th += 3.f * a12 * r * e1x * (rui * rvj + rvi * ruj) - e1x * (uv + vu);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        gi[0] += __shfl_xor_sync(0xffffffffu, gi[0], o);
        gi[1] += __shfl_xor_sync(0xffffffffu, gi[1], o);
        gi[2] += __shfl_xor_sync(0xffffffffu, gi[2], o);
    }
    if (i < N && lane < 3) {
        const size_t si = 3 * ((size_t)b * kp.S + kp.fd + i) + lane;
        grad[si] += w * (double)(lane == 0 ? gi[0] : lane == 1 ? gi[1] : gi[2]);
    }
    double tv[1] = {0.5 * w * (double)th * pfm2};
    block_reduce_add<1, 128>(tv, thacc + PIMD_TH_A_DD);
}

// Q(2/3, x) by the Numerical-Recipes series / continued fraction used by the forward
PIMD_D double q23(double x) {
    unsigned err = 0;
    return gammq2_3<double>(x, &err);
}

// Real-space terms of one bead that do not involve the dipole iterations, per O-O pair:
//   * the charge-field adjoint nu: d/dx [nu . E_q] at fixed charges for the dipole site M of
//     one molecule and the charged sites H1, H2, M of the other (smear2 ts1, ts2 with the
//     charge-dipole Thole a), the potential of nu at those charged sites, and d/da_cc via
//     d ts1 / d a12 = e^{-a12 r^3};
//   * d Uelec / d a_cc = sum q_a q_c d ts0 / d a12 with d ts0 / d a12 = a12^{-2/3} Gamma(2/3)
//     Q(2/3, a12 r^3) / 3 (smear.f90:2-34 differentiated);
//   * van der Waals: the gradient of C/r^6 + D e^{-E r} (+ A/r^12 + B/r^10) and its C, D, E
//     derivatives (the energy's own gradient: the force-only switch of pot_ttm.f90:171 is not
//     part of the energy).
__global__ void __launch_bounds__(128) k_adj_pairs(KP kp, Polfac pf, const double *ebar, const double *nu,
                                                   double *grad, double *phin, double *thacc) {
    const int b = blockIdx.y, N = kp.N;
    const int np = kp.npair[b];
    const double eb = ebar[b];
    const double4_32a *pos = kp.pos + (size_t)b * kp.S;
    double th[4] = {0, 0, 0, 0};  // a_cc, C, D, E
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int2 ij = kp.pairs[(size_t)b * kp.cap + p];
        const int i = ij.x, j = ij.y;
        const int mol[2] = {i, j};
        // van der Waals on the O sites
        {
            const double4_32a Oi = pos[i], Oj = pos[j];
            const double R[3] = {min_image_rn(__dsub_rn(Oi.x, Oj.x), kp.box[0], kp.boxi[0]),
                                 min_image_rn(__dsub_rn(Oi.y, Oj.y), kp.box[1], kp.boxi[1]),
                                 min_image_rn(__dsub_rn(Oi.z, Oj.z), kp.box[2], kp.boxi[2])};
            const double r2 = dot3_rn(R[0], R[1], R[2]), r = sqrt(r2), r2i = 1.0 / r2, r6i = r2i * r2i * r2i;
            const double ex = exp(-kp.vdwE * r);
            const double dudr_over_r = (-12.0 * kp.vdwA * r6i * r6i - 10.0 * kp.vdwB * r6i * r2i * r2i - 6.0 * kp.vdwC * r6i) * r2i -
                                       kp.vdwD * kp.vdwE * ex / r;
            double gv[3] = {dudr_over_r * R[0], dudr_over_r * R[1], dudr_over_r * R[2]};
            atomic3(grad + 3 * ((size_t)b * kp.S + i), gv, eb);
            atomic3(grad + 3 * ((size_t)b * kp.S + j), gv, -eb);
            th[1] += eb * r6i;
            th[2] += eb * ex;
            th[3] += -eb * kp.vdwD * r * ex;
        }
        // charged sites H1, H2, M (kinds 2..4) of both molecules
        for (int a = 2; a <= 4; a++) {
            for (int c = 2; c <= 4; c++) {
                const double4_32a sa = pos[(a - 1) * N + i], sc = pos[(c - 1) * N + j];
                double Rs[3];
                pair_vec(kp, pos[i], pos[j], sa, sc, Rs);  // r_a(i) - r_c(j)
                const double d2 = dot3_rn(Rs[0], Rs[1], Rs[2]);
                const double a12 = kp.pt.apol_cd[a][c];
                double ts1, ts2;
                smear2<double>(d2, a12, kp.ew, &ts1, &ts2);
                const double e1 = (d2 < 25.0) ? exp(-a12 * d2 * sqrt(d2)) : 0.0;
                const double pfac = pf.v[a] * pf.v[c];
                // Uelec d/da_cc (q_a q_c ts0 summed over the pair's site pairs)
                if (d2 < 25.0) {
                    const double x = a12 * d2 * sqrt(d2);
                    const double dts0 = (1.0 / 3.0) * pow(a12, -2.0 / 3.0) * 1.3541179394264 * q23(x);
                    th[0] += eb * sa.w * sc.w * dts0 * pfac;
                }
                // nu at M(i) in the field of charge c(j): E = q_c ts1 R, R = r_M(i) - r_c(j)
                for (int side = 0; side < 2; side++) {
                    const int dk = side == 0 ? a : c;  // the dipole end must be the M site
                    if (dk != 4) continue;
                    const int md = mol[side], mc = mol[1 - side];
                    const int ck = side == 0 ? c : a;
                    const double qc = side == 0 ? sc.w : sa.w;
                    const double sg = side == 0 ? 1.0 : -1.0;  // R = sg * Rs
                    const double R[3] = {sg * Rs[0], sg * Rs[1], sg * Rs[2]};
                    const size_t sm = (size_t)b * kp.S + 3 * N + md, scs = (size_t)b * kp.S + (ck - 1) * N + mc;
                    const double n[3] = {nu[3 * sm], nu[3 * sm + 1], nu[3 * sm + 2]};
                    const double rn = R[0] * n[0] + R[1] * n[1] + R[2] * n[2];
                    double gm[3];
                    for (int q = 0; q < 3; q++) gm[q] = qc * (ts1 * n[q] - 3.0 * ts2 * rn * R[q]);
                    atomic3(grad + 3 * sm, gm, 1.0);
                    atomic3(grad + 3 * scs, gm, -1.0);
                    atomicAdd(phin + scs, ts1 * rn);
                    th[0] += qc * e1 * rn * pfac;
                }
            }
        }
    }
    block_reduce_add<4, 128>(th, thacc + PIMD_TH_A_CC);  // slots A_CC, VDW_C, VDW_D, VDW_E (contiguous)
}

// NASA PES derivatives with respect to its four scale factors for one molecule
// (nasa.f90:2-103): Vc = 2 c_0 + efac sum_j c_j sym_j f3_j with c_j = sum_X f_X C^X_j, and
// deoh, phh1 proportional to f5z.
PIMD_D void nasa_theta(const double r1[3][3], const double box[3], const double boxi[3], double f5z, double d[4]) {
    double ROH1[3], ROH2[3], RHH[3];
    for (int c = 0; c < 3; c++) {
        ROH1[c] = min_image_rn(__dsub_rn(r1[1][c], r1[0][c]), box[c], boxi[c]);
        ROH2[c] = min_image_rn(__dsub_rn(r1[2][c], r1[0][c]), box[c], boxi[c]);
        RHH[c] = min_image_rn(__dsub_rn(r1[1][c], r1[2][c]), box[c], boxi[c]);
    }
    const double dROH1 = sqrt(ROH1[0] * ROH1[0] + ROH1[1] * ROH1[1] + ROH1[2] * ROH1[2]);
    const double dROH2 = sqrt(ROH2[0] * ROH2[0] + ROH2[1] * ROH2[1] + ROH2[2] * ROH2[2]);
    const double dRHH = sqrt(RHH[0] * RHH[0] + RHH[1] * RHH[1] + RHH[2] * RHH[2]);
    const double costh = (ROH1[0] * ROH2[0] + ROH1[1] * ROH2[1] + ROH1[2] * ROH2[2]) / (dROH1 * dROH2);
    const double reoh = PIMD_NASA_REOH, b1 = PIMD_NASA_B1, roh = PIMD_NASA_ROH, alphaoh = PIMD_NASA_ALPHAOH,
                 phh2 = PIMD_NASA_PHH2, costhe = -.24780227221366464506;
    const double exp1 = exp(-alphaoh * (dROH1 - roh)), exp2 = exp(-alphaoh * (dROH2 - roh));
    const double x1 = (dROH1 - reoh) / reoh, x2 = (dROH2 - reoh) / reoh, x3 = costh - costhe;
    double f1[16], f2[16], f3[16];
    f1[0] = f2[0] = f3[0] = 0.0;
    f1[1] = f2[1] = f3[1] = 1.0;
    for (int j = 2; j <= 15; j++) {
        f1[j] = f1[j - 1] * x1;
        f2[j] = f2[j - 1] * x2;
        f3[j] = f3[j - 1] * x3;
    }
    const double efac = exp(-b1 * ((dROH1 - reoh) * (dROH1 - reoh) + (dROH2 - reoh) * (dROH2 - reoh)));
    double sx[4] = {0, 0, 0, 0};
    for (int j = 1; j < 245; j++) {
        const int inI = c_idx[j][0], inJ = c_idx[j][1], inK = c_idx[j][2];
        const double t = (f1[inI] * f2[inJ] + f1[inJ] * f2[inI]) * f3[inK];
        for (int x = 0; x < 4; x++) sx[x] += c_nasa4[x][j] * t;
    }
    const double sc = 0.00285914375100642899;
    for (int x = 0; x < 4; x++) d[x] = sc * (2.0 * c_nasa4[x][0] + efac * sx[x]);
    // deoh = f5z DEOHA, phh1 = f5z PHH1A e^{phh2}
    d[0] += sc * (PIMD_NASA_DEOHA * (exp1 * (exp1 - 2.0) + exp2 * (exp2 - 2.0)) +
                  PIMD_NASA_PHH1A * exp(phh2) * exp(-phh2 * dRHH));
    (void)f5z;
}

// Per molecule: the monomer PES gradient, the fixed-charge gradient -q E of Uelec, the
// intramolecular part of the charge-field adjoint (the Ewald exclusions between M and H1, H2 of
// the same molecule, smear.f90:110-156), then -- with every site gradient and the total
// potential phi = ebar phi_q + phi_nu in place -- the chain through the DMS charges (grdq) and
// the M site (pot_ttm.f90:556-604), and d/d(dms1..3, gamma, NASA factors). Writes dRRt.
template <int PHASE>
__global__ void __launch_bounds__(128) k_adj_mol(KP kp, const double *ebar, const double *phiq, const double *nu,
                                                 double *grad, double *phin, double *dRRt, double *thacc) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, N = kp.N;
    double th[PIMD_NTHETA];
    for (int i = 0; i < PIMD_NTHETA; i++) th[i] = 0.0;
    if (w < N) {
        const double eb = ebar[b];
        const size_t base = (size_t)b * kp.S;
        const double4_32a *pos = kp.pos + base;
        double4_32a s[4];
        for (int k = 0; k < 4; k++) s[k] = pos[k * N + w];
        if (PHASE == 0) {
            // monomer PES
            double R[3][3], dr1[3][3], e1;
            for (int k = 0; k < 3; k++) {
                R[k][0] = s[k].x;
                R[k][1] = s[k].y;
                R[k][2] = s[k].z;
            }
            if (!kp.contraction) {
                nasa_pot(R, kp.box, kp.boxi, dr1, &e1, kp.c5z, kp.nasa_f5z);
                for (int k = 0; k < 3; k++)
                    for (int c = 0; c < 3; c++) grad[3 * (base + k * N + w) + c] += eb * dr1[k][c];
                double d4[4];
                nasa_theta(R, kp.box, kp.boxi, kp.nasa_f5z, d4);
                for (int x = 0; x < 4; x++) th[PIMD_TH_F5Z + x] += eb * d4[x];
            }
            // Uelec at fixed charges: -q E_q at the charged sites H1, H2, M
            for (int k = 1; k < 4; k++) {
                const double4_32a F = kp.F[base + k * N + w];
                grad[3 * (base + k * N + w) + 0] -= eb * s[k].w * F.x;
                grad[3 * (base + k * N + w) + 1] -= eb * s[k].w * F.y;
                grad[3 * (base + k * N + w) + 2] -= eb * s[k].w * F.z;
            }
            // intramolecular charge field at M from H1, H2: E = q_H ts1 R, R = r_M - r_H
            const size_t sm = base + 3 * N + w;
            const double n[3] = {nu[3 * sm], nu[3 * sm + 1], nu[3 * sm + 2]};
            for (int k = 1; k <= 2; k++) {
                const double R[3] = {min_image_rn(__dsub_rn(s[3].x, s[k].x), kp.box[0], kp.boxi[0]),
                                     min_image_rn(__dsub_rn(s[3].y, s[k].y), kp.box[1], kp.boxi[1]),
                                     min_image_rn(__dsub_rn(s[3].z, s[k].z), kp.box[2], kp.boxi[2])};
                double ts1, ts2;
                self2(dot3_rn(R[0], R[1], R[2]), kp.ew, &ts1, &ts2);
                const double rn = R[0] * n[0] + R[1] * n[1] + R[2] * n[2];
                for (int c = 0; c < 3; c++) {
                    const double gm = s[k].w * (ts1 * n[c] - 3.0 * ts2 * rn * R[c]);
                    grad[3 * sm + c] += gm;
                    grad[3 * (base + k * N + w) + c] -= gm;
                }
                phin[base + k * N + w] += ts1 * rn;
            }
        } else {
            // charge chain and the M site
            const double phH1 = eb * phiq[base + N + w] + phin[base + N + w];
            const double phH2 = eb * phiq[base + 2 * N + w] + phin[base + 2 * N + w];
            const double phM = eb * phiq[base + 3 * N + w] + phin[base + 3 * N + w];
            const double *g = kp.grdq + ((size_t)b * N + w) * 27;
            double dg[3][3];
            for (int c = 0; c < 3; c++) {
                dg[1][c] = g[0 + 0 + c] * phH1 + g[0 + 3 + c] * phH2 + g[0 + 6 + c] * phM;
                dg[2][c] = g[9 + 0 + c] * phH1 + g[9 + 3 + c] * phH2 + g[9 + 6 + c] * phM;
                dg[0][c] = g[18 + 0 + c] * phH1 + g[18 + 3 + c] * phH2 + g[18 + 6 + c] * phM;
            }
            const double xo[3] = {s[0].x, s[0].y, s[0].z}, xh1[3] = {s[1].x, s[1].y, s[1].z},
                         xh2[3] = {s[2].x, s[2].y, s[2].z};
            double r1[3], r2[3];
            for (int c = 0; c < 3; c++) {
                r1[c] = min_image_rn(__dsub_rn(xh1[c], xo[c]), kp.box[c], kp.boxi[c]);
                r2[c] = min_image_rn(__dsub_rn(xh2[c], xo[c]), kp.box[c], kp.boxi[c]);
            }
            const double gam = kp.gammaM;
            double gO[3], gH1[3], gH2[3], gM[3];
            for (int c = 0; c < 3; c++) {
                gO[c] = grad[3 * (base + w) + c] + dg[0][c];
                gH1[c] = grad[3 * (base + N + w) + c] + dg[1][c];
                gH2[c] = grad[3 * (base + 2 * N + w) + c] + dg[2][c];
                gM[c] = grad[3 * (base + 3 * N + w) + c];
            }
            double *out = dRRt + ((size_t)b * kp.natoms + 3 * w) * 3;
            for (int c = 0; c < 3; c++) {
                out[c] = gO[c] + (1.0 - gam) * gM[c];
                out[3 + c] = gH1[c] + 0.5 * gam * gM[c];
                out[6 + c] = gH2[c] + 0.5 * gam * gM[c];
            }
            // DMS charges q3 (x CHARGECON) and the corrections Q1, Q2 (nasa.f90:234-242)
            double R[3][3], q3[3], dq3[3][3][3];
            for (int k = 0; k < 3; k++) {
                R[k][0] = s[k].x;
                R[k][1] = s[k].y;
                R[k][2] = s[k].z;
            }
            nasa_dms(R, kp.box, kp.boxi, kp.dms1, kp.dms2, kp.dms3, q3, dq3);
            for (int k = 0; k < 3; k++) q3[k] *= CHARGECON;
            const double tmp = 0.5 * gam / (1.0 - gam);
            const double dq0 = phM / (1.0 - gam);                   // dE/dq3[0]
            const double dq1 = phH1 * (1.0 + tmp) + phH2 * tmp;     // dE/dq3[1]
            const double dq2 = phH1 * tmp + phH2 * (1.0 + tmp);     // dE/dq3[2]
            const double dQ1 = CHARGECON * (dq1 - dq0), dQ2 = CHARGECON * (dq2 - dq0);
            const double d1 = sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
            const double d2 = sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
            const double ax = r1[1] * r2[2] - r1[2] * r2[1], ay = -r1[0] * r2[2] + r1[2] * r2[0],
                         az = r1[0] * r2[1] - r1[1] * r2[0];
            const double costh = (r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2]) / (d1 * d2);
            const double ang = atan2(sqrt(ax * ax + ay * ay + az * az) / (d1 * d2), costh);
            const double ath0 = 1.82400520401572996557;
            th[PIMD_TH_DMS1] += dQ1 * (d1 - kp.dms2) + dQ2 * (d2 - kp.dms2);
            th[PIMD_TH_DMS2] += -kp.dms1 * (dQ1 + dQ2);
            th[PIMD_TH_DMS3] += (ang - ath0) * (dQ1 + dQ2);
            // gamma: q_H = q3_H + tmp (q3_1 + q3_2), q_M = q3_0 / (1 - gamma), r_M = r_O + gamma/2 (r1 + r2)
            const double dtmp = 0.5 / ((1.0 - gam) * (1.0 - gam));
            th[PIMD_TH_GAMMA_M] += (phH1 + phH2) * (q3[1] + q3[2]) * dtmp + phM * q3[0] / ((1.0 - gam) * (1.0 - gam));
            for (int c = 0; c < 3; c++) th[PIMD_TH_GAMMA_M] += gM[c] * 0.5 * (r1[c] + r2[c]);
        }
    }
    block_reduce_add<PIMD_NTHETA, 128>(th, thacc);
}

}  // namespace pimd

// ---------------------------------------------------------------------------------------
using namespace pimd;

static int adj_fail(Engine &E, int code, const char *msg) {
    E.last_error = msg;
    return code;
}

extern "C" {

int pimd_get_theta(pimd_ctx *ctx, double *theta) {
    if (!ctx || !theta) return PIMD_ERR_ARG;
    std::memcpy(theta, ctx->E.theta, sizeof(double) * PIMD_NTHETA);
    return PIMD_OK;
}

int pimd_set_theta(pimd_ctx *ctx, const double *theta) {
    if (!ctx || !theta) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (E.kp.model != 3) return adj_fail(E, PIMD_ERR_ARG, "theta is defined for TTM3-F contexts");
    if (!(theta[PIMD_TH_POLAR_M] > 0) || !(theta[PIMD_TH_A_DD] > 0) || !(theta[PIMD_TH_A_CC] > 0) ||
        !(theta[PIMD_TH_GAMMA_M] > 0 && theta[PIMD_TH_GAMMA_M] < 1))
        return adj_fail(E, PIMD_ERR_ARG, "theta out of range (polarisability, dampings > 0, 0 < gamma < 1)");
    cudaSetDevice(E.device);
    std::memcpy(E.theta, theta, sizeof(double) * PIMD_NTHETA);
    E.tape_valid = false;
    return apply_theta(E);
}

int pimd_pot_forward(pimd_ctx *ctx, const double *RRt, const double *RRc, double *Upott, int t) {
    if (!ctx || !RRt || !RRc) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (E.kp.model != 3) return adj_fail(E, PIMD_ERR_ARG, "the differentiation form needs a TTM3-F context");
    if (E.kp.guess && t > 4) return adj_fail(E, PIMD_ERR_ARG, "the dipole predictor must be off (guess_initdip = 0 or t <= 4)");
    cudaSetDevice(E.device);
    const KP &kp = E.kp;
    const int nd = kp.ld - kp.fd;
    if (!E.d_tape || E.tape_kmax != kp.polar_maxiter) {
        if (E.d_tape) cudaFree(E.d_tape);
        if (E.d_phiq) cudaFree(E.d_phiq);
        if (E.d_tapeS) cudaFree(E.d_tapeS);
        E.d_tape = E.d_phiq = nullptr;
        E.d_tapeS = nullptr;
        E.tape_kmax = 0;
        if (cudaMalloc((void **)&E.d_tape, sizeof(double) * (kp.polar_maxiter + 1) * kp.P * nd * 3) != cudaSuccess ||
            cudaMalloc((void **)&E.d_phiq, sizeof(double) * kp.P * kp.S) != cudaSuccess ||
            cudaMalloc((void **)&E.d_tapeS, sizeof(double2) * std::max(1, kp.polar_maxiter) * kp.P * kp.nk) != cudaSuccess)
            return adj_fail(E, PIMD_ERR_NOMEM, "tape allocation");
        E.tape_kmax = kp.polar_maxiter;
    }
    E.tape_on = true;
    const int save_check = ctx->check_every;
    const bool save_async = E.dd_async;
    ctx->check_every = 1;
    E.dd_async = false;  // one recorded SOR step per iteration
    int rc = pimd_full_bead_forces(ctx, RRt, RRc, Upott, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, t);
    ctx->check_every = save_check;
    E.dd_async = save_async;
    E.tape_on = false;
    E.tape_valid = rc == PIMD_OK;
    return rc;
}

int pimd_pot_backward(pimd_ctx *ctx, const double *Ebar, double *dRRt, double *dtheta) {
    if (!ctx || !Ebar) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (!E.tape_valid) return adj_fail(E, PIMD_ERR_STATE, "no recorded forward (pimd_pot_forward) for this backward");
    cudaSetDevice(E.device);
    KP &kp = E.kp;
    const size_t P = kp.P, S = kp.S, nd = kp.ld - kp.fd, sv = 3 * P * S;
    const bool mixed = E.precision == PIMD_MIXED;
    // scratch: g, u, v, Dr, grad, nu (site vectors), phin, Smu, Snu, bacc, bw, ebar, ones, thacc,
    // dRRt, FP32 u and v per site (mixed engine), iters
    const size_t nbytes = sizeof(double) * (3 * P * nd + 5 * sv + P * S + 4 * P * kp.nk + P * NACC + 3 * P + PIMD_NTHETA +
                                            P * kp.natoms * 3) + sizeof(float4) * 2 * P * S + sizeof(int) * P + 256;
    if (E.adj_bytes < nbytes) {
        if (E.d_adj) cudaFree(E.d_adj);
        if (cudaMalloc((void **)&E.d_adj, nbytes) != cudaSuccess) {
            E.d_adj = nullptr;
            E.adj_bytes = 0;
            return adj_fail(E, PIMD_ERR_NOMEM, "backward scratch");
        }
        E.adj_bytes = nbytes;
    }
    double *g = E.d_adj, *u = g + 3 * P * nd, *v = u + sv, *Dr = v + sv, *grad = Dr + sv, *nu = grad + sv;
    double *phin = nu + sv;
    const uintptr_t sa = (reinterpret_cast<uintptr_t>(phin + P * S) + 15) & ~uintptr_t(15);  // 16-byte rows
    double2 *Smu = reinterpret_cast<double2 *>(sa), *Snu = Smu + P * kp.nk;
    double *bacc = reinterpret_cast<double *>(Snu + P * kp.nk), *bw = bacc + P * NACC, *ebar = bw + P, *ones = ebar + P;
    double *thacc = ones + P, *dR = thacc + PIMD_NTHETA;
    const uintptr_t ua = (reinterpret_cast<uintptr_t>(dR + P * kp.natoms * 3) + 15) & ~uintptr_t(15);  // 16-byte rows
    float4 *uf = reinterpret_cast<float4 *>(ua), *vf = uf + P * S;
    int *iters = reinterpret_cast<int *>(vf + P * S);
    cudaStream_t st = E.stream;
    // per-bead iteration counts of the forward
    std::vector<double> acc(P * NACC);
    cudaMemcpyAsync(acc.data(), kp.acc, sizeof(double) * P * NACC, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    std::vector<int> it(P);
    int kmax = 0;
    for (size_t b = 0; b < P; b++) {
        it[b] = (int)acc[b * NACC + ACC_NITER];
        kmax = std::max(kmax, it[b]);
    }
    std::vector<double> one(P, 1.0);
    cudaMemcpyAsync(iters, it.data(), sizeof(int) * P, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(ebar, Ebar, sizeof(double) * P, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(ones, one.data(), sizeof(double) * P, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(grad, 0, sizeof(double) * sv, st);
    cudaMemsetAsync(nu, 0, sizeof(double) * sv, st);
    cudaMemsetAsync(u, 0, sizeof(double) * 2 * sv, st);
    cudaMemsetAsync(phin, 0, sizeof(double) * P * S, st);
    cudaMemsetAsync(bacc, 0, sizeof(double) * P * NACC, st);
    cudaMemsetAsync(thacc, 0, sizeof(double) * PIMD_NTHETA, st);
    const dim3 gd((unsigned)((nd + 127) / 128), (unsigned)P), gm((unsigned)((kp.N + 127) / 128), (unsigned)P);
    long nb = ((long)kp.N * 64 + 127) / 128;
    nb = std::max(8L, std::min(4096L, nb));
    const dim3 gp((unsigned)nb, (unsigned)P);
    Polfac pf;
    for (int i = 0; i < 5; i++) pf.v[i] = E.polfac[i];
    const double omega = kp.polar_sor;
    const dim3 gw((unsigned)((kp.N * 32 + 127) / 128), (unsigned)P);  // a warp per molecule
    // the mixed sweep's reciprocal passes on the tensor cores when the forward has them (the
    // structure factor, the field pass and the force pass's dipole half)
    const bool tcs = mixed && kp.model == 3 && E.tc_ready && E.sf_tc && E.tf_ready && E.ff_tc && E.tf_qd_ready &&
                     kp.Fx && kp.ld - kp.fd == kp.N;
    k_adj_init<<<gd, 128, 0, st>>>(kp, ebar, g, nu);
    for (int k = kmax; k >= 1; k--) {
        k_adj_u<<<gd, 128, 0, st>>>(kp, k, iters, E.d_tape, g, u, v, nu, bacc, bw, thacc, omega, mixed ? uf : nullptr,
                                    mixed ? vf : nullptr);
        cudaMemsetAsync(Dr, 0, sizeof(double) * sv, st);
        {  // D_real u: the forward's cached Thole tensors (FP64), or its per-entry smear scalars
           // with u in the molecule records (mixed)
            KP kq = kp;
            kq.dip = u;
            kq.Efdr = Dr;
            kq.acc = bacc;
            kq.dd_async = 0;
            const KP keep = E.kp;
            E.kp = kq;
            if (mixed)
                launch_dd_real_m(E);
            else
                launch_dd_real(E);
            E.kp = keep;
        }
        // S(v) = S(mu_{k-1}) is on the tape (the forward's iteration k formed it)
        const double2 *Smv = E.d_tapeS + (size_t)(k - 1) * P * kp.nk;
        adj_structure_factor(E, u, mixed ? uf : nullptr, Smu, bacc);
        if (tcs) {
            // tensor-core sweep: the field of u (TF_Q on the weights of S_u moved to slot 0) into
            // Fx, then the reciprocal bilinear term as the dipole force of v in the field of u
            // plus that of u in the field of v (TF_DG, slot 1 zero) into dR:
            // d/dx [u^T D_rec v] = -(dipole force of u in E_v + dipole force of v in E_u)
            const dim3 gk((unsigned)((kp.nk + 255) / 256), (unsigned)P);
            k_adj_wslots<0><<<gk, 256, 0, st>>>(kp, nullptr);
            KP kq = kp;
            kq.acc = bacc;
            kq.dd_async = 0;
            kq.fx_mode = 1;
            const KP keep = E.kp;
            E.kp = kq;
            launch_adj_field_tc(E);
            cudaMemsetAsync(kp.dR, 0, sizeof(double) * sv, st);
            E.kp.fx_mode = 0;
            E.kp.dipf = vf;
            launch_adj_dforce_tc(E);
            k_adj_wslots<1><<<gk, 256, 0, st>>>(kp, Smv);
            E.kp.dipf = uf;
            launch_adj_dforce_tc(E);
            E.kp = keep;
            E.nlaunch += 2;
            k_adj_g<<<gd, 128, 0, st>>>(kp, k, iters, g, u, Dr, omega, kp.Fx, kp.dR, bw, grad);
        } else {
            adj_dipole_field(E, Smu, bacc, Dr);
            k_adj_g<<<gd, 128, 0, st>>>(kp, k, iters, g, u, Dr, omega, nullptr, nullptr, bw, grad);
        }
        if (mixed)
            k_adj_ddbil_m<<<gw, 128, 0, st>>>(kp, pf.v[4] * pf.v[4], uf, vf, bw, grad, thacc);
        else
            k_adj_ddbil<<<gp, 128, 0, st>>>(kp, pf, u, v, bw, grad, thacc);
        if (!tcs) adj_rec(E, 0, u, v, Smu, Smv, bw, grad, nullptr);
    }
    k_adj_final<<<gd, 128, 0, st>>>(kp, g, nu, thacc, tcs ? uf : nullptr);
    // charge-field adjoint nu: real-space pairs, reciprocal, intramolecular; vdW; Uelec d/da_cc
    cudaMemsetAsync(bacc, 0, sizeof(double) * P * NACC, st);
    if (tcs) {
        // the cross term on the tensor cores: S_nu, the force pass's charge half on its weights
        // (Fx at the charged sites), then its dipole half of nu on the charge weights (dR)
        adj_structure_factor(E, nu, uf, Snu, bacc);
        KP kq = kp;
        kq.acc = bacc;
        kq.dd_async = 0;
        kq.fx_mode = 2;
        const KP keep = E.kp;
        E.kp = kq;
        launch_adj_qforce_tc(E);
        const dim3 gk((unsigned)((kp.nk + 255) / 256), (unsigned)P);
        k_adj_wslots<2><<<gk, 256, 0, st>>>(kp, kp.Sq);
        cudaMemsetAsync(kp.dR, 0, sizeof(double) * sv, st);
        E.kp.fx_mode = 0;
        E.kp.dipf = uf;
        launch_adj_dforce_tc(E);
        E.kp = keep;
        const dim3 gq((unsigned)((kp.S - kp.N + 127) / 128), (unsigned)P);
        k_adj_cross_fold<<<gq, 128, 0, st>>>(kp, kp.N, grad, phin);
        E.nlaunch += 2;
    } else {
        adj_structure_factor(E, nu, nullptr, Snu, bacc);
        adj_rec(E, 1, nu, nullptr, Snu, nullptr, ones, grad, phin);
    }
    if (mixed)
        launch_adj_pairs_m(E, pf.v, ebar, nu, grad, phin, thacc);
    else
        k_adj_pairs<<<gp, 128, 0, st>>>(kp, pf, ebar, nu, grad, phin, thacc);
    k_adj_mol<0><<<gm, 128, 0, st>>>(kp, ebar, E.d_phiq, nu, grad, phin, dR, thacc);
    k_adj_mol<1><<<gm, 128, 0, st>>>(kp, ebar, E.d_phiq, nu, grad, phin, dR, thacc);
    E.nlaunch += 5 + 8 * (long long)kmax;
    // d Uvdw_lrc / dC at fixed cutoff (potential.f90:152-154)
    std::vector<double> th(PIMD_NTHETA);
    cudaMemcpyAsync(th.data(), thacc, sizeof(double) * PIMD_NTHETA, cudaMemcpyDeviceToHost, st);
    if (dRRt) cudaMemcpyAsync(dRRt, dR, sizeof(double) * P * kp.natoms * 3, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return adj_fail(E, PIMD_ERR_CUDA, cudaGetErrorString(e));
    double esum = 0;
    for (size_t b = 0; b < P; b++) esum += Ebar[b];
    const double rc3 = E.rc * E.rc * E.rc;
    th[PIMD_TH_VDW_C] += esum * TWOPI * (double)(kp.N * kp.N) / kp.volume / (3.0 * rc3);
    if (dtheta) std::copy(th.begin(), th.end(), dtheta);
    return PIMD_OK;
}

}  // extern "C"

namespace pimd {
// constant tables of this translation unit: the NASA tables of nasa.cuh and the four PES
// coefficient sets for the scale-factor derivatives
void adjoint_init(Engine &E) {
    (void)E;
    nasa_upload_constants();
    static double tab[4][245];
    for (int j = 0; j < 245; j++) {
        tab[0][j] = PIMD_NASA_C5ZA[j];
        tab[1][j] = PIMD_NASA_CBASIS[j];
        tab[2][j] = PIMD_NASA_CCORE[j];
        tab[3][j] = PIMD_NASA_CREST[j];
    }
    cudaMemcpyToSymbol(c_nasa4, tab, sizeof(tab));
}
}  // namespace pimd
