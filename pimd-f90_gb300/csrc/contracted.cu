// contracted.cu -- ring-polymer contraction with multiple time steps (MD.f90:276-449,
// contracted_MD) and monomer PIMD (MD.f90:117-265, monomer_PIMD) on the device.
//
// The intramolecular (fast) forces -- the NASA monomer PES, pot_nasa of nasa.f90:2-103 -- act on
// every bead; the intermolecular (slow) ones on the centroid only, through a one-bead context of
// the centroid (contraction set for contracted_MD, so pot_ttm skips the monomer PES there,
// pot_ttm.f90:92-132; unset for monomer_PIMD, whose centroid call keeps it, as the reference's
// does). The bead monomer kernel is one thread per (molecule, bead); the inner MTS steps are the
// fast kicks, EvolveRing with the normal modes made for deltfast, and the monomer kernel again.
// The thermostats, kinetic energies and estimators are the MD step's (nm.cu).
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/pimd_gb300.h"
#include "engine.h"
#include "nasa.cuh"

namespace pimd {

// scratch of the contracted step in ctx->d_con: dRRc (3 Na), the centroid's Upot, virial trace,
// virialc (3), dip_momI / dip_momE of the centroid (3 Nw each), Upott (P), [virialmon,
// virialcmon] (2), [Upot, virial, virialc] (3), dRRmon (3 Na P, monomer PIMD)
struct ConScratch {
    double *dRRc, *cen3, *dI, *dE, *Upott, *vir2, *uvv, *dRRmon;
};
static ConScratch con_scratch(pimd_ctx *ctx) {
    const int na = ctx->E.kp.natoms, nw = na / 3, P = ctx->E.kp.P;
    ConScratch c;
    c.dRRc = ctx->d_con;
    c.cen3 = c.dRRc + 3 * (size_t)na;
    c.dI = c.cen3 + 3;
    c.dE = c.dI + 3 * (size_t)nw;
    c.Upott = c.dE + 3 * (size_t)nw;
    c.vir2 = c.Upott + P;
    c.uvv = c.vir2 + 2;
    c.dRRmon = c.uvv + 3;
    return c;
}
static size_t con_scratch_size(int na, int P) { return 3 * (size_t)na + 3 + 2 * (size_t)na + P + 5 + 3 * (size_t)na * P; }

// PPt = PPt - MASSCON g dt2 (MD.f90:308, 324, 381, 433)
__global__ void k_kick(double *PPt, const double *g, size_t n, double dt2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        PPt[i] = __dsub_rn(PPt[i], __dmul_rn(__dmul_rn(MASSCON, g[i]), dt2));
}

// free flight of one bead (P = 1): RRt = RRt + imass PPt dt (MD.f90:334-340)
__global__ void k_free_flight(double *RRt, const double *PPt, int natoms, double massO, double massH, double dt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * natoms; i += gridDim.x * blockDim.x) {
        const double im = 1.0 / ((i / 3) % 3 == 0 ? massO : massH);
        RRt[i] = __dadd_rn(RRt[i], __dmul_rn(__dmul_rn(im, PPt[i]), dt));
    }
}

// RRc = sum(RRt, 3) / Nbeads and the centroid-following PBC shift (main_stuff.f90:107-125)
__global__ void k_centroid_pbc(double *RRt, double *RRc, int natoms, int P, double box0, double boxi0) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * natoms; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < P; j++) s = __dadd_rn(s, RRt[i + (size_t)3 * natoms * j]);
        const double rc = __ddiv_rn(s, (double)P);
        const double shift = __dmul_rn(box0, round(__dmul_rn(rc, boxi0)));
        RRc[i] = __dsub_rn(rc, shift);
        for (int j = 0; j < P; j++) RRt[i + (size_t)3 * natoms * j] = __dsub_rn(RRt[i + (size_t)3 * natoms * j], shift);
    }
}

// pot_nasa on every (molecule, bead): the gradient rows into g; with acc, the energies into
// Upott[bead] and the monomer virials, bead separations into vir2[0] and centroid separations
// (RRc) into vir2[1] (MD.f90:348-378 / 182-217)
__global__ void __launch_bounds__(128) k_monomer_beads(KP kp, int P, const double *RRt, const double *RRc, double *g,
                                                       double *Upott, double *vir2, int acc) {
    const int iw = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, N = kp.N, na = 3 * N;
    double e1 = 0.0, v[2] = {0.0, 0.0};
    if (iw < N) {
        const double *rb = RRt + (size_t)3 * na * j + 9 * (size_t)iw;
        double r1[3][3], dr1[3][3];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int c = 0; c < 3; c++) r1[a][c] = rb[3 * a + c];
        nasa_pot(r1, kp.box, kp.boxi, dr1, &e1, kp.c5z, kp.nasa_f5z);
        double *gb = g + (size_t)3 * na * j + 9 * (size_t)iw;
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int c = 0; c < 3; c++) gb[3 * a + c] = dr1[a][c];
        if (acc) {
#pragma unroll
            for (int w = 0; w < 2; w++) {
                const double *rr = w ? RRc + 9 * (size_t)iw : rb;
                double d1 = 0.0, d2 = 0.0;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const double roh1 = min_image_rn(__dsub_rn(rr[3 + c], rr[c]), kp.box[c], kp.boxi[c]);
                    const double roh2 = min_image_rn(__dsub_rn(rr[6 + c], rr[c]), kp.box[c], kp.boxi[c]);
                    d1 = __dadd_rn(d1, __dmul_rn(roh1, dr1[1][c]));
                    d2 = __dadd_rn(d2, __dmul_rn(roh2, dr1[2][c]));
                }
                v[w] = __dadd_rn(d1, d2);
            }
        }
    }
    if (!acc) return;
    for (int o = 16; o > 0; o >>= 1) {
        e1 += __shfl_xor_sync(0xffffffffu, e1, o);
        v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
        v[1] += __shfl_xor_sync(0xffffffffu, v[1], o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(Upott + j, e1);
        atomicAdd(vir2, v[0]);
        atomicAdd(vir2 + 1, v[1]);
    }
}

// calc_monomer_dip_moments (force_calc.f90:205-264): DMS charges of every bead's monomer, the
// dipole about the M site (TTM3-F) or the O atom, plus the centroid's induced dipoles dE
__global__ void __launch_bounds__(128) k_monomer_dipoles(KP kp, int P, int model, double gammaM, const double *RRt,
                                                         const double *dE, double *dipI, double *dipE) {
    const int iw = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, N = kp.N, na = 3 * N;
    if (iw >= N) return;
    const double *rb = RRt + (size_t)3 * na * j + 9 * (size_t)iw;
    double r1[3][3], q3[3], dq3[3][3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int c = 0; c < 3; c++) r1[a][c] = rb[3 * a + c];
    nasa_dms(r1, kp.box, kp.boxi, kp.dms1, kp.dms2, kp.dms3, q3, dq3);
    const double tmp = 0.5 * gammaM / (1.0 - gammaM);
    for (int a = 0; a < 3; a++) q3[a] = q3[a] * CHARGECON;
    const double cH1 = q3[1] + tmp * (q3[1] + q3[2]), cH2 = q3[2] + tmp * (q3[1] + q3[2]);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const double roh1 = min_image_rn(__dsub_rn(rb[3 + c], rb[c]), kp.box[c], kp.boxi[c]);
        const double roh2 = min_image_rn(__dsub_rn(rb[6 + c], rb[c]), kp.box[c], kp.boxi[c]);
        double d;
        if (model == 3 || model == 4) {
            const double Rm = 0.5 * gammaM * (roh1 + roh2) + rb[c];
            const double h1 = min_image_rn(__dsub_rn(rb[3 + c], Rm), kp.box[c], kp.boxi[c]);
            const double h2 = min_image_rn(__dsub_rn(rb[6 + c], Rm), kp.box[c], kp.boxi[c]);
            d = cH1 * h1 + cH2 * h2;
        } else {
            d = cH1 * roh1 + cH2 * roh2;
        }
        const size_t o = c + 3 * (size_t)iw + (size_t)3 * N * j;
        if (dipI) dipI[o] = d + dE[3 * iw + c];
        if (dipE) dipE[o] = dE[3 * iw + c];
    }
}

// dRRt(:,:,j) = dRRc (+ dRRmon(:,:,j) for monomer PIMD) (MD.f90:220-222, 403-405)
__global__ void k_broadcast_grad(double *dRRt, const double *dRRc, const double *dRRmon, int natoms, int P) {
    const size_t n = (size_t)3 * natoms * P;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double gc = dRRc[i % (3 * (size_t)natoms)];
        dRRt[i] = dRRmon ? __dadd_rn(gc, dRRmon[i]) : gc;
    }
}

// v[0 .. n) = *x
__global__ void k_fill(double *v, const double *x, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) v[i] = *x;
}

// Upott and the step's Upot, virial and virialc (MD.f90:179, 198, 224-227 / 400, 421-423):
// cen3 = the centroid call's [Upot, virial trace, virialc]
__global__ void k_con_totals(int P, int mode, const double *cen3, double *Upott, const double *vir2, double *uvv) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double U = 0.0;
    for (int j = 0; j < P; j++) {
        if (mode == 0) Upott[j] = Upott[j] + cen3[0];
        U += Upott[j];
    }
    uvv[0] = U;
    uvv[1] = vir2[0] + cen3[1];
    uvv[2] = vir2[1] / P + cen3[2];
}

static int con_err(Engine &E, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PIMD_OK;
    E.last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return PIMD_ERR_CUDA;
}

}  // namespace pimd

using namespace pimd;

extern "C" {

int pimd_contracted_init(pimd_ctx *ctx, int mode, int intra_timesteps) {
    if (!ctx || (mode != 0 && mode != 1) || intra_timesteps < 1) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (E.kp.model != 2 && E.kp.model != 3) {
        E.last_error = "contracted_init: ring-polymer contraction needs a TTM model (the NASA monomer PES)";
        return PIMD_ERR_ARG;
    }
    cudaSetDevice(E.device);
    nasa_upload_constants();
    if (ctx->cen && ctx->con_mode != mode) {
        pimd_destroy(ctx->cen);
        ctx->cen = nullptr;
    }
    if (!ctx->cen) {
        pimd_params p = ctx->params;
        p.nbeads = 1;
        p.contraction = mode == 0 ? 1 : 0;
        int rc = pimd_create(&ctx->cen, &p);
        if (rc) {
            E.last_error = "contracted_init: the centroid context could not be made";
            return rc;
        }
        pimd_set_theta(ctx->cen, E.theta);
    }
    if (!ctx->d_con) {
        if (cudaMalloc((void **)&ctx->d_con, sizeof(double) * con_scratch_size(E.kp.natoms, E.kp.P)) != cudaSuccess)
            return PIMD_ERR_NOMEM;
        E.allocs.push_back(ctx->d_con);
    }
    ctx->con_mode = mode;
    ctx->con_intra = intra_timesteps;
    pimd_set_stream(ctx->cen, E.stream);
    return con_err(E, cudaDeviceSynchronize(), "contracted_init");
}

int pimd_contracted_step_device(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt,
                                double *dRRfast, double *RRc, const double *xi1, const double *xi2, int t, double *out,
                                double *dip_momIt, double *dip_momEt) {
    if (!ctx || !mp || !RRt || !PPt || !dRRt || !RRc || !out) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (!ctx->cen || E.nm_P != E.kp.P || !E.d_nh) return PIMD_ERR_STATE;
    const int mode = ctx->con_mode, nin = ctx->con_intra;
    if (mode == 0 && !dRRfast) return PIMD_ERR_ARG;
    if (E.nh_bead && mp->langevin) {
        E.last_error = "contracted_step: Langevin_NM and the bead Nose-Hoover chains exclude each other";
        return PIMD_ERR_ARG;
    }
    cudaSetDevice(E.device);
    const int P = E.kp.P, na = E.kp.natoms, N = E.kp.N;
    const size_t nall = (size_t)3 * na * P;
    const ConScratch s = con_scratch(ctx);
    cudaStream_t st = E.stream;
    pimd_set_stream(ctx->cen, st);
    launch_set_step(E, t);
    NMArgs a = nm_step_args(E, mp, xi1);
    a.fast = 0;
    const double delt = mp->delt, delt2 = delt / 2.0;
    const double deltfast = mode == 0 ? delt / nin : delt, delt2fast = deltfast / 2.0;
    const unsigned gb = (unsigned)std::min<size_t>((nall + 255) / 256, 4096);
    const dim3 gm((N + 127) / 128, P);
    cudaMemsetAsync(s.Upott, 0, sizeof(double) * (P + 2), st);
    // bead thermostat, global chain, slow half kick, then (monomer PIMD) the drift, and the
    // centroid with its PBC shift
    if (E.nh_global) {
        nm_launch_nh_global(E, nullptr, 3, delt2);
        a.s_pre = E.d_nh + 3;
    }
    a.nodrift = mode == 0 ? 1 : 0;
    nm_launch_md_pre(a, st, RRt, PPt, dRRt, RRc);
    a.s_pre = nullptr;
    a.nodrift = 0;
    if (mode == 0) {
        NMArgs af = a;
        af.delt = deltfast;
        for (int ti = 1; ti <= nin; ti++) {
            k_kick<<<gb, 256, 0, st>>>(PPt, dRRfast, nall, delt2fast);
            if (P > 1)
                nm_launch_evolve(af, st, RRt, PPt);
            else
                k_free_flight<<<(3 * na + 255) / 256, 256, 0, st>>>(RRt, PPt, na, mp->massO, mp->massH, deltfast);
            if (ti == nin) cudaMemsetAsync(s.vir2, 0, 2 * sizeof(double), st);
            k_monomer_beads<<<gm, 128, 0, st>>>(E.kp, P, RRt, RRc, dRRfast, s.Upott, s.vir2, ti == nin);
            k_kick<<<gb, 256, 0, st>>>(PPt, dRRfast, nall, delt2fast);
            E.nlaunch += 3;
        }
        k_centroid_pbc<<<(3 * na + 127) / 128, 128, 0, st>>>(RRt, RRc, na, P, E.kp.box[0], E.kp.boxi[0]);
        ++E.nlaunch;
    }
    // the slow force on the centroid
    int rc = pimd_full_bead_forces_device(ctx->cen, RRc, RRc, s.cen3, s.dRRc, s.cen3 + 1, s.cen3 + 2, s.dI, s.dE,
                                          nullptr, t);
    if (rc) {
        E.last_error = std::string("contracted_step: centroid force call: ") + pimd_last_error(ctx->cen);
        return rc;
    }
    if (mode == 1) {  // Upott(:) = Upot, then the monomer PES on the beads
        k_fill<<<1, 32, 0, st>>>(s.Upott, s.cen3, P);
        k_monomer_beads<<<gm, 128, 0, st>>>(E.kp, P, RRt, RRc, s.dRRmon, s.Upott, s.vir2, 1);
        E.nlaunch += 2;
    }
    k_con_totals<<<1, 32, 0, st>>>(P, mode, s.cen3, s.Upott, s.vir2, s.uvv);
    k_broadcast_grad<<<gb, 256, 0, st>>>(dRRt, s.dRRc, mode == 1 ? s.dRRmon : nullptr, na, P);
    if (dip_momIt || dip_momEt)
        k_monomer_dipoles<<<gm, 128, 0, st>>>(E.kp, P, E.kp.model, E.kp.gammaM, RRt, s.dE, dip_momIt, dip_momEt);
    nm_launch_ring_sums(a, st, RRt, PPt, E.d_nh + 5);
    // slow half kick, bead thermostat, kinetic energy, global chain
    double *uk = E.d_out + 3 * P;
    cudaMemsetAsync(uk, 0, sizeof(double), st);
    a.xi = xi2;
    a.phase = 1;
    nm_launch_md_post(a, st, PPt, dRRt, uk);
    const double *ukout = uk;
    if (E.nh_global) {
        nm_launch_nh_global(E, uk, 4, delt2);
        nm_launch_nh_scale(E, PPt);
        ukout = E.d_nh + 2;
    } else {
        cudaMemcpyAsync(E.d_nh + 2, uk, sizeof(double), cudaMemcpyDeviceToDevice, st);
    }
    nm_launch_estimators(E, ukout, s.uvv, out);
    E.nlaunch += 8;
    return con_err(E, cudaGetLastError(), "contracted_step");
}

int pimd_contracted_step(pimd_ctx *ctx, const pimd_md_params *mp, double *RRt, double *PPt, double *dRRt,
                         double *dRRfast, double *RRc, const double *xi1, const double *xi2, int t, double *out,
                         double *dip_momIt, double *dip_momEt) {
    if (!ctx || !mp || !RRt || !PPt || !dRRt || !out) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
    if (!ctx->cen) return PIMD_ERR_STATE;
    cudaSetDevice(E.device);
    const size_t n = (size_t)E.kp.P * E.kp.natoms * 3, nc = (size_t)E.kp.natoms * 3, nd = (size_t)E.kp.P * E.kp.N * 3;
    double *d = nullptr;
    if (cudaMalloc((void **)&d, sizeof(double) * (6 * n + nc + 2 * nd + PIMD_MD_NOUT)) != cudaSuccess)
        return PIMD_ERR_NOMEM;
    double *dR = d, *dP = dR + n, *dG = dP + n, *dF = dG + n, *dx1 = dF + n, *dx2 = dx1 + n, *dC = dx2 + n,
           *dI = dC + nc, *dE = dI + nd, *dO = dE + nd;
    cudaStream_t st = E.stream;
    cudaMemcpyAsync(dR, RRt, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dP, PPt, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dG, dRRt, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (dRRfast) cudaMemcpyAsync(dF, dRRfast, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (xi1) cudaMemcpyAsync(dx1, xi1, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (xi2) cudaMemcpyAsync(dx2, xi2, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    int rc = pimd_contracted_step_device(ctx, mp, dR, dP, dG, dRRfast ? dF : nullptr, dC, xi1 ? dx1 : nullptr,
                                         xi2 ? dx2 : nullptr, t, dO, dip_momIt ? dI : nullptr, dip_momEt ? dE : nullptr);
    if (rc == PIMD_OK) {
        cudaMemcpyAsync(RRt, dR, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(PPt, dP, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(dRRt, dG, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        if (dRRfast) cudaMemcpyAsync(dRRfast, dF, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        if (RRc) cudaMemcpyAsync(RRc, dC, sizeof(double) * nc, cudaMemcpyDeviceToHost, st);
        if (dip_momIt) cudaMemcpyAsync(dip_momIt, dI, sizeof(double) * nd, cudaMemcpyDeviceToHost, st);
        if (dip_momEt) cudaMemcpyAsync(dip_momEt, dE, sizeof(double) * nd, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(out, dO, sizeof(double) * PIMD_MD_NOUT, cudaMemcpyDeviceToHost, st);
        rc = con_err(E, cudaStreamSynchronize(st), "contracted_step");
    } else {
        cudaStreamSynchronize(st);
    }
    cudaFree(d);
    return rc;
}

}  // extern "C"
