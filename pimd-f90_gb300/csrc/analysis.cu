// analysis.cu -- the run analyses of PIMD-F90 on the device: water geometry and O-H histograms
// (geometry_calculator.f90), the mean-square displacement and diffusion constant
// (diffusion_calculator.f90), and the IR spectrum and the density of states from stored dipole
// and velocity time series (spectral_properties.f90 with math.f90:42-140), the transforms by cuFFT
// (single precision, as the reference's four1.f works on REAL data) in place of four1.
//
// Accumulators live in the context: a geometry accumulator (176 doubles, the layout of the
// reference's module variables), an MSD state, and the spectra's time series. The per-step calls
// are stream-ordered on the context's stream; the reports copy back and finish on the host.
// cuFFT is opened at the first spectrum call (dlopen), so the library does not depend on it
// otherwise.
#include <dlfcn.h>

#include <cmath>
#include <cstring>
#include <vector>

#include <cufft.h>

#include "../../include/pimd_gb300.h"
#include "engine.h"

namespace pimd {

constexpr int GEO_NB = 80, GEO_N = 176;
constexpr int MSD_TOUT = 20;

// default-real literals .6 and 1.6 of geometry_calculator.f90:3-5, and the bin width
PIMD_HD double geo_min() { return (double)0.6f; }
PIMD_HD double geo_max() { return (double)1.6f; }

// geometry_calculator.f90:235-259 binit (normal binning), atomically
PIMD_D void geo_binit(double *hist, double x) {
    const double lo = geo_min(), hi = geo_max(), delta = (hi - lo) / GEO_NB;
    if (x > lo && x < hi) {
        int bin = (int)round(__ddiv_rn(__dsub_rn(x, lo), delta));
        if (bin == 0) bin = 1;
        if (bin > GEO_NB) bin = GEO_NB;
        atomicAdd(hist + bin - 1, 1.0);
    }
}

PIMD_D void atomic_max_pos(double *a, double v) {  // non-negative doubles order as their bits
    atomicMax(reinterpret_cast<unsigned long long *>(a), (unsigned long long)__double_as_longlong(v));
}

// calc_geometry (geometry_calculator.f90:21-125) for one frame: one thread per (molecule, pass),
// pass 0 the centroid, 1..P the beads. The centroid pass leaves (d_OH1, d_OH2) of each molecule
// in dcen for the sequential maximum (k_geometry_cmax).
__global__ void k_geometry(double *acc, double *dcen, int natoms, int P, double3 box, double3 boxi, const double *RR,
                           const double *RRt) {
    const int nw = natoms / 3;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, pass = blockIdx.y;
    if (i >= nw) return;
    const double *X = pass == 0 ? RR : RRt + (size_t)3 * natoms * (pass - 1);
    const double *rO = X + 9 * (size_t)i, *rH2 = rO + 3, *rH1 = rO + 6;
    const double b[3] = {box.x, box.y, box.z}, bi[3] = {boxi.x, boxi.y, boxi.z};
    double R1[3], R2[3], RH[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        R1[c] = min_image_rn(__dsub_rn(rO[c], rH1[c]), b[c], bi[c]);
        R2[c] = min_image_rn(__dsub_rn(rO[c], rH2[c]), b[c], bi[c]);
        RH[c] = min_image_rn(__dsub_rn(rH2[c], rH1[c]), b[c], bi[c]);
    }
    // every product and sum rounded separately (as the oracle's), so the distances, and with them
    // the histogram bins and the maxima, are the reference's bit for bit
    const double dHH = sqrt(dot3_rn(RH[0], RH[1], RH[2]));
    const double d1 = sqrt(dot3_rn(R1[0], R1[1], R1[2]));
    const double d2 = sqrt(dot3_rn(R2[0], R2[1], R2[2]));
    const double dHOH = acos(__ddiv_rn(__dsub_rn(__dadd_rn(__dmul_rn(d1, d1), __dmul_rn(d2, d2)), __dmul_rn(dHH, dHH)),
                                       __dmul_rn(__dmul_rn(2.0, d1), d2)));
    const double dOHmax = 1.5;
    const int nwarn = (d1 > dOHmax) + (d2 > dOHmax);
    if (nwarn) atomicAdd(acc + 15, (double)nwarn);
    double *sm = acc + (pass == 0 ? 0 : 6);
    if (pass == 0) {
        dcen[2 * i] = d1;
        dcen[2 * i + 1] = d2;
        geo_binit(acc + 16, d1);
        geo_binit(acc + 16, d2);
    } else {
        atomic_max_pos(acc + 13, fmax(d1, d2));
        geo_binit(acc + 96, d1);
        geo_binit(acc + 96, d2);
    }
    atomicAdd(sm + 0, dHH);
    atomicAdd(sm + 1, d1 + d2);
    if (pass == 0 || fabs(dHOH) > 0) atomicAdd(sm + 2, dHOH);
    atomicAdd(sm + 3, dHH * dHH);
    atomicAdd(sm + 4, d1 * d1 + d2 * d2);
    atomicAdd(sm + 5, dHOH * dHOH);
}

// the centroid maximum in molecule order, as the reference's two ifs update it (the second takes
// d_OH1 when d_OH2 exceeds the running maximum, geometry_calculator.f90:57-58), and num_total
__global__ void k_geometry_cmax(double *acc, const double *dcen, int nw) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double m = acc[12];
    for (int i = 0; i < nw; i++) {
        const double d1 = dcen[2 * i], d2 = dcen[2 * i + 1];
        if (d1 > m) m = d1;
        if (d2 > m) m = d1;
    }
    acc[12] = m;
    acc[14] += nw;
}

// calc_diff_RMSD (diffusion_calculator.f90:14-58) for one frame, one block: state = [t,
// initialised, aMS(ntimes + 1), netdisp(3 Nw), Oxy(3 Nw)]; the tracked atom of molecule ia is atom
// 3 ia (1-based), as the reference's Oxy2(:,ia) = RRc(:,3*ia) takes it
__global__ void k_msd_step(double *st, int natoms, int ntimes, double box0, double boxi0, const double *RRc) {
    const int nw = natoms / 3;
    double *aMS = st + 2, *net = aMS + ntimes + 1, *Oxy = net + 3 * nw;
    __shared__ int t_sh;
    __shared__ bool first;
    __shared__ double red[32];
    if (threadIdx.x == 0) {
        first = st[1] == 0;
        st[0] = first ? 0.0 : st[0] + 1.0;
        st[1] = 1.0;
        t_sh = (int)st[0];
    }
    __syncthreads();
    double s = 0.0;
    for (int k = threadIdx.x; k < 3 * nw; k += blockDim.x) {
        const int i = k / 3, c = k % 3;
        const double o2 = RRc[3 * (3 * i + 2) + c];
        if (first) Oxy[k] = o2;
        double d = __dsub_rn(o2, Oxy[k]);
        d = __dsub_rn(d, __dmul_rn(box0, round(__dmul_rn(d, boxi0))));
        net[k] = __dadd_rn(net[k], d);
        Oxy[k] = o2;
        s += net[k] * net[k];
    }
    const int t = t_sh;
    if (t % MSD_TOUT != 0) return;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
        const int ti = t / MSD_TOUT + 1;
        if (ti <= ntimes + 1) aMS[ti - 1] = (aMS[ti - 1] + tot) / nw;
    }
}

// one frame of the spectra's time series (InputOutput.f90:680-688): the total dipole in Debye,
// sum over molecules of the bead-averaged dipoles (write_out's dip_mom, InputOutput.f90:578-590),
// and the centroid "H" velocities: slot 2i the first H's, slot 2i - 1 the O atom's momentum over
// massH, as the reference stores them
__global__ void k_spectra_record(int natoms, int P, double massH, const double *dipIt, const double *PPt,
                                 float *dip, float *hvel, int tr, int nmax) {
    const int nw = natoms / 3;
    __shared__ double red[3][32];
    double d[3] = {0.0, 0.0, 0.0};
    for (int iw = threadIdx.x; iw < nw; iw += blockDim.x) {
        if (dipIt)
            for (int c = 0; c < 3; c++) {
                double s = 0.0;
                for (int j = 0; j < P; j++) s = s + dipIt[c + 3 * (size_t)iw + (size_t)3 * nw * j] * DEBYE / CHARGECON;
                d[c] += s / P;
            }
        if (hvel) {
            const double imassH = 1.0 / massH;
            for (int a = 0; a < 2; a++) {  // a 0: atom 3i-2 (O) into slot 2i-1; a 1: atom 3i-1 (H1) into slot 2i
                const int atom = 3 * iw + a, slot = 2 * iw + a;
                for (int c = 0; c < 3; c++) {
                    double s = 0.0;
                    for (int j = 0; j < P; j++) s = s + PPt[c + 3 * (size_t)atom + (size_t)3 * natoms * j];
                    hvel[c + 3 * ((size_t)tr + (size_t)nmax * slot)] = (float)((s / P) * imassH);
                }
            }
        }
    }
    if (!dipIt) return;
    for (int c = 0; c < 3; c++) {
        double v = d[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[c][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double tot = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[threadIdx.x][w];
        dip[threadIdx.x + 3 * tr] = (float)tot;
    }
}

// z -> z conj(z) (the autocorrelation's transform), and z -> (Re z, 0)
__global__ void k_power(cufftComplex *z, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const cufftComplex v = z[i];
        z[i] = make_float2(v.x * v.x + v.y * v.y, 0.0f);
    }
}

// --- cuFFT, opened at first use ---------------------------------------------------------------
struct CufftApi {
    void *h = nullptr;
    cufftResult (*planMany)(cufftHandle *, int, int *, int *, int, int, int *, int, int, cufftType, int) = nullptr;
    cufftResult (*execC2C)(cufftHandle, cufftComplex *, cufftComplex *, int) = nullptr;
    cufftResult (*setStream)(cufftHandle, cudaStream_t) = nullptr;
    cufftResult (*destroy)(cufftHandle) = nullptr;
};
static CufftApi *cufft_api() {
    static CufftApi api;
    static bool tried = false;
    if (!tried) {
        tried = true;
        const char *names[] = {"libcufft.so.12", "libcufft.so.13", "libcufft.so"};
        for (const char *nm : names)
            if ((api.h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
        if (api.h) {
            api.planMany = reinterpret_cast<decltype(api.planMany)>(dlsym(api.h, "cufftPlanMany"));
            api.execC2C = reinterpret_cast<decltype(api.execC2C)>(dlsym(api.h, "cufftExecC2C"));
            api.setStream = reinterpret_cast<decltype(api.setStream)>(dlsym(api.h, "cufftSetStream"));
            api.destroy = reinterpret_cast<decltype(api.destroy)>(dlsym(api.h, "cufftDestroy"));
        }
    }
    return (api.planMany && api.execC2C && api.setStream && api.destroy) ? &api : nullptr;
}

// batched in-place C2C transforms of length n on the stream; four1's isign = 1 is cuFFT's
// inverse direction (exp(+2 pi i jk/n)), -1 its forward one, neither normalised
static int fft_batch(Engine &E, cufftComplex *d, int n, int batch, int isign) {
    CufftApi *f = cufft_api();
    if (!f) {
        E.last_error = "spectra: cuFFT (libcufft) could not be opened";
        return PIMD_ERR_CUDA;
    }
    cufftHandle plan;
    int nn[1] = {n};
    if (f->planMany(&plan, 1, nn, nullptr, 1, n, nullptr, 1, n, CUFFT_C2C, batch) != CUFFT_SUCCESS) {
        E.last_error = "spectra: cufftPlanMany failed";
        return PIMD_ERR_CUDA;
    }
    f->setStream(plan, E.stream);
    const cufftResult r = f->execC2C(plan, d, d, isign > 0 ? CUFFT_INVERSE : CUFFT_FORWARD);
    cudaStreamSynchronize(E.stream);
    f->destroy(plan);
    if (r != CUFFT_SUCCESS) {
        E.last_error = "spectra: cufftExecC2C failed";
        return PIMD_ERR_CUDA;
    }
    return PIMD_OK;
}

static int pow2_floor_log(int n, int add) { return 1 << ((int)std::floor(std::log((double)n) / std::log(2.0)) + add); }

static int an_err(Engine &E, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PIMD_OK;
    E.last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return PIMD_ERR_CUDA;
}

// math.f90:123-140 block_average
static void block_average(const double *in, int n, int N, double *out) {
    const int bs = (int)std::floor((float)n / (float)N);
    if (bs == 0) {
        for (int i = 0; i < N && i < n; i++) out[i] = in[i];
        return;
    }
    for (int i = 0; i < N; i++) {
        double s = 0;
        for (int k = i * bs; k < (i + 1) * bs; k++) s += in[k];
        out[i] = s / bs;
    }
}

}  // namespace pimd

using namespace pimd;

extern "C" {

int pimd_geometry_reset(pimd_ctx *ctx) {
    if (!ctx) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        cudaSetDevice(E.device);
    if (!ctx->an_geo) {
        if (cudaMalloc((void **)&ctx->an_geo, sizeof(double) * (GEO_N + 2 * (size_t)E.kp.N)) != cudaSuccess)
            return PIMD_ERR_NOMEM;
        E.allocs.push_back(ctx->an_geo);
        ctx->an_dcen = ctx->an_geo + GEO_N;
    }
    return an_err(E, cudaMemsetAsync(ctx->an_geo, 0, sizeof(double) * GEO_N, E.stream), "geometry_reset");
}

int pimd_geometry_accumulate_device(pimd_ctx *ctx, const double *RRc, const double *RRt) {
    if (!ctx || !RRc || !RRt) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        if (!ctx->an_geo) return PIMD_ERR_STATE;
    cudaSetDevice(E.device);
    const int nw = E.kp.N;
    const dim3 g((nw + 127) / 128, E.kp.P + 1);
    k_geometry<<<g, 128, 0, E.stream>>>(ctx->an_geo, ctx->an_dcen, E.kp.natoms, E.kp.P,
                                       make_double3(E.kp.box[0], E.kp.box[1], E.kp.box[2]),
                                       make_double3(E.kp.boxi[0], E.kp.boxi[1], E.kp.boxi[2]), RRc, RRt);
    k_geometry_cmax<<<1, 32, 0, E.stream>>>(ctx->an_geo, ctx->an_dcen, nw);
    E.nlaunch += 2;
    return an_err(E, cudaGetLastError(), "geometry_accumulate");
}

int pimd_geometry_report(pimd_ctx *ctx, double *out, double *hist_c, double *hist_b, double *counts) {
    if (!ctx || !out) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        if (!ctx->an_geo) return PIMD_ERR_STATE;
    cudaSetDevice(E.device);
    double acc[GEO_N];
    cudaError_t e = cudaStreamSynchronize(E.stream);
    if (e == cudaSuccess) e = cudaMemcpy(acc, ctx->an_geo, sizeof acc, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return an_err(E, e, "geometry_report");
    // write_out_geometry (geometry_calculator.f90:129-190)
    const double nt = acc[14], bn = nt * E.kp.P, deg = 180.0 / 3.141592;
    for (int b = 0; b < 2; b++) {
        const double *sm = acc + 6 * b;
        const double n = b ? bn : nt;
        const double aHH = sm[0] / n, aOH = sm[1] / (2.0 * n), aHOH = (sm[2] / n) * deg;
        const double aHH2 = sm[3] / n, aOH2 = sm[4] / (2.0 * n), aHOH2 = (sm[5] / n) * (deg * deg);
        out[6 * b + 0] = aHH;
        out[6 * b + 1] = std::sqrt(aHH2 - aHH * aHH);
        out[6 * b + 2] = aOH;
        out[6 * b + 3] = std::sqrt(aOH2 - aOH * aOH);
        out[6 * b + 4] = aHOH;
        out[6 * b + 5] = std::sqrt(aHOH2 - aHOH * aHOH);
    }
    out[12] = acc[12];
    out[13] = acc[13];
    // write_out_histogram (geometry_calculator.f90:192-205): bin ends and normalised counts
    const double delta = (geo_max() - geo_min()) / GEO_NB;
    for (int i = 0; i < GEO_NB; i++) {
        if (hist_c) {
            hist_c[2 * i] = geo_min() + delta * (i + 1);
            hist_c[2 * i + 1] = acc[16 + i] / (2 * nt);
        }
        if (hist_b) {
            hist_b[2 * i] = geo_min() + delta * (i + 1);
            hist_b[2 * i + 1] = acc[96 + i] / (2 * nt * E.kp.P);
        }
    }
    if (counts) std::memcpy(counts, acc, sizeof acc);
    return PIMD_OK;
}

int pimd_msd_init(pimd_ctx *ctx, int num_timesteps) {
    if (!ctx || num_timesteps < MSD_TOUT) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        cudaSetDevice(E.device);
    const int ntimes = (int)std::floor((float)num_timesteps / (float)MSD_TOUT);
    const size_t n = 2 + (size_t)ntimes + 1 + 6 * (size_t)E.kp.N;
    if (ctx->an_msd && ctx->an_msd_ntimes != ntimes) ctx->an_msd = nullptr;  // the old buffer stays with the context's allocations
    if (!ctx->an_msd) {
        if (cudaMalloc((void **)&ctx->an_msd, sizeof(double) * n) != cudaSuccess) return PIMD_ERR_NOMEM;
        E.allocs.push_back(ctx->an_msd);
    }
    ctx->an_msd_ntimes = ntimes;
    return an_err(E, cudaMemsetAsync(ctx->an_msd, 0, sizeof(double) * n, E.stream), "msd_init");
}

int pimd_msd_accumulate_device(pimd_ctx *ctx, const double *RRc) {
    if (!ctx || !RRc) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        if (!ctx->an_msd) return PIMD_ERR_STATE;
    cudaSetDevice(E.device);
    k_msd_step<<<1, 1024, 0, E.stream>>>(ctx->an_msd, E.kp.natoms, ctx->an_msd_ntimes, E.kp.box[0], E.kp.boxi[0], RRc);
    ++E.nlaunch;
    return an_err(E, cudaGetLastError(), "msd_accumulate");
}

int pimd_msd_report(pimd_ctx *ctx, double timestep, double *aMS, int *ntimes, double *out4) {
    if (!ctx || !out4) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        if (!ctx->an_msd) return PIMD_ERR_STATE;
    cudaSetDevice(E.device);
    const int nt = ctx->an_msd_ntimes;
    std::vector<double> a(nt + 1);
    cudaError_t e = cudaStreamSynchronize(E.stream);
    if (e == cudaSuccess) e = cudaMemcpy(a.data(), ctx->an_msd + 2, sizeof(double) * (nt + 1), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return an_err(E, e, "msd_report");
    if (aMS) std::memcpy(aMS, a.data(), sizeof(double) * nt);
    if (ntimes) *ntimes = nt;
    // write_out_diffusion (diffusion_calculator.f90:60-118)
    const float frac = 0.5f;
    std::vector<float> times(nt);
    for (int i = 1; i <= nt; i++) times[i - 1] = (float)(i * MSD_TOUT * timestep);
    const int ft = (int)std::floor(frac * nt) + 1, nfit = nt - ft;
    if (nfit < 3) return PIMD_ERR_STATE;
    double xbar = 0, ybar = 0, sx = 0, sy = 0, cr = 0;
    for (int i = ft; i <= nt; i++) xbar += (double)(times[i - 1] / (float)(nfit - 1));
    for (int i = ft; i <= nt; i++) ybar += a[i - 1] / (nfit - 1);
    for (int i = ft; i <= nt; i++) {
        sx += ((double)times[i - 1] - xbar) * ((double)times[i - 1] - xbar);
        sy += (a[i - 1] - ybar) * (a[i - 1] - ybar);
        cr += (a[i - 1] - ybar) * ((double)times[i - 1] - xbar);
    }
    const double b = cr / sx, icpt = ybar - b * xbar;
    const double errb = std::sqrt((sy / sx - b * b) / (nfit - 2));
    out4[0] = 10 * b / 6;
    out4[1] = errb / 6;
    out4[2] = b;
    out4[3] = icpt;
    return PIMD_OK;
}

int pimd_spectra_init(pimd_ctx *ctx, int max_steps, double massH) {
    if (!ctx || max_steps < 2 || !(massH > 0)) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        cudaSetDevice(E.device);
    if (ctx->an_nmax != max_steps) {
        const size_t n = 3 * (size_t)max_steps * (1 + 2 * (size_t)E.kp.N);
        float *p = nullptr;
        if (cudaMalloc((void **)&p, sizeof(float) * n) != cudaSuccess) return PIMD_ERR_NOMEM;
        E.allocs.push_back(p);
        ctx->an_dip = p;
        ctx->an_hvel = p + 3 * (size_t)max_steps;
        ctx->an_nmax = max_steps;
    }
    ctx->an_n = 0;
    ctx->an_massH = massH;
    return PIMD_OK;
}

int pimd_spectra_record_device(pimd_ctx *ctx, const double *dip_momIt, const double *PPt) {
    if (!ctx || (!dip_momIt && !PPt)) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        if (!ctx->an_dip) return PIMD_ERR_STATE;
    if (ctx->an_n >= ctx->an_nmax) {
        E.last_error = "spectra_record: the series is full (pimd_spectra_init's max_steps)";
        return PIMD_ERR_ARG;
    }
    cudaSetDevice(E.device);
    k_spectra_record<<<1, 256, 0, E.stream>>>(E.kp.natoms, E.kp.P, ctx->an_massH, dip_momIt, PPt, dip_momIt ? ctx->an_dip : nullptr,
                                              PPt ? ctx->an_hvel : nullptr, ctx->an_n, ctx->an_nmax);
    ++E.nlaunch;
    ctx->an_n++;
    return an_err(E, cudaGetLastError(), "spectra_record");
}

// calc_infrared_spectrum (spectral_properties.f90:10-123)
int pimd_ir_spectrum(pimd_ctx *ctx, double timestep, double temp, int *npoints, double *freq, double *ir) {
    if (!ctx || !npoints || !freq || !ir || *npoints < 1) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        if (!ctx->an_dip || ctx->an_n < 2) return PIMD_ERR_STATE;
    cudaSetDevice(E.device);
    const double ps2s = 1e-12, Cspeed = 3.00e10, Debye2SI = 3.33564e-30, eps0 = 8.854187e-12, kb = 0.0019872041;
    const double vol = (E.kp.box[0] * E.kp.box[1] * E.kp.box[2]) * 1e-30;
    const int tread = ctx->an_n, trun = pow2_floor_log(tread, 0), n = 2 * trun;
    std::vector<float> hd(3 * (size_t)tread);
    cudaError_t e = cudaStreamSynchronize(E.stream);
    if (e == cudaSuccess) e = cudaMemcpy(hd.data(), ctx->an_dip, sizeof(float) * 3 * tread, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return an_err(E, e, "ir_spectrum");
    std::vector<cufftComplex> h(3 * (size_t)n, make_float2(0.f, 0.f));  // three zero-padded series
    for (int ix = 0; ix < 3; ix++)
        for (int i = 0; i < trun; i++) h[(size_t)ix * n + i].x = hd[ix + 3 * (size_t)i];
    cufftComplex *d = nullptr;
    if (cudaMalloc((void **)&d, sizeof(cufftComplex) * 3 * n) != cudaSuccess) return PIMD_ERR_NOMEM;
    int rc = PIMD_OK;
    cudaMemcpy(d, h.data(), sizeof(cufftComplex) * 3 * n, cudaMemcpyHostToDevice);
    if (!(rc = fft_batch(E, d, n, 3, -1))) {
        k_power<<<(3 * n + 255) / 256, 256, 0, E.stream>>>(d, 3 * (size_t)n);
        rc = fft_batch(E, d, n, 3, 1);
    }
    if (!rc) {
        cudaMemcpy(h.data(), d, sizeof(cufftComplex) * 3 * n, cudaMemcpyDeviceToHost);
        for (int i = 0; i < n; i++) {  // ACF = sum over the components, complex as it is
            h[i].x = (h[i].x + h[n + i].x) + h[2 * n + i].x;
            h[i].y = (h[i].y + h[n + i].y) + h[2 * n + i].y;
        }
        cudaMemcpy(d, h.data(), sizeof(cufftComplex) * n, cudaMemcpyHostToDevice);
        rc = fft_batch(E, d, n, 1, -1);
    }
    if (!rc) cudaMemcpy(h.data(), d, sizeof(cufftComplex) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (rc) return rc;
    const double MinFreqOut = 1.0 / (timestep * ps2s * Cspeed * n);
    const double avail = std::floor(7000.0 / MinFreqOut);
    int navg;
    if (avail < *npoints) {
        *npoints = (int)avail;
        navg = 1;
    } else {
        navg = (int)std::floor(avail / *npoints);
    }
    for (int t = 0; t < *npoints; t++) {
        double avg = 0;
        for (int i = 1; i <= navg; i++) {
            const double omega = (t * navg + i) / (timestep * n * ps2s);
            const int k = t * navg + i;
            avg = avg + (omega * omega) * (double)(k < n ? h[k].x : 0.0f);
        }
        avg = avg / (double)(float)navg;
        double IR = (2.0 * 3.14159 * (Debye2SI * Debye2SI) * avg) / (3.0 * vol * 2.99e8 * kb * temp * eps0);
        IR = IR * ps2s * .01 * 2;
        freq[t] = (std::floor((t + .5f) * navg) / (timestep * n * ps2s)) / Cspeed;
        ir[t] = IR;
    }
    return PIMD_OK;
}

// calc_DOS (spectral_properties.f90:128-187) with calc_corr_function and calc_DFT (math.f90:45-116)
int pimd_dos(pimd_ctx *ctx, double timestep, int *npoints, double *freq, double *dos) {
    if (!ctx || !npoints || !freq || !dos || *npoints < 1) return PIMD_ERR_ARG;
    Engine &E = ctx->E;
        if (!ctx->an_hvel || ctx->an_n < 3) return PIMD_ERR_STATE;
    cudaSetDevice(E.device);
    const double ps2s = 1e-12, Cspeed = 3.00e10;
    const int tread = ctx->an_n, nhyd = 2 * E.kp.N, trun = pow2_floor_log(tread, 1), n = 2 * trun;
    const int batch = 3 * nhyd;
    std::vector<float> hv(3 * (size_t)ctx->an_nmax * nhyd);
    cudaError_t e = cudaStreamSynchronize(E.stream);
    if (e == cudaSuccess) e = cudaMemcpy(hv.data(), ctx->an_hvel, sizeof(float) * hv.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return an_err(E, e, "dos");
    std::vector<cufftComplex> h((size_t)batch * n, make_float2(0.f, 0.f));
    for (int iH = 0; iH < nhyd; iH++)
        for (int ix = 0; ix < 3; ix++)
            for (int i = 0; i < tread; i++)
                h[((size_t)iH * 3 + ix) * n + i].x = hv[ix + 3 * ((size_t)i + (size_t)ctx->an_nmax * iH)];
    cufftComplex *d = nullptr;
    if (cudaMalloc((void **)&d, sizeof(cufftComplex) * h.size()) != cudaSuccess) return PIMD_ERR_NOMEM;
    int rc = PIMD_OK;
    cudaMemcpy(d, h.data(), sizeof(cufftComplex) * h.size(), cudaMemcpyHostToDevice);
    if (!(rc = fft_batch(E, d, n, batch, 1))) {
        k_power<<<(unsigned)std::min<size_t>((h.size() + 255) / 256, 65535), 256, 0, E.stream>>>(d, h.size());
        rc = fft_batch(E, d, n, batch, -1);
    }
    std::vector<double> ACF(tread, 0.0);
    if (!rc) {
        cudaMemcpy(h.data(), d, sizeof(cufftComplex) * h.size(), cudaMemcpyDeviceToHost);
        std::vector<double> out(tread);
        for (int b = 0; b < batch; b++) {  // calc_corr_function's normalisation, then the sum
            for (int i = 0; i < tread; i++) out[i] = (double)h[(size_t)b * n + i].x;
            for (int i = 1; i <= tread - 1; i++) out[i - 1] = out[i - 1] / (tread - i);
            for (int i = 0; i < tread; i++) ACF[i] = ACF[i] + out[i];
        }
        const double a0 = ACF[0];
        for (int i = 0; i < tread; i++) ACF[i] = ACF[i] / nhyd / a0;
        // calc_DFT
        std::vector<cufftComplex> t1(n, make_float2(0.f, 0.f));
        for (int i = 0; i < tread; i++) t1[i].x = (float)ACF[i];
        cudaMemcpy(d, t1.data(), sizeof(cufftComplex) * n, cudaMemcpyHostToDevice);
        rc = fft_batch(E, d, n, 1, 1);
        if (!rc) cudaMemcpy(t1.data(), d, sizeof(cufftComplex) * n, cudaMemcpyDeviceToHost);
        if (!rc) {
            std::vector<double> DFT(tread), fr(tread);
            for (int i = 0; i < tread; i++) {
                DFT[i] = (double)t1[i].x / (2.0 * trun);
                fr[i] = (double)i / (timestep * 2.0 * trun) / (ps2s * Cspeed);
            }
            const int avail = std::min(tread, (int)std::floor(7000.0 / fr[1]));
            if (avail < *npoints) *npoints = avail;
            block_average(fr.data(), avail, *npoints, freq);
            block_average(DFT.data(), avail, *npoints, dos);
        }
    }
    cudaFree(d);
    return rc;
}

}  // extern "C"
