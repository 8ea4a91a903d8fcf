// noalloc.cu -- O-O half neighbour list for one bead without any device allocation.
//
// Some callers cannot let a library call cudaMalloc: a Fortran or C MD driver that owns all
// device memory through its own pool, a host application that forbids allocations after
// start-up (a fixed memory budget per GPU), and code that records CUDA graphs, where
// cudaMalloc is not a stream operation. For them this entry point builds the same list as the
// engine's neighbour step (find_neigh.f90:14-120, bit-identical) from caller-owned input and
// output buffers, and keeps its per-molecule counts and offsets in a fixed file-scope device
// array. That array exists once per GPU that loads the library and lives until exit.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/pimd_gb300.h"
#include "common.cuh"

namespace pimd {

constexpr int NOALLOC_MAXN = 16384;  // molecules (49152 atoms): 128 KB of scratch

// [0, MAXN): per-molecule pair counts; [MAXN, 2 MAXN): exclusive offsets
static __device__ __align__(256) int g_nbr_scratch[2 * NOALLOC_MAXN];

struct NbrArgs {
    const double *RR;  // (3, Natoms), atoms O H H ...
    int N, cap;
    double box[3], boxi[3], rc2;
    int *scratch;      // device address of g_nbr_scratch
    int2 *ij;
    int *npairs;
};

PIMD_D bool within(const double *a, const double *b, const NbrArgs &x) {
    const double dx = min_image_rn(__dsub_rn(a[0], b[0]), x.box[0], x.boxi[0]);
    const double dy = min_image_rn(__dsub_rn(a[1], b[1]), x.box[1], x.boxi[1]);
    const double dz = min_image_rn(__dsub_rn(a[2], b[2]), x.box[2], x.boxi[2]);
    return dot3_rn(dx, dy, dz) < x.rc2;
}

__global__ void __launch_bounds__(128) k_na_count(NbrArgs x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= x.N) return;
    const double *oi = x.RR + 9 * (size_t)i;
    int n = 0;
    for (int j = i + 1; j < x.N; j++) n += within(oi, x.RR + 9 * (size_t)j, x) ? 1 : 0;
    x.scratch[i] = n;  // every count is rewritten: nothing carries over between calls
}

__global__ void __launch_bounds__(1024) k_na_scan(NbrArgs x) {
    __shared__ int part[1024];
    const int nt = blockDim.x, per = (x.N + nt - 1) / nt;
    const int i0 = threadIdx.x * per, i1 = min(x.N, i0 + per);
    int s = 0;
    for (int i = i0; i < i1; i++) s += x.scratch[i];
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
        x.scratch[NOALLOC_MAXN + i] = base;
        base += x.scratch[i];
    }
    if (threadIdx.x == nt - 1) *x.npairs = part[nt - 1];
}

__global__ void __launch_bounds__(128) k_na_fill(NbrArgs x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= x.N) return;
    const double *oi = x.RR + 9 * (size_t)i;
    int o = x.scratch[NOALLOC_MAXN + i];
    for (int j = i + 1; j < x.N; j++)
        if (within(oi, x.RR + 9 * (size_t)j, x)) {
            if (o < x.cap) x.ij[o] = make_int2(i, j);
            o++;
        }
}

// device address of the scratch array, looked up once per device
static int *scratch_address(int *rc) {
    static std::mutex mu;
    static int *addr[64] = {nullptr};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        *rc = PIMD_ERR_CUDA;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_nbr_scratch);
        if (e != cudaSuccess) {
            fprintf(stderr, "pimd_neighbors_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            *rc = PIMD_ERR_CUDA;
            return nullptr;
        }
        addr[dev] = static_cast<int *>(p);
    }
    *rc = PIMD_OK;
    return addr[dev];
}

}  // namespace pimd

using namespace pimd;

extern "C" int pimd_neighbors_noalloc(const double *RR, int natoms, const double *box, double rc, int *ij, int cap,
                                      int *npairs, void *cuda_stream) {
    if (!RR || !box || !ij || !npairs || natoms <= 0 || natoms % 3 || cap < 0 || !(rc > 0)) return PIMD_ERR_ARG;
    for (int c = 0; c < 3; c++)
        if (!std::isfinite(box[c]) || !(box[c] > 0)) {
            fprintf(stderr, "pimd_neighbors_noalloc: box[%d] = %g is not a finite positive length\n", c, box[c]);
            return PIMD_ERR_ARG;
        }
    const int N = natoms / 3;
    if (N > NOALLOC_MAXN) {
        fprintf(stderr, "pimd_neighbors_noalloc: %d molecules exceed the static scratch limit of %d molecules\n", N,
                NOALLOC_MAXN);
        return PIMD_ERR_ARG;
    }
    // an error left pending by earlier, unrelated work is reported as such (and left for its
    // owner to read), so it is not mistaken for a failure of these launches
    const cudaError_t prior = cudaPeekAtLastError();
    if (prior != cudaSuccess) {
        fprintf(stderr, "pimd_neighbors_noalloc: a CUDA error from earlier work is pending: %s\n",
                cudaGetErrorString(prior));
        return PIMD_ERR_CUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    int cur = -1, sdev = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cudaStreamGetDevice(s, &sdev) != cudaSuccess) return PIMD_ERR_CUDA;
    if (sdev != cur) {
        fprintf(stderr, "pimd_neighbors_noalloc: the stream belongs to device %d, the current device is %d\n", sdev,
                cur);
        return PIMD_ERR_ARG;
    }
    int rc_ = PIMD_OK;
    int *scratch = scratch_address(&rc_);
    if (rc_) return rc_;
    NbrArgs x;
    x.RR = RR;
    x.N = N;
    x.cap = cap;
    for (int c = 0; c < 3; c++) {
        x.box[c] = box[c];
        x.boxi[c] = 1.0 / box[c];
    }
    x.rc2 = rc * rc;
    x.scratch = scratch;
    x.ij = reinterpret_cast<int2 *>(ij);
    x.npairs = npairs;
    const int blocks = (N + 127) / 128;
    k_na_count<<<blocks, 128, 0, s>>>(x);
    k_na_scan<<<1, 1024, 0, s>>>(x);
    k_na_fill<<<blocks, 128, 0, s>>>(x);
    return cudaGetLastError() == cudaSuccess ? PIMD_OK : PIMD_ERR_CUDA;
}
