// peak.cu -- CUDA-core FMA throughput probe (FP64 and FP32), the denominator of the roofline
// for kernels that are bound by the FP64 or FP32 pipe rather than HBM or tensor cores.
#include "../../include/pimd_gb300.h"
#include "engine.h"

namespace pimd {

template <typename T, int CH>
__global__ void __launch_bounds__(256) k_fma_peak(T *out, int iters, T a, T b) {
    T x[CH];
#pragma unroll
    for (int c = 0; c < CH; c++) x[c] = (T)(threadIdx.x + c);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < CH; c++) x[c] = fma(x[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < CH; c++) s += x[c];
    if (s == (T)-1.2345) out[threadIdx.x] = s;  // keeps the loop alive
}

}  // namespace pimd

using namespace pimd;

extern "C" int pimd_peak_flops(int device, int fp64, double *tflops) {
    if (!tflops) return PIMD_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return PIMD_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    void *out;
    if (cudaMalloc(&out, 1024 * sizeof(double)) != cudaSuccess) return PIMD_ERR_NOMEM;
    const int blocks = sms * 8, threads = 256;
    const int iters = fp64 ? 4096 : 65536;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        if (fp64)
            k_fma_peak<double, 8><<<blocks, threads>>>((double *)out, iters, 0.999999, 1e-7);
        else
            k_fma_peak<float, 8><<<blocks, threads>>>((float *)out, iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return PIMD_ERR_CUDA;
    const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return PIMD_OK;
}
