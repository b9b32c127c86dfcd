// FP64 pipe throughput probe: the denominator of the FP64 roofline of the
// MFV kernels (the measured peaks cover HBM copy and BF16 GEMM only).
// Independent fused multiply-add chains keep the FP64 pipe busy; one FMA
// counts as two floating-point operations.
#include "../../include/mlh.h"

#include <cuda_runtime.h>

namespace {

constexpr int CHAINS = 8;

__global__ void __launch_bounds__(256) k_dfma(double *out, double a, double b, int iters) {
    double acc[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) acc[c] = (double)(threadIdx.x + c) * 1e-9;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) acc[c] = fma(acc[c], a, b);
    }
    double s = 0.;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += acc[c];
    if (s == 123.456) out[blockIdx.x] = s;   // never true; keeps the chains live
}

}  // namespace

extern "C" int mlh_probe_fp64_tflops(double seconds, double *tflops) {
    if (!tflops) return MLH_ERR_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MLH_ERR_NO_DEVICE;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * 4096) != cudaSuccess) return MLH_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    int iters = 4096;
    double best = 0.;
    double elapsed_total = 0.;
    // warm up, then grow the loop until a launch takes ~10 ms, then repeat
    for (int rep = 0; rep < 64 && elapsed_total < seconds * 1e3; ++rep) {
        cudaEventRecord(e0);
        k_dfma<<<blocks, threads>>>(out, 0.999999, 1e-7, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        elapsed_total += ms;
        double flops = 2.0 * CHAINS * (double)iters * blocks * threads;
        double tf = flops / (ms * 1e-3) / 1e12;
        if (ms > 5.f && tf > best) best = tf;
        if (ms < 10.f) iters *= 2;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return MLH_ERR_CUDA;
    *tflops = best;
    return 0;
}
