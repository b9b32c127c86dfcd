// FP64 pipe throughput probe: the denominator of the FP64 roofline of the
// MFV kernels (measured HBM-copy and BF16-GEMM peaks give no FP64 figure).
// Independent fused multiply-add chains keep the FP64 pipe busy; one FMA
// counts as two floating-point operations.
#include "../../include/mlh.h"
#include "mlh_device.cuh"

#include <cuda_runtime.h>

namespace {

constexpr int CHAINS = 8;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// clk[0..1]: SM clock cycles and global-timer nanoseconds over the loop of
// block 0, thread 0 (the effective SM clock during the launch)
__global__ void __launch_bounds__(256) k_dfma(double *out, double a, double b, int iters,
                                              unsigned long long *clk) {
    const bool timer = blockIdx.x == 0 && threadIdx.x == 0;
    long long c0 = 0;
    unsigned long long t0 = 0;
    if (timer) { c0 = clock64(); t0 = global_ns(); }
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
    if (timer) {
        clk[0] = (unsigned long long)(clock64() - c0);
        clk[1] = global_ns() - t0;
    }
}

}  // namespace

extern "C" int mlh_probe_fp64_tflops(double seconds, double *tflops) {
    return mlh_probe_fp64_clock(seconds, tflops, nullptr);
}

extern "C" int mlh_probe_fp64_clock(double seconds, double *tflops, double *sm_mhz) {
    if (!tflops) return MLH_ERR_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MLH_ERR_NO_DEVICE;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * 4096 + 2 * sizeof(unsigned long long)) != cudaSuccess)
        return MLH_ERR_CUDA;
    unsigned long long *clk = reinterpret_cast<unsigned long long *>(out + 4096);
    double best_mhz = 0.;
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
        k_dfma<<<blocks, threads>>>(out, 0.999999, 1e-7, iters, clk);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        elapsed_total += ms;
        double flops = 2.0 * CHAINS * (double)iters * blocks * threads;
        double tf = flops / (ms * 1e-3) / 1e12;
        if (ms > 5.f && tf > best) {
            best = tf;
            unsigned long long h[2] = {0, 0};
            cudaMemcpy(h, clk, sizeof(h), cudaMemcpyDeviceToHost);
            best_mhz = h[1] ? (double)h[0] / (double)h[1] * 1e3 : 0.;
        }
        if (ms < 10.f) iters *= 2;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return MLH_ERR_CUDA;
    *tflops = best;
    if (sm_mhz) *sm_mhz = best_mhz;
    return 0;
}

namespace {

__global__ void k_fast_math(int n, const double *__restrict__ x, const double *__restrict__ y,
                            double *__restrict__ rcp, double *__restrict__ quot, double *__restrict__ rsq) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        rcp[i] = mlh::frcp(x[i]);
        quot[i] = mlh::fdiv(y[i], x[i]);
        rsq[i] = mlh::frsqrt(x[i]);
    }
}

__global__ void k_scale2(int n, const double *__restrict__ x, double *__restrict__ half, double *__restrict__ quarter,
                         double *__restrict__ twice) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        half[i] = mlh::scale_down<1>(x[i]);
        quarter[i] = mlh::scale_down<2>(x[i]);
        twice[i] = mlh::twice(x[i]);
    }
}

}  // namespace

// The integer-pipe scalings by 1/2, 1/4 and 2 (mlh_device.cuh: scale_down,
// twice) of host values, for checking them against IEEE products.
extern "C" int mlh_probe_scale2(int n, const double *x, double *half, double *quarter, double *twice) {
    if (n < 0 || (n > 0 && (!x || !half || !quarter || !twice))) return MLH_ERR_INVALID;
    if (n == 0) return 0;
    double *d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * 4 * (size_t)n) != cudaSuccess) return MLH_ERR_CUDA;
    const size_t b = sizeof(double) * (size_t)n;
    cudaError_t e = cudaMemcpy(d, x, b, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_scale2<<<(n + 255) / 256, 256>>>(n, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(half, d + n, b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(quarter, d + 2 * (size_t)n, b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(twice, d + 3 * (size_t)n, b, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? 0 : MLH_ERR_CUDA;
}

// The library's reciprocal, quotient and reciprocal square root
// (mlh_device.cuh: frcp, fdiv, frsqrt) of host arrays, for checking them
// against exact values: rcp = 1/x, quot = y/x, rsqrt = 1/sqrt(x).
extern "C" int mlh_probe_fast_math(int n, const double *x, const double *y, double *rcp, double *quot,
                                   double *rsqrt) {
    if (n < 0 || (n > 0 && (!x || !y || !rcp || !quot || !rsqrt))) return MLH_ERR_INVALID;
    if (n == 0) return 0;
    double *d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * 5 * (size_t)n) != cudaSuccess) return MLH_ERR_CUDA;
    const size_t b = sizeof(double) * (size_t)n;
    cudaError_t e = cudaMemcpy(d, x, b, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, y, b, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_fast_math<<<(n + 255) / 256, 256>>>(n, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n, d + 4 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(rcp, d + 2 * (size_t)n, b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(quot, d + 3 * (size_t)n, b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rsqrt, d + 4 * (size_t)n, b, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? 0 : MLH_ERR_CUDA;
}

namespace {

// k_dfma with the chains run only by the first `active` lanes of each warp
__global__ void __launch_bounds__(256) k_dfma_lanes(double *out, double a, double b, int iters, int active) {
    double acc[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) acc[c] = (double)(threadIdx.x + c) * 1e-9;
    if ((int)(threadIdx.x & 31) < active) {
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int c = 0; c < CHAINS; ++c) acc[c] = fma(acc[c], a, b);
        }
    }
    double s = 0.;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += acc[c];
    if (s == 123.456) out[blockIdx.x] = s;   // never true; keeps the chains live
}

}  // namespace

// Device time of the FMA chains of mlh_probe_fp64_tflops (8 blocks of 256
// threads per SM, `iters` steps of 8 chains) when only the first
// `active_lanes` lanes of every warp run them: how the FP64 pipe charges a
// partially active warp instruction (on GB300 the time does not depend on
// active_lanes, which is why the kernels keep warps convergent around FP64
// code).  The best of three launches after a warm-up.
extern "C" int mlh_probe_fp64_lanes(int active_lanes, int iters, double *ms) {
    if (!ms || active_lanes < 1 || active_lanes > 32 || iters < 1 || iters > (1 << 20)) return MLH_ERR_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MLH_ERR_NO_DEVICE;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * (size_t)blocks) != cudaSuccess) return MLH_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = -1.f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        k_dfma_lanes<<<blocks, threads>>>(out, 0.999999, 1e-7, iters, active_lanes);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && (best < 0.f || t < best)) best = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return MLH_ERR_CUDA;
    *ms = best;
    return 0;
}
