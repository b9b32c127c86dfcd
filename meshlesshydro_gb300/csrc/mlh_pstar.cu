// Learned initial guess for the Riemann star pressure p*.
//
// A 4-64-64-64-1 MLP with SiLU maps dimensionless left/right states of a face
// to a correction y = log(p* / p_TR) of the two-rarefaction guess p_TR (Toro
// eq. 4.46; the network itself only sees x and y).  Inputs (left = particle i,
// right = neighbour j, after rotation into the face frame):
//   x0 = log(rhoR/rhoL), x1 = (uR - uL)/cL, x2 = log(pR/pL), x3 = log(cR/cL)
// (the ratios enter as logarithms so that shock-strength ratios of 1e6 stay in
// range).  Weights are BF16 on the tensor cores with FP32 accumulation
// (mma.sync m16n8k16); the FP32 master copy, the gradients and Adam's moments
// are FP32.  The guess only seeds the exact Newton iteration of the face
// kernel, which falls back to the two-rarefaction guess if it does not
// converge.  This network has no counterpart in the reference.
//
// Parameter layout (8705 floats): W1[64][4], b1[64], W2[64][64], b2[64],
// W3[64][64], b3[64], W4[64], b4[1]  (W[out][in]).
#include "../../include/mlh.h"
#include "mlh_kernels.h"
#include "mlh_pstar.h"
#include "mlh_mlp.cuh"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace mlh {

// ------------------------------------------------------------------ packed weights

__global__ void k_pack_mlp(const float *__restrict__ prm, PackedMlp *__restrict__ pk) {
    const float *W1 = prm, *b1 = W1 + 256, *W2 = b1 + 64, *b2 = W2 + 4096, *W3 = b2 + 64, *b3 = W3 + 4096,
                *W4 = b3 + 64, *b4 = W4 + 64;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 64 * W_LD; k += gridDim.x * blockDim.x) {
        const int r = k / W_LD, c = k % W_LD;
        if (k < 64 * W1_LD) {
            const int r1 = k / W1_LD, c1 = k % W1_LD;
            pk->w1[k] = __float2bfloat16(c1 < 4 ? W1[r1 * 4 + c1] : 0.f);
        }
        pk->w2[k] = __float2bfloat16(c < 64 ? W2[r * 64 + c] : 0.f);
        pk->w3[k] = __float2bfloat16(c < 64 ? W3[r * 64 + c] : 0.f);
        pk->w2t[k] = __float2bfloat16(c < 64 ? W2[c * 64 + r] : 0.f);
        pk->w3t[k] = __float2bfloat16(c < 64 ? W3[c * 64 + r] : 0.f);
    }
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 64; k += gridDim.x * blockDim.x) {
        pk->b1[k] = b1[k];
        pk->b2[k] = b2[k];
        pk->b3[k] = b3[k];
        pk->w4[k] = W4[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) pk->b4 = b4[0];
}

__device__ __forceinline__ void load_packed(PackedMlp *s, const PackedMlp *g) {
    const int4 *src = reinterpret_cast<const int4 *>(g);
    int4 *dst = reinterpret_cast<int4 *>(s);
    for (int k = threadIdx.x; k < (int)(sizeof(PackedMlp) / 16); k += blockDim.x) dst[k] = src[k];
    __syncthreads();
}

// ------------------------------------------------------------------ inference

// y = MLP(x) for n rows; one warp per 32 rows (grid-stride, warp-uniform).
__global__ void __launch_bounds__(256) k_pstar_infer(const float4 *__restrict__ x, int n, const int *__restrict__ n_dev,
                                                     const PackedMlp *__restrict__ pk, float *__restrict__ y) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PackedMlp *s = reinterpret_cast<PackedMlp *>(smem_raw);
    load_packed(s, pk);
    if (n_dev && *n_dev < n) n = *n_dev;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int r0 = gw * 32; r0 < n; r0 += nw * 32) {
        const int r = r0 + lane;
        const float4 xi = r < n ? x[r] : make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t a0[2][1][4];
        input_frags<2>(xi, a0);
        Acc64 acc;
        uint32_t a[2][4][4];
        layer_mma<2, 1>(acc, a0, s->w1, W1_LD, s->b1);
        acc_to_a(acc, a, silu);
        layer_mma<2, 4>(acc, a, s->w2, W_LD, s->b2);
        acc_to_a(acc, a, silu);
        layer_mma<2, 4>(acc, a, s->w3, W_LD, s->b3);
        const float out = output_row(acc, s->w4, s->b4);
        if (r < n) y[r] = out;
    }
}

// ------------------------------------------------------------------ training

// One block = 4 warps = 128 samples: forward with the activations kept in
// shared memory, loss gradient, backward through the layers (dh = dz W on the
// tensor cores), and this block's share of the weight gradients
// dW = dz^T h (tensor cores over the block's 128 samples), written as a
// per-block partial; k_pstar_reduce sums the partials in a fixed order.
constexpr int TB = 128;              // samples per block
constexpr int T_LD = TB + 8;         // stride of the transposed [feature][sample] tiles
constexpr int NPRM = 8705;

struct TrainSmem {
    PackedMlp w;
    __nv_bfloat16 xT[16 * T_LD];            // inputs [feature (padded to 16)][sample]
    __nv_bfloat16 h1T[64 * T_LD], h2T[64 * T_LD];
    __nv_bfloat16 dz1T[64 * T_LD], dz2T[64 * T_LD], dz3T[64 * T_LD];
    __nv_bfloat16 sg[3][4][32][64];         // silu'(z_l) per warp, in fragment order of each lane
    float h3[TB][65];                       // last hidden layer (fp32) for dW4
    float dy[TB];
    float loss[4];
};

// store a C-fragment value for (row, col) of this warp's 32-row slab,
// transposed into a [col][sample] tile
__device__ __forceinline__ void storeT(__nv_bfloat16 *tile, int warp, int row, int col, float v) {
    tile[col * T_LD + warp * 32 + row] = __float2bfloat16(v);
}

template <class F>
__device__ __forceinline__ void for_frag(F f) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int row = m * 16 + g + (e >= 2 ? 8 : 0);
                const int col = nt * 8 + 2 * t + (e & 1);
                f(m, nt, e, row, col);
            }
}

// dW_partial[out][in] = sum over the block's samples of dzT[out][s] * hT[in][s]
// for an (64 x NIN) weight, NIN = 64 or 16 (padded input)
template <int NIN>
__device__ __forceinline__ void block_dw(const __nv_bfloat16 *dzT, const __nv_bfloat16 *hT, float *out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    constexpr int NT = NIN / 8;
    // 4 row tiles (m16) x NT column tiles, split over the 4 warps by row tile
    const int mt = warp;
    for (int nt = 0; nt < NT; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        for (int kt = 0; kt < TB / 16; ++kt) {
            uint32_t a[4];
            const __nv_bfloat16 *ar = dzT + (mt * 16 + g) * T_LD + kt * 16 + 2 * t;
            a[0] = lds32(ar);
            a[1] = lds32(ar + 8 * T_LD);
            a[2] = lds32(ar + 8);
            a[3] = lds32(ar + 8 * T_LD + 8);
            const __nv_bfloat16 *br = hT + (nt * 8 + g) * T_LD + kt * 16 + 2 * t;
            mma16816(d, a, lds32(br), lds32(br + 8));
        }
        const int r0 = mt * 16 + g, c0 = nt * 8 + 2 * t;
        out[r0 * NIN + c0] = d[0];
        out[r0 * NIN + c0 + 1] = d[1];
        out[(r0 + 8) * NIN + c0] = d[2];
        out[(r0 + 8) * NIN + c0 + 1] = d[3];
    }
}

// per-block partial layout: [dW1 64x16 (padded)] [db1 64] [dW2 64x64] [db2 64]
// [dW3 64x64] [db3 64] [dW4 64] [db4 1] [loss 1]
constexpr int PART = 64 * 16 + 64 + 4096 + 64 + 4096 + 64 + 64 + 1 + 1;

__global__ void __launch_bounds__(TB) k_pstar_train(const float4 *__restrict__ x, const float *__restrict__ target,
                                                    const int *__restrict__ index, int nbatch, float inv_batch,
                                                    const PackedMlp *__restrict__ pk, float *__restrict__ partials) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem &S = *reinterpret_cast<TrainSmem *>(smem_raw);
    load_packed(&S.w, pk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row_g = blockIdx.x * TB + warp * 32 + lane;   // sample of this lane
    const bool valid = row_g < nbatch;
    const int src = valid ? (index ? index[row_g] : row_g) : 0;
    const float4 xi = valid ? x[src] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float ti = valid ? target[src] : 0.f;
    // ---- forward
    uint32_t a0[2][1][4];
    input_frags<2>(xi, a0);
    {
        const float xv[4] = {xi.x, xi.y, xi.z, xi.w};
        for (int k = 0; k < 16; ++k) S.xT[k * T_LD + warp * 32 + lane] = __float2bfloat16(k < 4 ? xv[k] : 0.f);
    }
    Acc64 acc;
    uint32_t a[2][4][4];
    layer_mma<2, 1>(acc, a0, S.w.w1, W1_LD, S.w.b1);
    for_frag([&](int m, int nt, int e, int row, int col) {
        const float z = acc.v[m][nt][e];
        S.sg[0][warp][lane][(m * 8 + nt) * 4 + e] = __float2bfloat16(silu_grad(z));
        storeT(S.h1T, warp, row, col, silu(z));
    });
    acc_to_a(acc, a, silu);
    layer_mma<2, 4>(acc, a, S.w.w2, W_LD, S.w.b2);
    for_frag([&](int m, int nt, int e, int row, int col) {
        const float z = acc.v[m][nt][e];
        S.sg[1][warp][lane][(m * 8 + nt) * 4 + e] = __float2bfloat16(silu_grad(z));
        storeT(S.h2T, warp, row, col, silu(z));
    });
    acc_to_a(acc, a, silu);
    layer_mma<2, 4>(acc, a, S.w.w3, W_LD, S.w.b3);
    for_frag([&](int m, int nt, int e, int row, int col) {
        const float z = acc.v[m][nt][e];
        S.sg[2][warp][lane][(m * 8 + nt) * 4 + e] = __float2bfloat16(silu_grad(z));
        S.h3[warp * 32 + row][col] = silu(z);
    });
    const float yv = output_row(acc, S.w.w4, S.w.b4);
    // ---- loss = mean (y - t)^2 over the batch
    const float err = valid ? yv - ti : 0.f;
    S.dy[warp * 32 + lane] = 2.f * err * inv_batch;
    float l = err * err * inv_batch;
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (lane == 0) S.loss[warp] = l;
    __syncwarp();
    // ---- backward: dz3 = (dy W4) * silu'(z3)
    for_frag([&](int m, int nt, int e, int row, int col) {
        const float dh = S.dy[warp * 32 + row] * S.w.w4[col];
        acc.v[m][nt][e] = dh * __bfloat162float(S.sg[2][warp][lane][(m * 8 + nt) * 4 + e]);
        storeT(S.dz3T, warp, row, col, acc.v[m][nt][e]);
    });
    // dh2 = dz3 W3 (B operand = W3^T rows), dz2 = dh2 * silu'(z2)
    {
        const float zero[64] = {0};
        acc_to_a(acc, a, [](float v) { return v; });
        layer_mma<2, 4>(acc, a, S.w.w3t, W_LD, zero);
    }
    for_frag([&](int m, int nt, int e, int row, int col) {
        acc.v[m][nt][e] *= __bfloat162float(S.sg[1][warp][lane][(m * 8 + nt) * 4 + e]);
        storeT(S.dz2T, warp, row, col, acc.v[m][nt][e]);
    });
    {
        const float zero[64] = {0};
        acc_to_a(acc, a, [](float v) { return v; });
        layer_mma<2, 4>(acc, a, S.w.w2t, W_LD, zero);
    }
    for_frag([&](int m, int nt, int e, int row, int col) {
        acc.v[m][nt][e] *= __bfloat162float(S.sg[0][warp][lane][(m * 8 + nt) * 4 + e]);
        storeT(S.dz1T, warp, row, col, acc.v[m][nt][e]);
    });
    __syncthreads();
    // ---- this block's weight gradients
    float *P = partials + (size_t)blockIdx.x * PART;
    float *dW1 = P, *db1 = dW1 + 64 * 16, *dW2 = db1 + 64, *db2 = dW2 + 4096, *dW3 = db2 + 64, *db3 = dW3 + 4096,
          *dW4 = db3 + 64, *db4 = dW4 + 64, *lossp = db4 + 1;
    block_dw<16>(S.dz1T, S.xT, dW1);
    block_dw<64>(S.dz2T, S.h1T, dW2);
    block_dw<64>(S.dz3T, S.h2T, dW3);
    // bias gradients and the last layer on the CUDA cores (fixed order)
    for (int c = threadIdx.x; c < 64; c += blockDim.x) {
        float s1 = 0.f, s2 = 0.f, s3 = 0.f, s4 = 0.f;
        for (int sidx = 0; sidx < TB; ++sidx) {
            s1 += __bfloat162float(S.dz1T[c * T_LD + sidx]);
            s2 += __bfloat162float(S.dz2T[c * T_LD + sidx]);
            s3 += __bfloat162float(S.dz3T[c * T_LD + sidx]);
            s4 += S.dy[sidx] * S.h3[sidx][c];
        }
        db1[c] = s1; db2[c] = s2; db3[c] = s3; dW4[c] = s4;
    }
    if (threadIdx.x == 0) {
        float s = 0.f, ls = 0.f;
        for (int sidx = 0; sidx < TB; ++sidx) s += S.dy[sidx];
        for (int w = 0; w < 4; ++w) ls += S.loss[w];
        *db4 = s;
        *lossp = ls;
    }
}

// Sum of the per-block partials in block order -> gradient in the parameter
// layout (dW1 unpadded) and the loss.
__global__ void k_pstar_reduce(const float *__restrict__ partials, int nblocks, float *__restrict__ grad,
                               float *__restrict__ loss) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < PART; k += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblocks; ++b) s += partials[(size_t)b * PART + k];
        // map the partial layout to the parameter layout
        if (k < 64 * 16) {
            const int r = k / 16, c = k % 16;
            if (c < 4) grad[r * 4 + c] = s;
        } else {
            const int q = k - 64 * 16;     // db1 ... db4 follow W1 in both layouts
            if (q < NPRM - 256) grad[256 + q] = s;
            else if (q == NPRM - 256) *loss = s;
        }
    }
}

__global__ void k_adam(float *__restrict__ prm, const float *__restrict__ grad, float *__restrict__ m1,
                       float *__restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const float gk = grad[k];
        const float a = b1 * m1[k] + (1.f - b1) * gk;
        const float b = b2 * m2[k] + (1.f - b2) * gk * gk;
        m1[k] = a;
        m2[k] = b;
        prm[k] -= lr * (a * c1) / (sqrtf(b * c2) + eps);
    }
}

size_t pstar_train_smem() { return sizeof(TrainSmem); }
size_t pstar_infer_smem() { return sizeof(PackedMlp); }

void pstar_pack(const float *prm, void *packed, cudaStream_t s) {
    k_pack_mlp<<<32, 256, 0, s>>>(prm, (PackedMlp *)packed);
}

void pstar_infer(const float4 *x, int n, const void *packed, float *y, int sm_count, cudaStream_t s) {
    const int warps = (n + 31) / 32;
    int blocks = (warps + 7) / 8;
    if (blocks > sm_count * 8) blocks = sm_count * 8;
    if (blocks < 1) blocks = 1;
    k_pstar_infer<<<blocks, 256, sizeof(PackedMlp), s>>>(x, n, nullptr, (const PackedMlp *)packed, y);
}

void pstar_infer_dev(const float4 *x, const int *n_dev, int cap, const void *packed, float *y, int sm_count,
                     cudaStream_t s) {
    k_pstar_infer<<<sm_count * 4, 256, sizeof(PackedMlp), s>>>(x, cap, n_dev, (const PackedMlp *)packed, y);
}

size_t pstar_packed_bytes() { return sizeof(PackedMlp); }
int pstar_partial_floats() { return PART; }

void pstar_train_batch(const float4 *x, const float *target, const int *index, int nbatch, const void *packed,
                       float *partials, float *grad, float *loss, cudaStream_t s) {
    const int blocks = (nbatch + TB - 1) / TB;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_pstar_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
        attr = true;
    }
    k_pstar_train<<<blocks, TB, sizeof(TrainSmem), s>>>(x, target, index, nbatch, 1.f / (float)nbatch,
                                                        (const PackedMlp *)packed, partials);
    k_pstar_reduce<<<(PART + 255) / 256, 256, 0, s>>>(partials, blocks, grad, loss);
}

void pstar_adam(float *prm, const float *grad, float *m1, float *m2, float lr, int step, cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
    k_adam<<<(NPRM + 255) / 256, 256, 0, s>>>(prm, grad, m1, m2, NPRM, lr, b1, b2, 1e-8f, c1, c2);
}

}  // namespace mlh

// ------------------------------------------------------------------ C ABI

namespace {

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 16); }
    template <class T> T *as() const { return (T *)p; }
};

int fail(cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    mlh::set_last_error(m.c_str());
    return MLH_ERR_CUDA;
}

#define PCK(call)                                 \
    do {                                          \
        cudaError_t e_ = (call);                  \
        if (e_ != cudaSuccess) return fail(e_, #call); \
    } while (0)

int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

}  // namespace

using namespace mlh;

extern "C" int mlh_pstar_infer(const float *weights, const float *x, int n, float *y) {
    if (!weights || !x || !y || n < 1) return MLH_ERR_INVALID;
    DevBuf w, pk, dx, dy;
    PCK(w.alloc(sizeof(float) * PSTAR_PARAMS));
    PCK(pk.alloc(pstar_packed_bytes()));
    PCK(dx.alloc(sizeof(float) * 4 * (size_t)n));
    PCK(dy.alloc(sizeof(float) * (size_t)n));
    PCK(cudaMemcpy(w.p, weights, sizeof(float) * PSTAR_PARAMS, cudaMemcpyHostToDevice));
    PCK(cudaMemcpy(dx.p, x, sizeof(float) * 4 * (size_t)n, cudaMemcpyHostToDevice));
    pstar_pack(w.as<float>(), pk.p, 0);
    pstar_infer(dx.as<float4>(), n, pk.p, dy.as<float>(), sm_count(), 0);
    PCK(cudaGetLastError());
    PCK(cudaMemcpy(y, dy.p, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int mlh_pstar_grad(const float *weights, const float *x, const float *t, int n, float *loss, float *grad) {
    if (!weights || !x || !t || !loss || !grad || n < 1) return MLH_ERR_INVALID;
    const int blocks = (n + 127) / 128;
    DevBuf w, pk, dx, dt, part, g, l;
    PCK(w.alloc(sizeof(float) * PSTAR_PARAMS));
    PCK(pk.alloc(pstar_packed_bytes()));
    PCK(dx.alloc(sizeof(float) * 4 * (size_t)n));
    PCK(dt.alloc(sizeof(float) * (size_t)n));
    PCK(part.alloc(sizeof(float) * (size_t)pstar_partial_floats() * blocks));
    PCK(g.alloc(sizeof(float) * PSTAR_PARAMS));
    PCK(l.alloc(sizeof(float)));
    PCK(cudaMemcpy(w.p, weights, sizeof(float) * PSTAR_PARAMS, cudaMemcpyHostToDevice));
    PCK(cudaMemcpy(dx.p, x, sizeof(float) * 4 * (size_t)n, cudaMemcpyHostToDevice));
    PCK(cudaMemcpy(dt.p, t, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice));
    pstar_pack(w.as<float>(), pk.p, 0);
    pstar_train_batch(dx.as<float4>(), dt.as<float>(), nullptr, n, pk.p, part.as<float>(), g.as<float>(),
                      l.as<float>(), 0);
    PCK(cudaGetLastError());
    PCK(cudaMemcpy(grad, g.p, sizeof(float) * PSTAR_PARAMS, cudaMemcpyDeviceToHost));
    PCK(cudaMemcpy(loss, l.p, sizeof(float), cudaMemcpyDeviceToHost));
    return 0;
}

// Adam on the GPU over `epochs` passes of shuffled mini-batches of `batch`
// samples, the learning rate decayed from lr to lr / 100 along a half cosine
// over the run (Adam moves every parameter by about the learning rate per
// step whatever its gradient, so at a constant rate the final weights, and
// with them the output's offset, land anywhere in a band of a few lr);
// weights are read from and written back to `weights` (host);
// loss_history[e] receives the mean mini-batch loss of epoch e.
extern "C" int mlh_pstar_train(const float *x, const float *t, long long n, int epochs, int batch, float lr,
                               unsigned seed, float *weights, float *loss_history) {
    if (!x || !t || !weights || n < 1 || epochs < 1 || batch < 128 || n > (1ll << 31) - 1) return MLH_ERR_INVALID;
    if (batch > n) batch = (int)n;
    const int blocks = (batch + 127) / 128;
    DevBuf w, pk, dx, dt, part, g, l, m1, m2, idx;
    PCK(w.alloc(sizeof(float) * PSTAR_PARAMS));
    PCK(pk.alloc(pstar_packed_bytes()));
    PCK(dx.alloc(sizeof(float) * 4 * (size_t)n));
    PCK(dt.alloc(sizeof(float) * (size_t)n));
    PCK(part.alloc(sizeof(float) * (size_t)pstar_partial_floats() * blocks));
    PCK(g.alloc(sizeof(float) * PSTAR_PARAMS));
    PCK(l.alloc(sizeof(float) * (size_t)epochs * (size_t)(n / batch + 1)));
    PCK(m1.alloc(sizeof(float) * PSTAR_PARAMS));
    PCK(m2.alloc(sizeof(float) * PSTAR_PARAMS));
    PCK(idx.alloc(sizeof(int) * (size_t)n));
    PCK(cudaMemcpy(w.p, weights, sizeof(float) * PSTAR_PARAMS, cudaMemcpyHostToDevice));
    PCK(cudaMemcpy(dx.p, x, sizeof(float) * 4 * (size_t)n, cudaMemcpyHostToDevice));
    PCK(cudaMemcpy(dt.p, t, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice));
    PCK(cudaMemset(m1.p, 0, sizeof(float) * PSTAR_PARAMS));
    PCK(cudaMemset(m2.p, 0, sizeof(float) * PSTAR_PARAMS));
    std::vector<int> perm((size_t)n);
    for (long long i = 0; i < n; ++i) perm[i] = (int)i;
    std::mt19937_64 rng(seed);
    const long long per_epoch = n / batch;
    const double total = (double)epochs * (double)per_epoch;
    int step = 0;
    for (int e = 0; e < epochs; ++e) {
        std::shuffle(perm.begin(), perm.end(), rng);
        PCK(cudaMemcpy(idx.p, perm.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
        for (long long b = 0; b < per_epoch; ++b) {
            pstar_pack(w.as<float>(), pk.p, 0);
            pstar_train_batch(dx.as<float4>(), dt.as<float>(), idx.as<int>() + b * batch, batch, pk.p,
                              part.as<float>(), g.as<float>(), l.as<float>() + (size_t)e * per_epoch + b, 0);
            const double frac = total > 1. ? (double)step / (total - 1.) : 1.;
            const float lr_t = (float)(lr * (0.01 + 0.99 * 0.5 * (1. + cos(3.14159265358979323846 * frac))));
            pstar_adam(w.as<float>(), g.as<float>(), m1.as<float>(), m2.as<float>(), lr_t, ++step, 0);
        }
    }
    PCK(cudaGetLastError());
    PCK(cudaMemcpy(weights, w.p, sizeof(float) * PSTAR_PARAMS, cudaMemcpyDeviceToHost));
    if (loss_history) {
        std::vector<float> lh((size_t)epochs * per_epoch);
        PCK(cudaMemcpy(lh.data(), l.p, sizeof(float) * lh.size(), cudaMemcpyDeviceToHost));
        for (int e = 0; e < epochs; ++e) {
            double s = 0.;
            for (long long b = 0; b < per_epoch; ++b) s += lh[(size_t)e * per_epoch + b];
            loss_history[e] = (float)(s / (double)per_epoch);
        }
    }
    return 0;
}
