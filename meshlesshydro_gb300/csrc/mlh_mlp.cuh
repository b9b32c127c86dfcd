// Tensor-core pieces of the learned star-pressure network (4-64-64-64-1 SiLU
// MLP), shared by its training/inference kernels (mlh_pstar.cu) and by the
// face kernel, which evaluates it in-block for its strong-shock faces
// (mlh_kernels.cu).  BF16 operands, FP32 accumulation, mma.sync m16n8k16.
// A warp evaluates MT M-tiles of 16 rows each (MT = 2: 32 rows, one per lane;
// MT = 1: 16 rows on lanes 0..15).
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace mlh {

// global/shared layout of the BF16 operand matrices (rows padded so that the
// fragment loads of a warp hit 32 different banks)
constexpr int W1_LD = 24;   // W1 padded to K = 16, row stride 24
constexpr int W_LD = 72;    // 64-wide rows, stride 72

struct PackedMlp {
    __nv_bfloat16 w1[64 * W1_LD];
    __nv_bfloat16 w2[64 * W_LD], w3[64 * W_LD];     // [out][in]
    __nv_bfloat16 w2t[64 * W_LD], w3t[64 * W_LD];   // [in][out]
    float b1[64], b2[64], b3[64], w4[64], b4;
    float pad[3];                                   // size a multiple of 16 bytes
};
static_assert(sizeof(PackedMlp) % 16 == 0, "PackedMlp is copied in 16-byte words");

__device__ __forceinline__ void mma16816(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

// C fragments of a 64-wide layer output for MT M-tiles of 16 rows
template <int MT>
struct AccT {
    float v[MT][8][4];
};
using Acc64 = AccT<2>;

// acc = bias + A(16 MT x K) * W^T, W rows [out][in] with stride ld, A
// fragments given per M-tile and K-tile.
template <int MT, int KT>
__device__ __forceinline__ void layer_mma(AccT<MT> &acc, const uint32_t (*afr)[KT][4], const __nv_bfloat16 *w,
                                          int ld, const float *bias) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bb0 = bias[nt * 8 + 2 * t], bb1 = bias[nt * 8 + 2 * t + 1];
#pragma unroll
        for (int m = 0; m < MT; ++m) {
            acc.v[m][nt][0] = bb0; acc.v[m][nt][1] = bb1; acc.v[m][nt][2] = bb0; acc.v[m][nt][3] = bb1;
        }
#pragma unroll
        for (int kt = 0; kt < KT; ++kt) {
            const __nv_bfloat16 *wr = w + (nt * 8 + g) * ld + kt * 16 + 2 * t;
            const uint32_t b0 = lds32(wr), b1 = lds32(wr + 8);
#pragma unroll
            for (int m = 0; m < MT; ++m) mma16816(acc.v[m][nt], afr[m][kt], b0, b1);
        }
    }
}

// C fragments of a 64-wide layer (after f) -> A fragments of the next layer
template <int MT, class F>
__device__ __forceinline__ void acc_to_a(const AccT<MT> &acc, uint32_t (*afr)[4][4], F f) {
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const float *c0 = acc.v[m][2 * kt], *c1 = acc.v[m][2 * kt + 1];
            afr[m][kt][0] = pack2(f(c0[0]), f(c0[1]));
            afr[m][kt][1] = pack2(f(c0[2]), f(c0[3]));
            afr[m][kt][2] = pack2(f(c1[0]), f(c1[1]));
            afr[m][kt][3] = pack2(f(c1[2]), f(c1[3]));
        }
}

// A fragments of the (16 MT) x 16 input slab (4 features, zero padded) from
// the features held by each lane for its own row (row r on lane r)
template <int MT>
__device__ __forceinline__ void input_frags(const float4 x, uint32_t (*a0)[1][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int m = 0; m < MT; ++m) {
        // the shuffled value is evaluated on the source lane: move all four
        // features of rows g and g+8, then pick columns 2t, 2t+1 here
        const int r0 = m * 16 + g, r1 = r0 + 8;
        const float p0 = __shfl_sync(0xffffffffu, x.x, r0), p1 = __shfl_sync(0xffffffffu, x.y, r0);
        const float p2 = __shfl_sync(0xffffffffu, x.z, r0), p3 = __shfl_sync(0xffffffffu, x.w, r0);
        const float q0 = __shfl_sync(0xffffffffu, x.x, r1), q1 = __shfl_sync(0xffffffffu, x.y, r1);
        const float q2 = __shfl_sync(0xffffffffu, x.z, r1), q3 = __shfl_sync(0xffffffffu, x.w, r1);
        a0[m][0][0] = t == 0 ? pack2(p0, p1) : (t == 1 ? pack2(p2, p3) : 0u);
        a0[m][0][1] = t == 0 ? pack2(q0, q1) : (t == 1 ? pack2(q2, q3) : 0u);
        a0[m][0][2] = 0u;
        a0[m][0][3] = 0u;
    }
}

// y of the row of this lane (MT = 2: row = lane; MT = 1: row = lane % 16),
// from the C fragments of the last hidden layer
template <int MT>
__device__ __forceinline__ float output_row(const AccT<MT> &acc3, const float *w4, float b4) {
    const int lane = threadIdx.x & 31, t = lane & 3;
    float part[MT][2];   // [m][row g / g+8]
#pragma unroll
    for (int m = 0; m < MT; ++m) { part[m][0] = 0.f; part[m][1] = 0.f; }
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float wa = w4[nt * 8 + 2 * t], wb = w4[nt * 8 + 2 * t + 1];
            part[m][0] += silu(acc3.v[m][nt][0]) * wa + silu(acc3.v[m][nt][1]) * wb;
            part[m][1] += silu(acc3.v[m][nt][2]) * wa + silu(acc3.v[m][nt][3]) * wb;
        }
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            part[m][h] += __shfl_xor_sync(0xffffffffu, part[m][h], 1);
            part[m][h] += __shfl_xor_sync(0xffffffffu, part[m][h], 2);
        }
    // row r of M-tile m is held by lane 4 * (r % 8), in half r / 8
    const int m = MT == 2 ? lane >> 4 : 0, r = lane & 15;
    const int src = 4 * (r & 7);
    const float v0 = __shfl_sync(0xffffffffu, part[0][0], src), v1 = __shfl_sync(0xffffffffu, part[0][1], src);
    float v = r < 8 ? v0 : v1;
    if (MT == 2) {
        const float v2 = __shfl_sync(0xffffffffu, part[MT - 1][0], src);
        const float v3 = __shfl_sync(0xffffffffu, part[MT - 1][1], src);
        if (m == 1) v = r < 8 ? v2 : v3;
    }
    return v + b4;
}

// y = MLP(x) for the rows of this warp (row r's input on lane r), weights w
// in shared or global memory
template <int MT>
__device__ __forceinline__ float mlp_rows(const PackedMlp *w, const float4 xi) {
    uint32_t a0[MT][1][4];
    input_frags<MT>(xi, a0);
    AccT<MT> acc;
    uint32_t a[MT][4][4];
    layer_mma<MT, 1>(acc, a0, w->w1, W1_LD, w->b1);
    acc_to_a<MT>(acc, a, silu);
    layer_mma<MT, 4>(acc, a, w->w2, W_LD, w->b2);
    acc_to_a<MT>(acc, a, silu);
    layer_mma<MT, 4>(acc, a, w->w3, W_LD, w->b3);
    return output_row<MT>(acc, w->w4, w->b4);
}

}  // namespace mlh
