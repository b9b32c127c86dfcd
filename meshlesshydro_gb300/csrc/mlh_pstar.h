// Host-side entry points of the learned p* guess (mlh_pstar.cu).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace mlh {

constexpr int PSTAR_PARAMS = 8705;

size_t pstar_packed_bytes();
size_t pstar_train_smem();
int pstar_partial_floats();
void pstar_pack(const float *prm, void *packed, cudaStream_t s);
void pstar_infer(const float4 *x, int n, const void *packed, float *y, int sm_count, cudaStream_t s);
void pstar_train_batch(const float4 *x, const float *target, const int *index, int nbatch, const void *packed,
                       float *partials, float *grad, float *loss, cudaStream_t s);
void pstar_adam(float *prm, const float *grad, float *m1, float *m2, float lr, int step, cudaStream_t s);

}  // namespace mlh
