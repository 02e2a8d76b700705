// selector_launch.h -- host-side launchers of the learned stencil selector
// (selector_train.cu, selector_mma.cu).  All return cudaGetLastError() of
// the launch.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "device.h"

namespace mgpu {
namespace sel {

// BF16 weight image in the tensor cores' shared-memory layout plus FP32 biases
constexpr int WEIGHT_IMAGE_BYTES = 25216;

// feature rows X [n][96] and class labels Y [n][4] of the listed cells;
// nb4 selects the FP32 form's neighbour layout; masks may be null (no labels)
cudaError_t launch_harvest(const TenoArgs& a, bool nb4, const double* U, const uint32_t* cells, uint32_t n,
                           const uint8_t* masks, float* X, uint8_t* Y, cudaStream_t s);
// C (+)= op(A) op(B), row-major.  splits > 1 splits K and needs work of
// splits * M * N floats and a contiguous C (ldc == N).
cudaError_t launch_sgemm(bool ta, bool tb, int M, int N, int K, const float* A, int lda, const float* B, int ldb,
                         float* C, int ldc, bool accumulate, int splits, float* work, cudaStream_t s);
cudaError_t launch_bias_act(int rows, int cols, float* Z, const float* b, float* A, bool act, cudaStream_t s);
cudaError_t launch_gelu_back(int n, const float* dA, const float* Z, float* dZ, cudaStream_t s);
cudaError_t launch_xent(int rows, const float* Z, const uint8_t* Y, float scale, float* dZ, float* part,
                        cudaStream_t s);
int xent_blocks(int rows);
cudaError_t launch_colsum(int rows, int cols, const float* dZ, float* db, cudaStream_t s);
cudaError_t launch_adam(int n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                        float bc1, float bc2, cudaStream_t s);
cudaError_t launch_gather_rows(int rows, const uint32_t* idx, const float* X, const uint8_t* Y, float* Xb,
                               uint8_t* Yb, cudaStream_t s);

// tcgen05 inference.  thr_central / thr_directional: minimum probability
// for a confident prediction of the central class / a directional class
// (outside (0, 1]: never confident).  err: device flag, bit 0 set when a
// bounded wait ran out.
int mlp_smem_bytes();
// raises the kernels' dynamic shared memory limit; call once per device
// before the first launch (outside any stream capture)
cudaError_t mlp_prepare();
cudaError_t launch_mlp_rows(const uint8_t* wimg, int n, const float* X, float* logits, uint8_t* pred,
                            float thr_central, float thr_directional, unsigned* err, cudaStream_t s);
// trusted = pred with the confident bit kept only where every face
// neighbour's same variable is confident too (both [n][4] bytes)
cudaError_t launch_trust(int n, const int4* cfaces, const int2* lr, const uint8_t* pred, uint8_t* trusted,
                         cudaStream_t s);
cudaError_t launch_mlp_cells(const uint8_t* wimg, const TenoArgs& a, const float* U, float thr_central,
                             float thr_directional, uint8_t* pred, unsigned* err, cudaStream_t s);

}  // namespace sel
}  // namespace mgpu
