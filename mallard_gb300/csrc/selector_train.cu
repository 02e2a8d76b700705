// selector_train.cu -- harvest and training kernels of the learned stencil
// selector (FP32, CUDA cores).
//
// Training is plain minibatch back-propagation through the 96-64-64-32 MLP
// with a softmax cross-entropy per variable head and Adam.  Every reduction
// has a fixed order (split-K partial sums reduced in chunk order, column
// sums in row order), so a training run is deterministic for a given seed.
#include <cstdint>

#include "fp_convert.cuh"
#include "selector.cuh"
#include "selector_launch.h"

namespace mgpu {
namespace sel {
namespace {

// FP64 -> FP32, round to nearest, on the integer pipe
struct ToFloatRN {
    __device__ float operator()(double x) const { return f32_rn(x); }
};

// One thread per (selected cell, variable): feature row and class label.
template <bool NB4>
__global__ void __launch_bounds__(128) harvest_kernel(const TenoArgs a, const double* __restrict__ U,
                                                      const uint32_t* __restrict__ cells, uint32_t n,
                                                      const uint8_t* __restrict__ masks, float* __restrict__ X,
                                                      uint8_t* __restrict__ Y) {
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gt >> 2;
    const int v = gt & 3;
    if (i >= n) return;
    const int cell = (int)cells[i];
    float x[PER_VAR];
    features<NB4>(a, U, cell, v, a.smask[cell], ToFloatRN{}, x);
    float* row = X + (size_t)i * IN + v * PER_VAR;
#pragma unroll
    for (int k = 0; k < PER_VAR; ++k) row[k] = x[k];
    if (masks) Y[(size_t)i * NV + v] = (uint8_t)class_of_mask(masks[(size_t)cell * NV + v]);
}

// C (+)= op(A) op(B), row-major; op(A) is M x K, op(B) is K x N.
// blockIdx.z selects a K chunk of length kchunk; with more than one chunk
// each chunk writes its own partial product at C + z * M * N.
constexpr int BM = 64, BN = 64, BK = 16;
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) sgemm_kernel(int M, int N, int K, const float* __restrict__ A, int lda,
                                                    const float* __restrict__ B, int ldb, float* __restrict__ C,
                                                    int ldc, int kchunk, int accumulate) {
    __shared__ float As[BK][BM + 4];
    __shared__ float Bs[BK][BN + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int k_begin = blockIdx.z * kchunk, k_end = min(K, k_begin + kchunk);
    float acc[4][4] = {};
    for (int k0 = k_begin; k0 < k_end; k0 += BK) {
        for (int e = threadIdx.x; e < BK * BM; e += 256) {
            const int kk = e / BM, mm = e % BM;
            const int gm = m0 + mm, gk = k0 + kk;
            float val = 0.0f;
            if (gm < M && gk < k_end) val = TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
            As[kk][mm] = val;
        }
        for (int e = threadIdx.x; e < BK * BN; e += 256) {
            const int kk = e / BN, nn = e % BN;
            const int gn = n0 + nn, gk = k0 + kk;
            float val = 0.0f;
            if (gn < N && gk < k_end) val = TB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
            Bs[kk][nn] = val;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    float* Cz = C + (size_t)blockIdx.z * M * N;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gm = m0 + ty * 4 + i;
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gn = n0 + tx * 4 + j;
            if (gn >= N) continue;
            float* c = (gridDim.z > 1 ? Cz + (size_t)gm * N + gn : C + (size_t)gm * ldc + gn);
            *c = (accumulate && gridDim.z == 1) ? *c + acc[i][j] : acc[i][j];
        }
    }
}

// C[i] = sum_z P[z][i], chunks in order
__global__ void splitk_reduce_kernel(int n, int splits, const float* __restrict__ P, float* __restrict__ C) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.0f;
    for (int z = 0; z < splits; ++z) s += P[(size_t)z * n + i];
    C[i] = s;
}

// Z += b; A = gelu(Z) (or A = Z without the activation)
__global__ void bias_act_kernel(int rows, int cols, float* __restrict__ Z, const float* __restrict__ b,
                                float* __restrict__ A, int act) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const float z = Z[i] + b[i % cols];
    Z[i] = z;
    if (A) A[i] = act ? gelu(z) : z;
}

// dZ = dA * gelu'(Z)
__global__ void gelu_back_kernel(int n, const float* __restrict__ dA, const float* __restrict__ Z,
                                 float* __restrict__ dZ) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dZ[i] = dA[i] * gelu_grad(Z[i]);
}

// Softmax cross-entropy over the 4 heads of 8 classes.  dZ = (p - onehot) *
// scale; per-block loss sums go to part[blockIdx.x] (fixed order).
__global__ void __launch_bounds__(128) xent_kernel(int rows, const float* __restrict__ Z,
                                                   const uint8_t* __restrict__ Y, float scale,
                                                   float* __restrict__ dZ, float* __restrict__ part) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = gt >> 2, h = gt & 3;
    float loss = 0.0f;
    if (r < rows) {
        const float* z = Z + (size_t)r * OUT + h * NCLS;
        float mx = z[0];
#pragma unroll
        for (int c = 1; c < NCLS; ++c) mx = fmaxf(mx, z[c]);
        float e[NCLS], s = 0.0f;
#pragma unroll
        for (int c = 0; c < NCLS; ++c) {
            e[c] = expf(z[c] - mx);
            s += e[c];
        }
        const int y = Y[(size_t)r * NV + h];
        const float inv = 1.0f / s;
        loss = logf(s) - (z[y] - mx);
        float* d = dZ + (size_t)r * OUT + h * NCLS;
#pragma unroll
        for (int c = 0; c < NCLS; ++c) d[c] = (e[c] * inv - (c == y ? 1.0f : 0.0f)) * scale;
    }
    __shared__ float red[128];
    red[threadIdx.x] = loss;
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// db[j] = sum over rows of dZ[r][j], rows in order
__global__ void colsum_kernel(int rows, int cols, const float* __restrict__ dZ, float* __restrict__ db) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    float s = 0.0f;
    for (int r = 0; r < rows; ++r) s += dZ[(size_t)r * cols + j];
    db[j] = s;
}

__global__ void adam_kernel(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

__global__ void gather_rows_kernel(int rows, const uint32_t* __restrict__ idx, const float* __restrict__ X,
                                   const uint8_t* __restrict__ Y, float* __restrict__ Xb, uint8_t* __restrict__ Yb) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = gt / IN, k = gt % IN;
    if (r >= rows) return;
    const size_t src = idx[r];
    Xb[(size_t)r * IN + k] = X[src * IN + k];
    if (k < NV) Yb[(size_t)r * NV + k] = Y[src * NV + k];
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

cudaError_t launch_harvest(const TenoArgs& a, bool nb4, const double* U, const uint32_t* cells, uint32_t n,
                           const uint8_t* masks, float* X, uint8_t* Y, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const unsigned b = nblk((long long)n * 4, 128);
    if (nb4) harvest_kernel<true><<<b, 128, 0, s>>>(a, U, cells, n, masks, X, Y);
    else harvest_kernel<false><<<b, 128, 0, s>>>(a, U, cells, n, masks, X, Y);
    return cudaGetLastError();
}

cudaError_t launch_sgemm(bool ta, bool tb, int M, int N, int K, const float* A, int lda, const float* B, int ldb,
                         float* C, int ldc, bool accumulate, int splits, float* work, cudaStream_t s) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    if (splits < 1) splits = 1;
    const int kchunk = ((K + splits - 1) / splits + BK - 1) / BK * BK;
    splits = kchunk > 0 ? (K + kchunk - 1) / kchunk : 1;
    if (splits < 1) splits = 1;
    dim3 grid(nblk(N, BN), nblk(M, BM), splits);
    float* out = splits > 1 ? work : C;
    const int acc = accumulate ? 1 : 0;
    if (!ta && !tb) sgemm_kernel<false, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, out, ldc, kchunk, acc);
    else if (ta && !tb) sgemm_kernel<true, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, out, ldc, kchunk, acc);
    else if (!ta && tb) sgemm_kernel<false, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, out, ldc, kchunk, acc);
    else sgemm_kernel<true, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, out, ldc, kchunk, acc);
    if (splits > 1) {
        // partial products are M x N contiguous; C must be contiguous too (ldc == N)
        splitk_reduce_kernel<<<nblk((long long)M * N, 256), 256, 0, s>>>(M * N, splits, work, C);
    }
    return cudaGetLastError();
}

cudaError_t launch_bias_act(int rows, int cols, float* Z, const float* b, float* A, bool act, cudaStream_t s) {
    if (rows * cols == 0) return cudaSuccess;
    bias_act_kernel<<<nblk((long long)rows * cols, 256), 256, 0, s>>>(rows, cols, Z, b, A, act ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_gelu_back(int n, const float* dA, const float* Z, float* dZ, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    gelu_back_kernel<<<nblk(n, 256), 256, 0, s>>>(n, dA, Z, dZ);
    return cudaGetLastError();
}

cudaError_t launch_xent(int rows, const float* Z, const uint8_t* Y, float scale, float* dZ, float* part,
                        cudaStream_t s) {
    if (rows == 0) return cudaSuccess;
    xent_kernel<<<nblk((long long)rows * 4, 128), 128, 0, s>>>(rows, Z, Y, scale, dZ, part);
    return cudaGetLastError();
}

int xent_blocks(int rows) { return (int)nblk((long long)rows * 4, 128); }

cudaError_t launch_colsum(int rows, int cols, const float* dZ, float* db, cudaStream_t s) {
    colsum_kernel<<<nblk(cols, 64), 64, 0, s>>>(rows, cols, dZ, db);
    return cudaGetLastError();
}

cudaError_t launch_adam(int n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                        float bc1, float bc2, cudaStream_t s) {
    adam_kernel<<<nblk(n, 256), 256, 0, s>>>(n, p, g, m, v, lr, b1, b2, eps, bc1, bc2);
    return cudaGetLastError();
}

cudaError_t launch_gather_rows(int rows, const uint32_t* idx, const float* X, const uint8_t* Y, float* Xb,
                               uint8_t* Yb, cudaStream_t s) {
    if (rows == 0) return cudaSuccess;
    gather_rows_kernel<<<nblk((long long)rows * IN, 256), 256, 0, s>>>(rows, idx, X, Y, Xb, Yb);
    return cudaGetLastError();
}

}  // namespace sel
}  // namespace mgpu
