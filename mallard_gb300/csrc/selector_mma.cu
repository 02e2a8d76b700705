// selector_mma.cu -- inference of the learned stencil selector on the
// tcgen05 tensor cores (BF16 operands, FP32 accumulation in TMEM).
//
// One CTA evaluates the 96-64-64-32 MLP for 128 cells (M = 128 rows):
//   * the weight image (BF16, already in the tensor cores' shared-memory
//     layout) and the biases arrive with one cp.async.bulk copy tracked by
//     an mbarrier;
//   * four threads per cell (one per variable) build the cell's feature row
//     in BF16 in shared memory;
//   * one elected thread issues tcgen05.mma per 16-wide K slice (6, 4 and 4
//     per layer), accumulating into 64 TMEM columns, and commits to an
//     mbarrier;
//   * every warp reads its 32 TMEM lanes back (tcgen05.ld 32x32b), adds the
//     bias, applies GELU and writes the next layer's BF16 operand.
// Operands use the no-swizzle K-major layout: 8 x 16-byte core matrices,
// core matrix (row/8, k/8) at ((row/8) * K/8 + k/8) * 128 bytes, so the
// leading (K) byte offset is 128 and the stride (row) byte offset K/8 * 128.
// Every mbarrier wait is bounded; a CTA whose wait runs out raises an error
// flag, gives its copies a second bounded wait, frees its TMEM and returns.
#include <cstdint>

#include <cuda_bf16.h>

#include "fp_convert.cuh"
#include "selector.cuh"
#include "selector_launch.h"

namespace mgpu {
namespace sel {
namespace {

constexpr int ROWS = 128;
constexpr int TMEM_COLS = 64;
constexpr unsigned WAIT_LIMIT = 1u << 22;

// byte offsets inside the dynamic shared memory
constexpr int SM_W1 = 0;
constexpr int SM_W2 = SM_W1 + HID * IN * 2;   // 12288
constexpr int SM_W3 = SM_W2 + HID * HID * 2;  // 20480
constexpr int SM_B = SM_W3 + OUT * HID * 2;   // 24576: b1 b2 b3 (FP32)
constexpr int BLOB = SM_B + (HID + HID + OUT) * 4;  // 25216
// one activation buffer: each layer's operand is written after the previous
// layer's MMAs (which read the buffer) have completed
constexpr int SM_ACT = BLOB;                  // 128 x 96 BF16 (then 128 x 64, twice)
// the stencil neighbour ids of the CTA's 16 tiles (FP32 form's grouped
// layout), staged by one bulk copy for the feature gathers
constexpr int NB_GJ = (MR + 3) / 4;
constexpr int SM_NB = SM_ACT + ROWS * IN * 2;
constexpr int NB_TILE_BYTES = S * NB_GJ * TILE * 16;  // 2560
constexpr int SM_BAR = SM_NB + (ROWS / TILE) * NB_TILE_BYTES;
constexpr int SM_TOTAL = SM_BAR + 32;
constexpr int THREADS = ROWS * NV;            // one thread per (cell, variable)
static_assert(BLOB % 16 == 0 && SM_ACT % 128 == 0 && SM_NB % 16 == 0 && SM_BAR % 8 == 0, "alignment");
static_assert(BLOB == WEIGHT_IMAGE_BYTES, "weight image size");

// GELU of the inference epilogue with the hardware tanh (tanh.approx.f32,
// relative error about 2^-11): its output is rounded to BF16 (2^-8) next.
__device__ __forceinline__ float gelu_approx(float x) {
    const float c = 0.7978845608028654f;  // sqrt(2 / pi)
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(c * (x + 0.044715f * x * x * x)));
    return 0.5f * x * (1.0f + t);
}

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const uint32_t a = su32(bar);
    for (unsigned i = 0; i < WAIT_LIMIT; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     su32(dst)),
                 "l"(src), "r"(bytes), "r"(su32(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(TMEM_COLS) : "memory");
}
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// shared-memory matrix descriptor: no swizzle, K-major
__device__ __forceinline__ uint64_t desc(const void* p, uint32_t sbo) {
    const uint32_t a = su32(p);
    uint64_t d = (uint64_t)((a & 0x3FFFFu) >> 4);
    d |= (uint64_t)(128u >> 4) << 16;            // leading (K) byte offset
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;  // stride (row) byte offset
    d |= 1ull << 46;                              // descriptor version
    return d;
}
// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// byte offset of the 16-byte chunk (row, k..k+7) of a K-wide operand
__device__ __forceinline__ uint32_t chunk_off(int row, int k, int K) {
    return (uint32_t)((((row >> 3) * (K >> 3) + (k >> 3)) << 7) + ((row & 7) << 4));
}
__device__ __forceinline__ uint4 pack8(const float* x) {
    uint4 u;
    __nv_bfloat162 h;
    h = __floats2bfloat162_rn(x[0], x[1]);
    u.x = *reinterpret_cast<uint32_t*>(&h);
    h = __floats2bfloat162_rn(x[2], x[3]);
    u.y = *reinterpret_cast<uint32_t*>(&h);
    h = __floats2bfloat162_rn(x[4], x[5]);
    u.z = *reinterpret_cast<uint32_t*>(&h);
    h = __floats2bfloat162_rn(x[6], x[7]);
    u.w = *reinterpret_cast<uint32_t*>(&h);
    return u;
}

// the FP32 copy of the state is read as is
struct AsFloat {
    __device__ float operator()(float x) const { return x; }
};

// SRC 0: feature rows from X [n][IN]; SRC 1: features of cells 0..n-1 of a
// FP32-form context computed from U (the FP32 copy of the state).  Outputs (each optional): logits
// [n][OUT] and per (cell, variable) predictions: the predicted TENO mask,
// bit 7 set when the class probability reaches the threshold of its kind
// (central or directional; a probability p passes when sum_c exp(z_c - z_max)
// = 1/p is at most the limit 1/threshold).
// Thread t builds the features of row t / 4, variable t % 4; for the
// epilogues warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows) and
// columns 16 (w / 4) .. + 15.
template <int SRC>
__global__ void __launch_bounds__(THREADS, 2) mlp_kernel(const uint8_t* __restrict__ wimg, int n,
                                                      const float* __restrict__ X, const TenoArgs a,
                                                      const float* __restrict__ U, float lim_central,
                                                      float lim_directional,
                                                      float* __restrict__ logits, uint8_t* __restrict__ pred,
                                                      unsigned* __restrict__ err) {
    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t* bar_w = reinterpret_cast<uint64_t*>(smem + SM_BAR);
    uint64_t* bar_m = bar_w + 1;
    uint64_t* bar_n = bar_w + 2;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar_w + 3);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tile0 = blockIdx.x * (ROWS / TILE);
    const int n_tiles = SRC == 1 ? min(ROWS / TILE, (n + TILE - 1) / TILE - tile0) : 0;

    if (tid == 0) {
        mbar_init(bar_w, 1);
        mbar_init(bar_m, 1);
        mbar_init(bar_n, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (SRC == 1) {
            mbar_expect_tx(bar_n, (unsigned)(n_tiles * NB_TILE_BYTES));
            bulk_g2s(smem + SM_NB, reinterpret_cast<const uint8_t*>(a.nb4) + (size_t)tile0 * NB_TILE_BYTES,
                     (unsigned)(n_tiles * NB_TILE_BYTES), bar_n);
        }
    }
    if (warp == 0) tmem_alloc(tslot);
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tbase = *tslot;
    if (tid == 0) {
        mbar_expect_tx(bar_w, BLOB);
        bulk_g2s(smem, wimg, BLOB, bar_w);
    }

    // layer-0 operand: features of (row, v) in BF16
    uint8_t* act = smem + SM_ACT;
    bool ok_n = true;
    if (SRC == 1) ok_n = __syncthreads_and(mbar_wait(bar_n, 0));
    {
        const int row = tid >> 2, v = tid & 3, cell = blockIdx.x * ROWS + row;
        float x[PER_VAR];
        if (cell < n && ok_n) {
            if (SRC == 0) {
#pragma unroll
                for (int k = 0; k < PER_VAR; ++k) x[k] = X[(size_t)cell * IN + v * PER_VAR + k];
            } else {
                features<true>(a, U, cell, v, a.smask[cell], AsFloat{}, x,
                               reinterpret_cast<const uint4*>(smem + SM_NB), tile0);
            }
        } else {
#pragma unroll
            for (int k = 0; k < PER_VAR; ++k) x[k] = 0.0f;
        }
        // BF16 pairs (a variable's 20 entries do not fill whole 16-byte chunks)
#pragma unroll
        for (int k = 0; k < PER_VAR; k += 2) {
            const int kk = v * PER_VAR + k;
            __nv_bfloat162 h = __floats2bfloat162_rn(x[k], x[k + 1]);
            *reinterpret_cast<uint32_t*>(act + chunk_off(row, kk, IN) + (kk & 7) * 2) =
                *reinterpret_cast<uint32_t*>(&h);
        }
    }
    fence_async_smem();
    bool ok = mbar_wait(bar_w, 0) && ok_n;
    ok = __syncthreads_and(ok);

    const float* bias = reinterpret_cast<const float*>(smem + SM_B);
    const int erow = 32 * (warp & 3) + lane, cgrp = warp >> 2;
    const uint32_t tl = tbase + ((uint32_t)(32 * (warp & 3)) << 16) + 16 * cgrp;
    float out[16];
    int phase = 0;
#pragma unroll 1
    for (int layer = 0; layer < 3 && ok; ++layer) {
        const uint8_t* Bp = smem + (layer == 0 ? SM_W1 : (layer == 1 ? SM_W2 : SM_W3));
        const int K = layer == 0 ? IN : HID;
        tc_after();
        if (tid == 0) {
            const uint32_t id = layer == 2 ? idesc(ROWS, OUT) : idesc(ROWS, HID);
            for (int kk = 0; kk < K / 16; ++kk)
                mma(tbase, desc(act + kk * 256, (K / 8) * 128), desc(Bp + kk * 256, (K / 8) * 128), id, kk > 0);
            mma_commit(bar_m);
        }
        ok = mbar_wait(bar_m, phase & 1);
        ++phase;
        ok = __syncthreads_and(ok);
        if (!ok) break;
        tc_after();
        const float* b = bias + (layer == 0 ? 0 : (layer == 1 ? HID : 2 * HID));
        if (layer < 2) {
            // the MMAs that read act have completed: overwrite it with this layer's output
            tmem_ld16(tl, out);
#pragma unroll
            for (int i = 0; i < 16; ++i) out[i] = gelu_approx(out[i] + b[cgrp * 16 + i]);
            *reinterpret_cast<uint4*>(act + chunk_off(erow, cgrp * 16, HID)) = pack8(out);
            *reinterpret_cast<uint4*>(act + chunk_off(erow, cgrp * 16 + 8, HID)) = pack8(out + 8);
            fence_async_smem();
            tc_before();
            __syncthreads();
        } else if (cgrp < OUT / 16) {
            tmem_ld16(tl, out);
#pragma unroll
            for (int i = 0; i < 16; ++i) out[i] += b[cgrp * 16 + i];
        }
    }
    const int cell = blockIdx.x * ROWS + erow;
    if (!ok) {
        if (tid == 0) atomicOr(err, 1u);
        // give the copies and the last commit one more bounded wait
        mbar_wait(bar_w, 0);
        if (SRC == 1) mbar_wait(bar_n, 0);
        if (phase > 0) mbar_wait(bar_m, (phase - 1) & 1);
    } else if (cgrp < OUT / 16 && cell < n) {
        if (logits) {
#pragma unroll
            for (int i = 0; i < 16; ++i) logits[(size_t)cell * OUT + cgrp * 16 + i] = out[i];
        }
        if (pred) {
            // this warp holds heads 2 cgrp and 2 cgrp + 1
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const float* z = out + hh * NCLS;
                float mx = z[0];
                int arg = 0;
#pragma unroll
                for (int c = 1; c < NCLS; ++c)
                    if (z[c] > mx) {
                        mx = z[c];
                        arg = c;
                    }
                float sum = 0.0f;
#pragma unroll
                for (int c = 0; c < NCLS; ++c) sum += __expf(z[c] - mx);
                pred[(size_t)cell * NV + 2 * cgrp + hh] =
                    (uint8_t)(mask_of_class(arg) | (sum <= (arg == 0 ? lim_central : lim_directional) ? 0x80u : 0u));
            }
        }
    }
    tc_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase);
}

// Trust a confident prediction only where the same variable is confident in
// every face neighbour too: predictions made once per step then keep a
// one-cell margin to any discontinuity, more than it moves within a step.
__global__ void __launch_bounds__(256) trust_kernel(int n, const int4* __restrict__ cfaces,
                                                   const int2* __restrict__ lr, const uint32_t* __restrict__ pred,
                                                   uint32_t* __restrict__ trusted) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    uint32_t keep = pred[c] & 0x80808080u;
    const int4 cf = cfaces[c];
    const int fs[4] = {cf.x, cf.y, cf.z, cf.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        if (fs[e] < 0) break;
        const int2 o = lr[fs[e]];
        const int other = o.x == c ? o.y : o.x;
        if (other >= 0) keep &= pred[other];
    }
    trusted[c] = (pred[c] & 0x7f7f7f7fu) | keep;
}

}  // namespace

int mlp_smem_bytes() { return SM_TOTAL; }

cudaError_t launch_trust(int n, const int4* cfaces, const int2* lr, const uint8_t* pred, uint8_t* trusted,
                         cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    trust_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, cfaces, lr, reinterpret_cast<const uint32_t*>(pred),
                                                   reinterpret_cast<uint32_t*>(trusted));
    return cudaGetLastError();
}

cudaError_t mlp_prepare() {
    cudaError_t e = cudaFuncSetAttribute(mlp_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(mlp_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
}

namespace {
float limit_of(float threshold) { return threshold > 0.0f && threshold <= 1.0f ? 1.0f / threshold : 0.0f; }
}  // namespace

cudaError_t launch_mlp_rows(const uint8_t* wimg, int n, const float* X, float* logits, uint8_t* pred,
                            float thr_central, float thr_directional, unsigned* err, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    mlp_kernel<0><<<(n + ROWS - 1) / ROWS, THREADS, SM_TOTAL, s>>>(wimg, n, X, TenoArgs{}, nullptr,
                                                                    limit_of(thr_central),
                                                                    limit_of(thr_directional), logits, pred, err);
    return cudaGetLastError();
}

cudaError_t launch_mlp_cells(const uint8_t* wimg, const TenoArgs& a, const float* U, float thr_central,
                             float thr_directional, uint8_t* pred, unsigned* err, cudaStream_t s) {
    if (a.n_cells <= 0) return cudaSuccess;
    mlp_kernel<1><<<(a.n_cells + ROWS - 1) / ROWS, THREADS, SM_TOTAL, s>>>(
        wimg, a.n_cells, nullptr, a, U, limit_of(thr_central), limit_of(thr_directional), nullptr, pred, err);
    return cudaGetLastError();
}

}  // namespace sel
}  // namespace mgpu
