// kernels_fast.cu -- the stage update and spectral radius of the fast
// forms (FP64-fast and FP32, single case and batched), from stage.cuh,
// compiled with -fmad=true: the update's a + b c terms, the primitive
// recovery and the spectral sums contract to FMAs (the FP64 unit is these
// kernels' limit on GB300).  The exact form's instantiations are in
// kernels.cu, compiled with -fmad=false.

#include "stage.cuh"

namespace mgpu {

using namespace stage;

cudaError_t update_fast(const UpdateArgs& a, const GasParams& g, int stage, int scheme, unsigned blocks,
                        cudaStream_t s) {
    return update_go<true>(a, g, stage, scheme, blocks, s);
}

cudaError_t spectral_fast(const SpecArgs& a, unsigned blocks, cudaStream_t s) {
    if (a.u32) spectral_kernel<2><<<blocks, 256, 0, s>>>(a);
    else spectral_kernel<1><<<blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_update_batch(const BatchLaunch& b, const GasParams& g, int stage, cudaStream_t s) {
    const long long blocks = (b.cell0[b.n_groups] + 255) / 256;
    if (blocks == 0) return cudaSuccess;
    switch (stage) {
        case 1: update_batch_kernel<1><<<(unsigned)blocks, 256, 0, s>>>(b, g); break;
        case 2: update_batch_kernel<2><<<(unsigned)blocks, 256, 0, s>>>(b, g); break;
        case 3: update_batch_kernel<3><<<(unsigned)blocks, 256, 0, s>>>(b, g); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_spectral_batch(const BatchLaunch& b, cudaStream_t s) {
    const long long blocks = (b.cell0[b.n_groups] + 255) / 256;
    if (blocks) spectral_batch_kernel<<<(unsigned)blocks, 256, 0, s>>>(b);
    return cudaGetLastError();
}

}  // namespace mgpu
