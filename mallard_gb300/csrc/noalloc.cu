// noalloc.cu -- the CFL time step (spectral radius -> dt) without any device
// allocation at call time.
//
// Who needs it: callers that must not call cudaMalloc/cudaFree once they are
// stepping.  A host application that owns all device memory through its own
// pool or arena (so that a library allocating on its own would fragment the
// pool or overrun the budget it planned), and real-time loops, where the
// implicit device synchronisation of cudaMalloc/cudaFree would stall every
// stream, are two such callers.  They create their context once at start-up
// (which does allocate) and then call mgpu_calc_dt_noalloc every step with
// their own output buffers.
//
// The reduction scratch is a file-scope static device array of fixed size
// (kMaxBlocks partial maxima, 512 KiB), held by every GPU that loads the
// library until the process exits.  Each call writes one partial per block
// before reading any, so nothing has to be cleared between calls; calls that
// overlap on the GPU (two streams at once) share the array and race.
#include <cstdint>
#include <mutex>
#include <string>

#include "device.h"
#include "host.h"
#include "spectral32.cuh"

namespace mgpu {
// Defined in host_ctx.cpp: the context's spectral-radius inputs.
bool ctx_spectral_view(mgpu_ctx* ctx, SpecArgs* a, const uint32_t** cell_old, cudaStream_t* stream, int* device,
                       unsigned** flags);
}  // namespace mgpu

namespace {

constexpr int kBlock = 256;
constexpr int kMaxBlocks = 65536;  // one partial per block: at most 16,777,216 cells per call
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned long long g_partial_max[kMaxBlocks];

std::mutex g_setup_mutex;
unsigned long long* g_partial_addr[kMaxDevices] = {};

struct Rows {
    __device__ __forceinline__ size_t u(size_t c) const { return c; }
};

// Per cell: the spectral radius of the time-step kernel of the main path
// (SpectralRadiusFunctor, solver.cpp:634-706): the FP64 formula with the
// reference's divisions, or (F32) the FP32 form's radius from its FP32
// state rows, bit for bit; per block: the maximum, as the bit pattern of a
// non-negative double, written to this block's slot.
template <bool F32>
__global__ void __launch_bounds__(kBlock) spectral_partial_kernel(const mgpu::SpecArgs a,
                                                                 unsigned long long* __restrict__ partial,
                                                                 double* __restrict__ rho_out,
                                                                 const uint32_t* __restrict__ cell_old) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double tot = 0.0;
    if (F32 && c < a.n_cells) {
        tot = mgpu::f64_of(mgpu::spectral_cell32(a, c, Rows{}));
        if (rho_out) rho_out[cell_old[c]] = tot;
    } else if (c < a.n_cells) {
        const int4 cf = a.cfaces[c];
        const int ent[4] = {cf.x, cf.y, cf.z, cf.w};
        double conv = 0.0, acou = 0.0;
        int nf = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            if (ent[e] < 0) break;
            ++nf;
            const int f = ent[e];
            const int2 lr = a.lr[f];
            const int L = lr.x, R = lr.y < 0 ? lr.x : lr.y;
            const double2 n = a.nrm[f];
            const double dxn = a.dxn[f];
            const double rl = a.U[(size_t)L * 4], rr = a.U[(size_t)R * 4];
            const double* wl = a.prim + (size_t)L * 5;
            const double* wr = a.prim + (size_t)R * 5;
            const double al = sqrt(a.gamma * wl[2] / rl), ar = sqrt(a.gamma * wr[2] / rr);
            const double af = 0.5 * (al + ar);
            const double uf0 = 0.5 * (wl[0] + wr[0]), uf1 = 0.5 * (wl[1] + wr[1]);
            const double un = fabs(uf0 * n.x + uf1 * n.y);
            conv += un / dxn;
            const double t = af / dxn;
            acou += t * t;
        }
        const double geom = 3.0 / nf;
        conv *= 1.37 * geom;
        acou = 1.37 * sqrt(geom * acou);
        tot = conv + acou;
        if (rho_out) rho_out[cell_old[c]] = tot;
    }
    unsigned long long bits = c < a.n_cells ? (unsigned long long)__double_as_longlong(tot) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
        bits = other > bits ? other : bits;
    }
    __shared__ unsigned long long warp_max[kBlock / 32];
    if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = bits;
    __syncthreads();
    if (threadIdx.x < 32) {
        bits = threadIdx.x < (kBlock / 32) ? warp_max[threadIdx.x] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
            bits = other > bits ? other : bits;
        }
        if (threadIdx.x == 0) partial[blockIdx.x] = bits;
    }
}

// One block: the maximum over the used partial slots, then dt = cfl / max;
// a dt that is not a finite non-negative number sets bit 1 of the context's
// status word, as the main path's time-step kernel does.
__global__ void __launch_bounds__(1024) dt_from_partials_kernel(const unsigned long long* __restrict__ partial,
                                                                int n_partials, double cfl,
                                                                double* __restrict__ dt_out,
                                                                unsigned* __restrict__ flags) {
    unsigned long long bits = 0ull;
    for (int i = threadIdx.x; i < n_partials; i += blockDim.x) {
        const unsigned long long v = partial[i];
        bits = v > bits ? v : bits;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
        bits = other > bits ? other : bits;
    }
    __shared__ unsigned long long warp_max[32];
    if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = bits;
    __syncthreads();
    if (threadIdx.x < 32) {
        bits = threadIdx.x < (blockDim.x >> 5) ? warp_max[threadIdx.x] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
            bits = other > bits ? other : bits;
        }
        if (threadIdx.x == 0) {
            const double d = cfl / __longlong_as_double((long long)bits);
            *dt_out = d;
            if (!(d >= 0.0) || !isfinite(d)) atomicOr(flags, 2u);
        }
    }
}

// Device address of the scratch array for `device`, looked up once per device
// (with that device current) and cached.
cudaError_t partial_scratch(int device, unsigned long long** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partial_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_partial_max);
        if (e != cudaSuccess) return e;
        g_partial_addr[device] = static_cast<unsigned long long*>(p);
    }
    *out = g_partial_addr[device];
    return cudaSuccess;
}

}  // namespace

extern "C" int mgpu_calc_dt_noalloc(mgpu_ctx* ctx, double cfl, double* dt_device, double* spectral_radius_device) {
    mgpu::SpecArgs a{};
    const uint32_t* cell_old = nullptr;
    cudaStream_t stream = nullptr;
    unsigned* flags = nullptr;
    int device = 0;
    if (!ctx || !dt_device) {
        mgpu::set_error("mgpu_calc_dt_noalloc: null argument");
        return MGPU_ERR_ARG;
    }
    if (!mgpu::ctx_spectral_view(ctx, &a, &cell_old, &stream, &device, &flags)) {
        mgpu::set_error("mgpu_calc_dt_noalloc: context not finalized");
        return MGPU_ERR_STATE;
    }
    if (a.n_cells <= 0) {
        mgpu::set_error("mgpu_calc_dt_noalloc: the mesh has no cells");
        return MGPU_ERR_ARG;
    }
    const long long blocks = ((long long)a.n_cells + kBlock - 1) / kBlock;
    if (blocks > kMaxBlocks) {
        mgpu::set_error("mgpu_calc_dt_noalloc: mesh has " + std::to_string(a.n_cells) +
                        " cells; this entry point handles at most " + std::to_string((long long)kMaxBlocks * kBlock) +
                        " (use mgpu_calc_dt)");
        return MGPU_ERR_ARG;
    }
    // work on the context's device, then give the caller back its own
    int caller_device = -1;
    cudaError_t e = cudaGetDevice(&caller_device);
    if (e == cudaSuccess) e = cudaSetDevice(device);
    unsigned long long* partial = nullptr;
    if (e == cudaSuccess) e = partial_scratch(device, &partial);
    if (e == cudaSuccess) {
        if (a.u32)
            spectral_partial_kernel<true><<<(unsigned)blocks, kBlock, 0, stream>>>(a, partial, spectral_radius_device,
                                                                                  cell_old);
        else
            spectral_partial_kernel<false><<<(unsigned)blocks, kBlock, 0, stream>>>(a, partial, spectral_radius_device,
                                                                                   cell_old);
        e = cudaGetLastError();
        if (e == cudaSuccess) {
            dt_from_partials_kernel<<<1, 1024, 0, stream>>>(partial, (int)blocks, cfl, dt_device, flags);
            e = cudaGetLastError();
        }
    }
    if (caller_device >= 0 && caller_device != device) {
        const cudaError_t r = cudaSetDevice(caller_device);
        if (e == cudaSuccess) e = r;
    }
    if (e != cudaSuccess) {
        mgpu::set_error(std::string("mgpu_calc_dt_noalloc: ") + cudaGetErrorString(e));
        return MGPU_ERR_CUDA;
    }
    return MGPU_OK;
}
