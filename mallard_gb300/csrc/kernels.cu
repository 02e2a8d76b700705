// kernels.cu -- sm_103a kernels of the Mallard residual-and-update path, FP64.
//
// Compiled with -fmad=false: every a*b+c below rounds twice, as in the
// reference's (non-FMA) CPU build, and each expression keeps the
// reference's operation order, so that results agree with the reference bit
// for bit wherever the reference's math library agrees with correctly
// rounded results.  Where an explicit fma() appears it is part of an
// error-free transformation (exact products), not a contraction.
//
// Per stage the host launches: reconstruction (TENO or first order) ->
// face flux -> gather/update; once per step the spectral radius and dt.
// The gather replaces the reference's atomic scatter: each cell sums its
// faces' fluxes in the order the reference's serial build adds them, so the
// residual is deterministic and identical to Kokkos::Serial's.
#include <cstdint>

#include "physics.cuh"

namespace mgpu {

namespace {

// FirstOrderFunctor (face_reconstruction.cpp:59-99): both sides take the
// adjacent cell averages; boundary faces fill side 0 only.
__global__ void __launch_bounds__(256) first_order_kernel(int n_faces, const int2* __restrict__ lr,
                                                          const double* __restrict__ U, double* __restrict__ fv) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = gt >> 2, v = gt & 3;
    if (f >= n_faces) return;
    const int2 c = lr[f];
    fv[(size_t)f * 8 + v] = U[(size_t)c.x * NC + v];
    if (c.y >= 0) fv[(size_t)f * 8 + 4 + v] = U[(size_t)c.y * NC + v];
}

// ---------------------------------------------------------------------------
// Residual gather + SSPRK3 stage update (solver_rhs.cpp:18-55,
// time_integrator.cpp:135-163, solver.cpp:533-578)
// ---------------------------------------------------------------------------

template <int STAGE>
__global__ void __launch_bounds__(256) update_kernel(const UpdateArgs a, const GasParams g) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const int4 gl = a.gat[c];
    const int ent[4] = {gl.x, gl.y, gl.z, gl.w};
    double r[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        if (ent[e] < 0) break;
        const double2* Gf = reinterpret_cast<const double2*>(a.G + (size_t)(ent[e] >> 1) * 4);
        const double2 g0 = Gf[0], g1 = Gf[1];
        const double x[4] = {g0.x, g0.y, g1.x, g1.y};
        if (ent[e] & 1) {
#pragma unroll
            for (int i = 0; i < 4; i++) r[i] = r[i] + (-x[i]);
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) r[i] = r[i] + x[i];
        }
    }
    const double vol = a.vol[c];
#pragma unroll
    for (int i = 0; i < 4; i++) r[i] = r[i] / vol;
    double2* out2;
    if (STAGE == 0) {
        out2 = reinterpret_cast<double2*>(a.rhs + (size_t)c * 4);
        out2[0] = make_double2(r[0], r[1]);
        out2[1] = make_double2(r[2], r[3]);
        return;
    }
    const double dt = *a.dt;
    const double2* U2 = reinterpret_cast<const double2*>(a.U + (size_t)c * 4);
    const double2* W2 = reinterpret_cast<const double2*>(a.W + (size_t)c * 4);
    double2* Ut2 = reinterpret_cast<double2*>(a.Ut + (size_t)c * 4);
    double2* Wo2 = reinterpret_cast<double2*>(a.W + (size_t)c * 4);
    if (STAGE == 1) {
        const double2 u0 = U2[0], u1 = U2[1];
        const double u[4] = {u0.x, u0.y, u1.x, u1.y};
        const double c1 = dt * (1.0 / 6.0);
        double t[4], w[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            t[i] = u[i] + dt * r[i];
            w[i] = u[i] + c1 * r[i];
        }
        Ut2[0] = make_double2(t[0], t[1]);
        Ut2[1] = make_double2(t[2], t[3]);
        Wo2[0] = make_double2(w[0], w[1]);
        Wo2[1] = make_double2(w[2], w[3]);
    } else if (STAGE == 2) {
        const double2 u0 = U2[0], u1 = U2[1], s0 = Ut2[0], s1 = Ut2[1], w0 = W2[0], w1 = W2[1];
        const double u[4] = {u0.x, u0.y, u1.x, u1.y};
        const double s[4] = {s0.x, s0.y, s1.x, s1.y};
        double w[4] = {w0.x, w0.y, w1.x, w1.y};
        const double c1 = dt * (1.0 / 6.0), q = dt / 4.0;
        double t[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            t[i] = 3.0 / 4.0 * u[i] + 1.0 / 4.0 * s[i];
            t[i] = t[i] + q * r[i];
            w[i] = w[i] + c1 * r[i];
        }
        Ut2[0] = make_double2(t[0], t[1]);
        Ut2[1] = make_double2(t[2], t[3]);
        Wo2[0] = make_double2(w[0], w[1]);
        Wo2[1] = make_double2(w[2], w[3]);
    } else {
        const double2 w0 = W2[0], w1 = W2[1];
        const double w[4] = {w0.x, w0.y, w1.x, w1.y};
        const double c3 = dt * (2.0 / 3.0);
        double u[4];
#pragma unroll
        for (int i = 0; i < 4; i++) u[i] = w[i] + c3 * r[i];
        double2* Uo2 = reinterpret_cast<double2*>(a.U + (size_t)c * 4);
        Uo2[0] = make_double2(u[0], u[1]);
        Uo2[1] = make_double2(u[2], u[3]);
        double p[5];
        primitives(g, u, p);
        double* po = a.prim + (size_t)c * NPR;
#pragma unroll
        for (int i = 0; i < NPR; i++) po[i] = p[i];
        bool ok = true;
#pragma unroll
        for (int i = 0; i < 4; i++) ok = ok && isfinite(u[i]);
        if (!ok) atomicOr(a.flags, 1u);
    }
}

// ---------------------------------------------------------------------------
// Spectral radius and dt (solver.cpp:580-742)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) spectral_kernel(const SpecArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double tot = 0.0;
    if (c < a.n_cells) {
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
            const double rl = a.U[(size_t)L * NC], rr = a.U[(size_t)R * NC];
            const double* wl = a.prim + (size_t)L * NPR;
            const double* wr = a.prim + (size_t)R * NPR;
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
        a.rho_cell[c] = tot;
    }
    // block max of positive doubles via their bit patterns
    unsigned long long bits = c < a.n_cells ? (unsigned long long)__double_as_longlong(tot) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
        bits = other > bits ? other : bits;
    }
    __shared__ unsigned long long red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = bits;
    __syncthreads();
    if (threadIdx.x < 32) {
        bits = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
            bits = other > bits ? other : bits;
        }
        if (threadIdx.x == 0) atomicMax(a.rmax_bits, bits);
    }
}

__global__ void dt_kernel(const unsigned long long* rmax_bits, double cfl, double* dt, double* t, unsigned* flags) {
    const double rmax = __longlong_as_double((long long)*rmax_bits);
    const double d = cfl / rmax;
    *dt = d;
    if (!(d >= 0.0) || !isfinite(d)) atomicOr(flags, 2u);
    if (t) *t = *t + d;
}

__global__ void set_scalar_kernel(double* dst, double value) { *dst = value; }

// Row permutations between the caller's cell order and the internal one:
// gather: dst[c] = src[idx[c]]; scatter: dst[idx[c]] = src[c].
__global__ void permute_rows_kernel(int n, int width, const uint32_t* __restrict__ idx, const double* __restrict__ src,
                                    double* __restrict__ dst, int scatter) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * width) return;
    const int c = (int)(t / width), k = (int)(t % width);
    const size_t o = idx[c];
    if (scatter) dst[o * width + k] = src[(size_t)c * width + k];
    else dst[(size_t)c * width + k] = src[o * width + k];
}

// ---------------------------------------------------------------------------
// Unit-level kernels
// ---------------------------------------------------------------------------

// buf: per problem 13 doubles: n0 n1 rho_l ul0 ul1 p_l gamma_l h_l rho_r ur0 ur1 p_r gamma_r h_r ... (14)
template <int RS>
__global__ void riemann_batch_kernel(uint32_t n, const double* __restrict__ in, double* __restrict__ flux) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* b = in + (size_t)i * 14;
    const double nn[2] = {b[0], b[1]};
    const double ul[2] = {b[3], b[4]};
    const double ur[2] = {b[9], b[10]};
    double F[4];
    riemann<RS>(F, nn, b[2], ul, b[5], b[6], b[7], b[8], ur, b[11], b[12], b[13]);
#pragma unroll
    for (int k = 0; k < 4; k++) flux[(size_t)i * 4 + k] = F[k];
}

__global__ void primitives_batch_kernel(const GasParams g, uint32_t n, const double* __restrict__ U,
                                        double* __restrict__ W) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double u[4], w[5];
#pragma unroll
    for (int k = 0; k < 4; k++) u[k] = U[(size_t)i * 4 + k];
    primitives(g, u, w);
#pragma unroll
    for (int k = 0; k < 5; k++) W[(size_t)i * 5 + k] = w[k];
}

// Independent FMA chains; 2 flops per fma.
__global__ void fp64_probe_kernel(double* out, int iters, double seed) {
    double a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
           a7 = a0 + 7;
    const double m = 0.999999999, c = 1e-9;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
        a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
    const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.678) out[0] = s;  // keeps the chains live
}

}  // namespace

cudaError_t launch_first_order(int n_faces, const int2* lr, const double* U, double* fv, cudaStream_t s) {
    const long long threads = (long long)n_faces * 4;
    const unsigned blocks = (unsigned)((threads + 255) / 256);
    if (blocks == 0) return cudaSuccess;
    first_order_kernel<<<blocks, 256, 0, s>>>(n_faces, lr, U, fv);
    return cudaGetLastError();
}

cudaError_t launch_update(const UpdateArgs& a, const GasParams& g, int stage, cudaStream_t s) {
    const unsigned blocks = (unsigned)((a.n_cells + 255) / 256);
    if (blocks == 0) return cudaSuccess;
    switch (stage) {
        case 0: update_kernel<0><<<blocks, 256, 0, s>>>(a, g); break;
        case 1: update_kernel<1><<<blocks, 256, 0, s>>>(a, g); break;
        case 2: update_kernel<2><<<blocks, 256, 0, s>>>(a, g); break;
        case 3: update_kernel<3><<<blocks, 256, 0, s>>>(a, g); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_spectral(const SpecArgs& a, cudaStream_t s) {
    const unsigned blocks = (unsigned)((a.n_cells + 255) / 256);
    if (blocks == 0) return cudaSuccess;
    spectral_kernel<<<blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_dt(const unsigned long long* rmax_bits, double cfl, double* dt, double* t, unsigned* flags,
                      cudaStream_t s) {
    dt_kernel<<<1, 1, 0, s>>>(rmax_bits, cfl, dt, t, flags);
    return cudaGetLastError();
}

cudaError_t launch_set_scalar(double* dst, double value, cudaStream_t s) {
    set_scalar_kernel<<<1, 1, 0, s>>>(dst, value);
    return cudaGetLastError();
}

cudaError_t launch_permute_rows(int n, int width, const uint32_t* idx, const double* src, double* dst, bool scatter,
                                cudaStream_t s) {
    const long long threads = (long long)n * width;
    const unsigned blocks = (unsigned)((threads + 255) / 256);
    if (blocks == 0) return cudaSuccess;
    permute_rows_kernel<<<blocks, 256, 0, s>>>(n, width, idx, src, dst, scatter ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_riemann_batch(int rsolver, uint32_t n, const double* in, double* flux, cudaStream_t s) {
    const unsigned blocks = (n + 127) / 128;
    if (blocks == 0) return cudaSuccess;
    switch (rsolver) {
        case MGPU_RIEMANN_RUSANOV: riemann_batch_kernel<MGPU_RIEMANN_RUSANOV><<<blocks, 128, 0, s>>>(n, in, flux); break;
        case MGPU_RIEMANN_HLL: riemann_batch_kernel<MGPU_RIEMANN_HLL><<<blocks, 128, 0, s>>>(n, in, flux); break;
        case MGPU_RIEMANN_HLLC: riemann_batch_kernel<MGPU_RIEMANN_HLLC><<<blocks, 128, 0, s>>>(n, in, flux); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_primitives_batch(const GasParams& g, uint32_t n, const double* U, double* W, cudaStream_t s) {
    const unsigned blocks = (n + 127) / 128;
    if (blocks == 0) return cudaSuccess;
    primitives_batch_kernel<<<blocks, 128, 0, s>>>(g, n, U, W);
    return cudaGetLastError();
}

cudaError_t run_fp64_probe(int device, double* gflops) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return e;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    double* out = nullptr;
    if ((e = cudaMalloc(&out, sizeof(double))) != cudaSuccess) return e;
    const int blocks = sms * 8, threads = 256, iters = 4096;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    fp64_probe_kernel<<<blocks, threads>>>(out, 64, 1.0);  // warm-up
    cudaEventRecord(a);
    fp64_probe_kernel<<<blocks, threads>>>(out, iters, 1.0);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return e;
    const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    *gflops = flops / (ms * 1e-3) / 1e9;
    return cudaGetLastError();
}

}  // namespace mgpu
