// stage.cuh -- the residual gather and RK stage update (fused with the
// primitive recovery, the FP32 copy of the state and the NaN flag), and the
// spectral radius, shared by two translation units: kernels.cu instantiates
// the exact forms (-fmad=false: the reference's roundings) and
// kernels_fast.cu the fast forms (FP64-fast and FP32: -fmad=true, so that
// a*b+c contracts to one FMA on GB300's scarce FP64 unit), including the
// batched form's kernels.
#pragma once

#include <cstdint>

#include "device.h"
#include "fp_convert.cuh"
#include "physics.cuh"
#include "spectral32.cuh"

namespace mgpu {

// The fast forms' launchers (kernels_fast.cu), for kernels.cu's dispatch.
cudaError_t update_fast(const UpdateArgs& a, const GasParams& g, int stage, int scheme, unsigned blocks,
                        cudaStream_t s);
cudaError_t spectral_fast(const SpecArgs& a, unsigned blocks, cudaStream_t s);

namespace stage {
namespace {  // each translation unit keeps its own instantiations

// ---------------------------------------------------------------------------
// Residual gather + SSPRK3 stage update (solver_rhs.cpp:18-55,
// time_integrator.cpp:135-163, solver.cpp:533-578)
// ---------------------------------------------------------------------------

// Primitive recovery of the fast forms: one reciprocal of the density (and a
// precomputed 1/cv) instead of five divisions.
__device__ __forceinline__ void primitives_rcp(const GasParams& g, const double* U, double* W) {
    const double rho = U[0], ir = 1.0 / rho;
    const double u0 = U[1] * ir, u1 = U[2] * ir;
    const double E = U[3] * ir;
    const double e = E - 0.5 * (u0 * u0 + u1 * u1);
    const double p = fmax(g.p_min, fmin(g.p_max, (g.gamma - 1.0) * rho * e));
    W[0] = u0;
    W[1] = u1;
    W[2] = p;
    W[3] = e * g.icv;
    W[4] = e + p * ir;
}

// Sound speed of a cell, as the spectral radius evaluates it per face
// (solver.cpp:662-696); stored once per cell, bit for bit the same value.
__device__ __forceinline__ double sound_speed(double gamma, double rho, const double* W) {
    return sqrt(gamma * W[2] / rho);
}

// Row indices (see fp32_fast.cu): one case, or case cs of a batch group
// whose rows are interleaved per 8-row tile.
struct Ix1 {
    __device__ __forceinline__ size_t u(size_t c) const { return c; }
    __device__ __forceinline__ size_t f(size_t fi) const { return fi; }
};
struct IxB {
    size_t ubase, fbase;
    unsigned C, cs;
    __device__ __forceinline__ size_t u(size_t c) const { return ubase + (((c >> 3) * C + cs) << 3) + (c & 7); }
    __device__ __forceinline__ size_t f(size_t fi) const { return fbase + (((fi >> 3) * C + cs) << 3) + (fi & 7); }
};

// FAST: residual times a precomputed 1/volume and primitives_rcp (the
// FP64-fast and FP32 forms); otherwise the reference's divisions.
// Cell c (local index) of one case; dt and the NaN flag are the case's.
// State arrays an update reads and writes (one case's, or a batch's).
struct StageState {
    const double* G;
    double *U, *Ut, *W, *rhs;
    double *prim, *snd;  // null in the FP32 form, which recovers them on demand
    float* u32;          // FP32 copy of the stage's output state, or null
};

__device__ __forceinline__ void store_f32(float* dst, const double* x) {
    *reinterpret_cast<float4*>(dst) = make_float4(f32_rn(x[0]), f32_rn(x[1]), f32_rn(x[2]), f32_rn(x[3]));
}

// SCHEME: MGPU_INTEGRATOR_*; STAGE 1.. its stages (the last one writes U,
// the primitives and the NaN flag), 0 the residual alone.
template <int STAGE, bool FAST, int SCHEME, class IX>
__device__ __forceinline__ void update_cell(const UpdateArgs& a, const StageState& st, const GasParams& g, int c,
                                            const IX& ix, const double* dtp, unsigned* flag) {
    const size_t row = ix.u(c);
    const int4 gl = a.gat[c];
    const int ent[4] = {gl.x, gl.y, gl.z, gl.w};
    double r[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        if (ent[e] < 0) break;
        const double2* Gf = reinterpret_cast<const double2*>(st.G + ix.f((size_t)(ent[e] >> 1)) * 4);
        const double2 g0 = Gf[0], g1 = Gf[1];
        const double x[4] = {g0.x, g0.y, g1.x, g1.y};
        if (FAST && e == 0) {
            // the first contribution starts the sum (0 + x is x but for the
            // sign of a zero): one FP64 add less per variable
#pragma unroll
            for (int i = 0; i < 4; i++) r[i] = (ent[e] & 1) ? -x[i] : x[i];
        } else if (ent[e] & 1) {
#pragma unroll
            for (int i = 0; i < 4; i++) r[i] = r[i] + (-x[i]);
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) r[i] = r[i] + x[i];
        }
    }
    // FAST SSPRK3 stages fold 1/volume into their per-cell coefficients
    // (dt/volume, ...: one FP64 multiply each instead of four); elsewhere
    // iv stays 1 and the residual itself is scaled
    constexpr bool FOLD = FAST && STAGE > 0 && SCHEME == MGPU_INTEGRATOR_SSPRK3;
    double iv = 1.0;
    if (FOLD) {
        iv = a.ivol[c];
    } else if (FAST) {
        const double v = a.ivol[c];
#pragma unroll
        for (int i = 0; i < 4; i++) r[i] = r[i] * v;
    } else {
        const double vol = a.vol[c];
#pragma unroll
        for (int i = 0; i < 4; i++) r[i] = r[i] / vol;
    }
    double2* out2;
    if (STAGE == 0) {
        out2 = reinterpret_cast<double2*>(st.rhs + row * 4);
        out2[0] = make_double2(r[0], r[1]);
        out2[1] = make_double2(r[2], r[3]);
        return;
    }
    const double dt = *dtp;
    const double2* U2 = reinterpret_cast<const double2*>(st.U + row * 4);
    const double2* W2 = reinterpret_cast<const double2*>(st.W + row * 4);
    double2* Ut2 = reinterpret_cast<double2*>(st.Ut + row * 4);
    double2* Wo2 = reinterpret_cast<double2*>(st.W + row * 4);
    double u[4];  // the new state, on the scheme's last stage
    if (SCHEME == MGPU_INTEGRATOR_FE) {
        // FE::take_step (time_integrator.cpp:57-69): U += dt rhs
        const double2 u0 = U2[0], u1 = U2[1];
        const double v[4] = {u0.x, u0.y, u1.x, u1.y};
#pragma unroll
        for (int i = 0; i < 4; i++) u[i] = v[i] + dt * r[i];
    } else if (SCHEME == MGPU_INTEGRATOR_RK4) {
        // RK4::take_step (time_integrator.cpp:85-120), coefficients (:71-79):
        // U_temp = U + (dt/2) k1,
        // U + (dt/2) k2, U + dt k3; U += dt/6 k1 + dt/3 k2 + dt/3 k3 + dt/6 k4,
        // accumulated in W in that order
        const double cs = STAGE == 1 ? dt * (1.0 / 6.0) : (STAGE == 4 ? dt * (1.0 / 6.0) : dt * (1.0 / 3.0));
        const double2 w0 = W2[0], w1 = W2[1];
        if (STAGE < 4) {
            const double2 u0 = U2[0], u1 = U2[1];
            const double v[4] = {u0.x, u0.y, u1.x, u1.y};
            const double h = STAGE == 3 ? dt : dt / 2.0;
            double t[4], w[4] = {w0.x, w0.y, w1.x, w1.y};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                t[i] = v[i] + h * r[i];
                w[i] = (STAGE == 1 ? v[i] : w[i]) + cs * r[i];
            }
            Ut2[0] = make_double2(t[0], t[1]);
            Ut2[1] = make_double2(t[2], t[3]);
            Wo2[0] = make_double2(w[0], w[1]);
            Wo2[1] = make_double2(w[2], w[3]);
            if (st.u32) store_f32(st.u32 + row * 4, t);
            return;
        }
        const double w[4] = {w0.x, w0.y, w1.x, w1.y};
#pragma unroll
        for (int i = 0; i < 4; i++) u[i] = w[i] + cs * r[i];
    } else if (STAGE == 1) {
        const double2 u0 = U2[0], u1 = U2[1];
        const double u[4] = {u0.x, u0.y, u1.x, u1.y};
        const double ht = dt * iv, hw = dt * (1.0 / 6.0) * iv;
        double t[4], w[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            t[i] = u[i] + ht * r[i];
            w[i] = u[i] + hw * r[i];
        }
        Ut2[0] = make_double2(t[0], t[1]);
        Ut2[1] = make_double2(t[2], t[3]);
        Wo2[0] = make_double2(w[0], w[1]);
        Wo2[1] = make_double2(w[2], w[3]);
        if (st.u32) store_f32(st.u32 + row * 4, t);
        return;
    } else if (STAGE == 2 && FOLD) {
        // 3/4 U + 1/4 (U + dt k1) + dt/4 k2 = U + dt/4 (k1 + k2) = U + 3/2 (W - U) with
        // the running sum W = U + dt/6 (k1 + k2): no read of the stage state
        const double2 u0 = U2[0], u1 = U2[1], w0 = W2[0], w1 = W2[1];
        const double u[4] = {u0.x, u0.y, u1.x, u1.y};
        double w[4] = {w0.x, w0.y, w1.x, w1.y};
        const double c1 = dt * (1.0 / 6.0) * iv;
        double t[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            w[i] = w[i] + c1 * r[i];
            t[i] = u[i] + 1.5 * (w[i] - u[i]);
        }
        Ut2[0] = make_double2(t[0], t[1]);
        Ut2[1] = make_double2(t[2], t[3]);
        Wo2[0] = make_double2(w[0], w[1]);
        Wo2[1] = make_double2(w[2], w[3]);
        if (st.u32) store_f32(st.u32 + row * 4, t);
        return;
    } else if (STAGE == 2) {
        const double2 u0 = U2[0], u1 = U2[1], s0 = Ut2[0], s1 = Ut2[1], w0 = W2[0], w1 = W2[1];
        const double u[4] = {u0.x, u0.y, u1.x, u1.y};
        const double s[4] = {s0.x, s0.y, s1.x, s1.y};
        double w[4] = {w0.x, w0.y, w1.x, w1.y};
        const double c1 = dt * (1.0 / 6.0) * iv, q = dt / 4.0 * iv;
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
        if (st.u32) store_f32(st.u32 + row * 4, t);
        return;
    } else {
        const double2 w0 = W2[0], w1 = W2[1];
        const double w[4] = {w0.x, w0.y, w1.x, w1.y};
        const double c3 = dt * (2.0 / 3.0) * iv;
#pragma unroll
        for (int i = 0; i < 4; i++) u[i] = w[i] + c3 * r[i];
    }
    {
        double2* Uo2 = reinterpret_cast<double2*>(st.U + row * 4);
        Uo2[0] = make_double2(u[0], u[1]);
        Uo2[1] = make_double2(u[2], u[3]);
        if (st.u32) store_f32(st.u32 + row * 4, u);
        if (st.prim) {
            double p[5];
            if (FAST) primitives_rcp(g, u, p);
            else primitives(g, u, p);
            double* po = st.prim + row * NPR;
#pragma unroll
            for (int i = 0; i < NPR; i++) po[i] = p[i];
            st.snd[row] = sound_speed(g.gamma, u[0], p);
        }
        // finite: the exponent field is not all ones (inf, NaN), tested on
        // the high word's bits with integer instructions, which leaves the
        // FP64 unit (this kernel's limit on GB300) to the update itself
        unsigned bad = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) bad |= ((unsigned)__double2hiint(u[i]) & 0x7ff00000u) == 0x7ff00000u;
        if (bad) atomicOr(flag, 1u);
    }
}

template <int STAGE, bool FAST, int SCHEME>
__global__ void __launch_bounds__(256) update_kernel(const UpdateArgs a, const GasParams g) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const StageState st{a.G, a.U, a.Ut, a.W, a.rhs, a.prim, a.snd, a.u32};
    update_cell<STAGE, FAST, SCHEME>(a, st, g, c, Ix1{}, a.dt, a.flags);
}

// ---------------------------------------------------------------------------
// Spectral radius and dt (solver.cpp:580-742)
// ---------------------------------------------------------------------------

// The sound speeds come from the per-cell array written with the
// primitives.  FAST multiplies by precomputed 1/dxn instead of dividing.
template <bool FAST, class IX>
__device__ __forceinline__ double spectral_cell(const SpecArgs& a, const double* __restrict__ prim,
                                                const double* __restrict__ snd, int c, const IX& ix) {
    double tot;
    {
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
            const double* wl = prim + ix.u(L) * NPR;
            const double* wr = prim + ix.u(R) * NPR;
            const double al = snd[ix.u(L)], ar = snd[ix.u(R)];
            const double af = 0.5 * (al + ar);
            const double uf0 = 0.5 * (wl[0] + wr[0]), uf1 = 0.5 * (wl[1] + wr[1]);
            const double un = fabs(uf0 * n.x + uf1 * n.y);
            if (FAST) {
                const double idx = a.idxn[f];
                conv += un * idx;
                const double t = af * idx;
                acou += t * t;
            } else {
                const double dxn = a.dxn[f];
                conv += un / dxn;
                const double t = af / dxn;
                acou += t * t;
            }
        }
        const double geom = nf == 3 ? 1.0 : 0.75;  // 3.0 / nf, exactly
        conv *= 1.37 * geom;
        acou = 1.37 * sqrt(geom * acou);
        tot = conv + acou;
    }
    return tot;
}

// MODE 0: the reference's divisions; 1: the FP64-fast form; 2: the FP32
// form (spectral32.cuh, from the FP32 state rows).
template <int MODE>
__global__ void __launch_bounds__(256) spectral_kernel(const SpecArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double tot = 0.0;
    if (c < a.n_cells) {
        tot = MODE == 2 ? f64_of(spectral_cell32(a, c, Ix1{})) : spectral_cell<MODE == 1>(a, a.prim, a.snd, c, Ix1{});
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


// ---------------------------------------------------------------------------
// Batched form (see BatchLaunch): thread (case, cell); 8 consecutive threads
// are one 8-cell tile of one case.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int batch_group(const long long* start, int n, long long gt) {
    int g = 0;
    while (g + 1 < n && gt >= start[g + 1]) ++g;
    return g;
}

template <int STAGE>
__global__ void __launch_bounds__(256) update_batch_kernel(const BatchLaunch b, const GasParams g) {
    const long long total = b.cell0[b.n_groups];
    for (long long gt = (long long)blockIdx.x * 256 + threadIdx.x; gt < total; gt += (long long)gridDim.x * 256) {
        const int gi = batch_group(b.cell0, b.n_groups, gt);
        const unsigned t = (unsigned)(gt - b.cell0[gi]);
        const unsigned tc = t >> 3, C = b.C[gi], cs = tc % C;
        const int c = (int)(tc / C) * 8 + (int)(t & 7);
        const unsigned gc = b.case0[gi] + cs;
        if (c >= b.n_cells[gi] || b.flags[gc] != 0u) continue;
        const StageState st{b.G, b.U, b.Ut, b.W, nullptr, nullptr, nullptr, STAGE == 3 ? b.U32 : b.Ut32};
        update_cell<STAGE, true, MGPU_INTEGRATOR_SSPRK3>(b.upd[gi], st, g, c, IxB{b.ubase[gi], b.fbase[gi], C, cs}, b.dt + gc, b.flags + gc);
    }
}

// Spectral radius per cell (the FP32 form's, from the FP32 state rows),
// maximum per case (8 lanes of one case-tile reduce, then one atomic per
// tile).
__global__ void __launch_bounds__(256) spectral_batch_kernel(const BatchLaunch b) {
    const long long total = b.cell0[b.n_groups];
    for (long long gt = (long long)blockIdx.x * 256 + threadIdx.x; gt < total; gt += (long long)gridDim.x * 256) {
        const int gi = batch_group(b.cell0, b.n_groups, gt);
        const unsigned t = (unsigned)(gt - b.cell0[gi]);
        const unsigned tc = t >> 3, C = b.C[gi], cs = tc % C;
        const int c = (int)(tc / C) * 8 + (int)(t & 7);
        double tot = 0.0;
        if (c < b.n_cells[gi] && b.flags[b.case0[gi] + cs] == 0u)
            tot = f64_of(spectral_cell32(b.spec[gi], c, IxB{b.ubase[gi], b.fbase[gi], C, cs}));
        unsigned long long bits = (unsigned long long)__double_as_longlong(tot);
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
            bits = other > bits ? other : bits;
        }
        if ((t & 7) == 0) atomicMax(b.rmax + b.case0[gi] + cs, bits);
    }
}


template <bool FAST>
cudaError_t update_go(const UpdateArgs& a, const GasParams& g, int stage, int scheme, unsigned blocks,
                      cudaStream_t s) {
    constexpr int SS = MGPU_INTEGRATOR_SSPRK3, FE = MGPU_INTEGRATOR_FE, RK = MGPU_INTEGRATOR_RK4;
    if (stage == 0) {
        update_kernel<0, FAST, SS><<<blocks, 256, 0, s>>>(a, g);
    } else if (scheme == SS && stage <= 3) {
        if (stage == 1) update_kernel<1, FAST, SS><<<blocks, 256, 0, s>>>(a, g);
        else if (stage == 2) update_kernel<2, FAST, SS><<<blocks, 256, 0, s>>>(a, g);
        else update_kernel<3, FAST, SS><<<blocks, 256, 0, s>>>(a, g);
    } else if (scheme == FE && stage == 1) {
        update_kernel<1, FAST, FE><<<blocks, 256, 0, s>>>(a, g);
    } else if (scheme == RK && stage <= 4) {
        if (stage == 1) update_kernel<1, FAST, RK><<<blocks, 256, 0, s>>>(a, g);
        else if (stage == 2) update_kernel<2, FAST, RK><<<blocks, 256, 0, s>>>(a, g);
        else if (stage == 3) update_kernel<3, FAST, RK><<<blocks, 256, 0, s>>>(a, g);
        else update_kernel<4, FAST, RK><<<blocks, 256, 0, s>>>(a, g);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace
}  // namespace stage
}  // namespace mgpu
