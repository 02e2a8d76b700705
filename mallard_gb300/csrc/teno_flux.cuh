// teno_flux.cuh -- TENO reconstruction and face-flux kernels (FP64).
//
// Included twice: teno_flux_exact.cu (MGPU_FAST 0, compiled -fmad=false) keeps
// the reference's rounding step for step; teno_flux_fast.cu (MGPU_FAST 1,
// -fmad=true) lets the compiler fuse a*b+c and uses fewer FP64 instructions
// for the smoothness indicator, x^6 and the face evaluation.  The fast form
// agrees with the exact one to a few ulps per operation.
#pragma once

#include "physics.cuh"

#ifndef MGPU_NS
#error "define MGPU_NS and MGPU_FAST before including teno_flux.cuh"
#endif

namespace mgpu {
namespace MGPU_NS {
namespace {

// ---------------------------------------------------------------------------
// TENO reconstruction (face_reconstruction.cpp:866-1039)
// ---------------------------------------------------------------------------
// Four lanes per cell, one per conserved variable; eight cells per warp.
// Each lane keeps the reduced coefficients of all four stencils in
// registers until the weights are known, then writes its variable at the
// quadrature points of the cell's three faces.

// The robust variant's per-cell step (after the face values of all four
// variables are known): a cell with a boundary face takes its average at
// every face point; otherwise each variable's deviations from the average
// are scaled by one factor into the central stencil's range [dlo, dhi]
// (around the average), and a cell with a face state that is then not
// admissible (density positive and 2 rho E > |rho u|^2) takes its average
// at every face point.  live: the warp's lanes
// whose cells exist; the four lanes of a cell exchange their variables.
// Returns the factor the variable's polynomial was scaled by (1: kept, 0:
// replaced by the average).
template <int NF, int NQ>
__device__ __forceinline__ double robust_cell(const TenoArgs& a, int cell, unsigned live, double uc, double dlo,
                                              double dhi, double (&out)[NF][NQ]) {
    const bool boundary = a.bcell[cell] != 0;
    double th = 1.0;
    if (!boundary) {
#pragma unroll
        for (int fl = 0; fl < NF; ++fl)
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const double d = out[fl][q] - uc;
                if (d > dhi) th = fmin(th, dhi / d);
                else if (d < dlo) th = fmin(th, dlo / d);
            }
        if (th < 1.0)
#pragma unroll
            for (int fl = 0; fl < NF; ++fl)
#pragma unroll
                for (int q = 0; q < NQ; ++q) out[fl][q] = uc + th * (out[fl][q] - uc);
    }
    bool bad = boundary;
#pragma unroll
    for (int fl = 0; fl < NF; ++fl)
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const double rho = __shfl_sync(live, out[fl][q], 0, 4);
            const double m0 = __shfl_sync(live, out[fl][q], 1, 4);
            const double m1 = __shfl_sync(live, out[fl][q], 2, 4);
            const double E = __shfl_sync(live, out[fl][q], 3, 4);
            // density positive and 2 rho E > |rho u|^2 (pressure positive), no division
            const double m2 = m0 * m0 + m1 * m1;
            if (!(rho > 0.0 && 2.0 * rho * E > m2)) bad = true;
        }
    if (bad)
#pragma unroll
        for (int fl = 0; fl < NF; ++fl)
#pragma unroll
            for (int q = 0; q < NQ; ++q) out[fl][q] = uc;
    return bad ? 0.0 : th;
}

// Viscous gradients from the reconstruction: lane v holds the gradient
// (gx, gy) of conserved variable v's polynomial at the cell centroid and
// the cell average uc; the cell's lane 0 writes the (u, v, T) gradients
// (the averages' primitives, as uvT computes them, and the quotient rule).
__device__ __forceinline__ void write_visc_grad(const TenoArgs& a, int cell, int v, unsigned live, double uc,
                                                double gx, double gy) {
    double r[4], x[4], y[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        r[i] = __shfl_sync(live, uc, i, 4);
        x[i] = __shfl_sync(live, gx, i, 4);
        y[i] = __shfl_sync(live, gy, i, 4);
    }
    if (v != 0) return;
    const double rho = r[0];
#if MGPU_FAST
    const double ir = 1.0 / rho;
    const double u = r[1] * ir, w = r[2] * ir, E = r[3] * ir;
    const double ux = (x[1] - u * x[0]) * ir, uy = (y[1] - u * y[0]) * ir;
    const double vx = (x[2] - w * x[0]) * ir, vy = (y[2] - w * y[0]) * ir;
    const double ex = (x[3] - E * x[0]) * ir - (u * ux + w * vx), ey = (y[3] - E * y[0]) * ir - (u * uy + w * vy);
    const double icv = 1.0 / a.cv;
    const double Tx = ex * icv, Ty = ey * icv;
#else
    const double u = r[1] / rho, w = r[2] / rho, E = r[3] / rho;
    const double ux = (x[1] - u * x[0]) / rho, uy = (y[1] - u * y[0]) / rho;
    const double vx = (x[2] - w * x[0]) / rho, vy = (y[2] - w * y[0]) / rho;
    const double ex = (x[3] - E * x[0]) / rho - (u * ux + w * vx), ey = (y[3] - E * y[0]) / rho - (u * uy + w * vy);
    const double Tx = ex / a.cv, Ty = ey / a.cv;
#endif
    double* g = a.vgrad + (size_t)cell * 6;
    g[0] = ux;
    g[1] = uy;
    g[2] = vx;
    g[3] = vy;
    g[4] = Tx;
    g[5] = Ty;
}

template <int K, int M, int NQ, int VARIANT>
__global__ void __launch_bounds__(128) teno_kernel(const TenoArgs a, const double* __restrict__ U,
                                                   double* __restrict__ fv, uint8_t* __restrict__ masks) {
    constexpr int KR = K - 1, MR = M - 1, NF = 3, S = 4;
    constexpr bool ROBUST = VARIANT == MGPU_TENO_ROBUST;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int cell = gt >> 2, v = gt & 3;
    const bool vgrad = a.vgrad != nullptr;
    const unsigned live = (ROBUST || vgrad) ? __ballot_sync(0xffffffffu, cell < a.n_cells) : 0u;
    if (cell >= a.n_cells) return;
    const int tile = cell >> 3, lane = cell & 7;
    const double uc = U[(size_t)cell * NC + v];
    const unsigned sm = a.smask[cell];

    double coef[S][KR];
    double w[S];
    double dlo = 0.0, dhi = 0.0;  // the robust variant's central-stencil range around uc
#pragma unroll
    for (int s = 0; s < S; ++s) {
#pragma unroll
        for (int k = 0; k < KR; ++k) coef[s][k] = 0.0;
        w[s] = 0.0;
        if (!((sm >> s) & 1u)) continue;
        const size_t base = ((size_t)tile * S + s) * MR;
        const uint32_t* nbp = a.nb + base * TILE + lane;
        const double* arp = a.ar + base * TILE + lane;
        const double* Pp = a.P + base * KR * TILE + lane;
#pragma unroll 4
        for (int j = 0; j < MR; ++j) {
            const uint32_t nbj = __ldg(nbp + j * TILE);
            const double d = __ldg(U + (size_t)nbj * NC + v) - uc;
            const double b = __ldg(arp + j * TILE) * d;
            if (ROBUST && s == 0) {
                dlo = fmin(dlo, d);
                dhi = fmax(dhi, d);
            }
#pragma unroll
            for (int k = 0; k < KR; ++k) coef[s][k] = coef[s][k] + __ldg(Pp + (j * KR + k) * TILE) * b;
        }
        // smoothness indicator a^T (OI a), dof 0 omitted (its coefficient is exactly zero)
        double si = 0.0;
#if MGPU_FAST
        // OI is symmetric: a^T OI a = sum_i a_i (OI_ii a_i + sum_{l>i} 2 OI_il a_l)
#pragma unroll
        for (int i = 0; i < KR; ++i) {
            double oa = a.oi2[i * KR + i] * coef[s][i];
#pragma unroll
            for (int l = i + 1; l < KR; ++l) oa = oa + a.oi2[i * KR + l] * coef[s][l];
            si = si + coef[s][i] * oa;
        }
        const double x = si + 1.0e-12, x2 = x * x;
        w[s] = 1.0 / (x2 * x2 * x2);
#else
#pragma unroll
        for (int i = 0; i < KR; ++i) {
            double oa = 0.0;
#pragma unroll
            for (int l = 0; l < KR; ++l) oa = oa + a.oi[i * KR + l] * coef[s][l];
            si = si + coef[s][i] * oa;
        }
        w[s] = 1.0 / pow6(si + 1.0e-12);
#endif
    }

    // stencil selection (face_reconstruction.cpp:947-981)
    double sd = 0.0;
#pragma unroll
    for (int s = 1; s < S; ++s) sd = sd + w[s];
    unsigned mask = 0;
    if (w[0] / (sd + w[0]) > 1.0e-7) {
        w[0] = 1.0;
#pragma unroll
        for (int s = 1; s < S; ++s) w[s] = 0.0;
        mask = 1;
    } else {
#pragma unroll
        for (int s = 1; s < S; ++s)
            if (w[s] / sd > 1.0e-5) {
                w[s] = (1.0 / K);
                mask |= 1u << s;
            }
        if (VARIANT != MGPU_TENO_REFERENCE) {
            w[0] = 0.0;
#pragma unroll
            for (int s = 1; s < S; ++s)
                if (!((mask >> s) & 1u)) w[s] = 0.0;
        }
        sd = 0.0;
#pragma unroll
        for (int s = 1; s < S; ++s) sd = sd + w[s];
#pragma unroll
        for (int s = 1; s < S; ++s) w[s] = w[s] / sd;
    }
    if (masks) masks[(size_t)cell * NC + v] = (uint8_t)mask;
#if MGPU_FAST
    // fold each weight into its coefficients once instead of at every point
#pragma unroll
    for (int s = 0; s < S; ++s)
#pragma unroll
        for (int k = 0; k < KR; ++k) coef[s][k] *= w[s];
#endif

    // face states at the quadrature points
    double outv[NF][NQ];
    uint32_t slots[NF];
#pragma unroll
    for (int fl = 0; fl < NF; ++fl) {
        slots[fl] = __ldg(a.cface + ((size_t)tile * NF + fl) * TILE + lane);
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const double* php = a.phi + (((size_t)tile * NF + fl) * NQ + q) * KR * TILE + lane;
            double phi[KR];
#pragma unroll
            for (int k = 0; k < KR; ++k) phi[k] = __ldg(php + k * TILE);
            double out = uc;
#pragma unroll
            for (int s = 0; s < S; ++s) {
                if (w[s] == 0.0) continue;
#pragma unroll
#if MGPU_FAST
                for (int k = 0; k < KR; ++k) out = out + coef[s][k] * phi[k];
#else
                for (int k = 0; k < KR; ++k) out = out + (w[s] * coef[s][k]) * phi[k];
#endif
            }
            outv[fl][q] = out;
        }
    }
    // the polynomial's gradient at the centroid (d/dxi, then the frame's
    // inverse Jacobian), summed in the face evaluation's order
    double gx = 0.0, gy = 0.0;
    if (vgrad) {
        double g0 = 0.0, g1 = 0.0;
#pragma unroll
        for (int s = 0; s < S; ++s) {
            if (w[s] == 0.0) continue;
#pragma unroll
            for (int k = 0; k < KR; ++k) {
#if MGPU_FAST
                g0 = g0 + coef[s][k] * a.dphi[2 * k];
                g1 = g1 + coef[s][k] * a.dphi[2 * k + 1];
#else
                const double ck = w[s] * coef[s][k];
                g0 = g0 + ck * a.dphi[2 * k];
                g1 = g1 + ck * a.dphi[2 * k + 1];
#endif
            }
        }
        const double* J = a.ji + (size_t)cell * 4;
        gx = J[0] * g0 + J[2] * g1;
        gy = J[1] * g0 + J[3] * g1;
    }
    if (ROBUST) {
        const double keep = robust_cell<NF, NQ>(a, cell, live, uc, dlo, dhi, outv);
        if (keep == 0.0) {
            gx = 0.0;
            gy = 0.0;
        } else if (keep < 1.0) {
            gx = keep * gx;
            gy = keep * gy;
        }
    }
    if (vgrad) write_visc_grad(a, cell, v, live, uc, gx, gy);
#pragma unroll
    for (int fl = 0; fl < NF; ++fl) {
        const size_t f = slots[fl] >> 1;
        const unsigned side = slots[fl] & 1u;
#pragma unroll
        for (int q = 0; q < NQ; ++q) fv[((f * NQ + q) * 2 + side) * NC + v] = outv[fl][q];
    }
}

// ---------------------------------------------------------------------------
// Face flux (flux_functor.h:124-178 and src/boundary/boundary_*.cpp)
// ---------------------------------------------------------------------------

template <int RS, int NQ, bool POSITIVITY>
__global__ void __launch_bounds__(128) flux_kernel(const FluxArgs a, const GasParams g, const BcTable bct) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.n_faces) return;
    const int2 lr = a.lr[f];
    const double2 nn = a.nrm[f];
    const double n[2] = {nn.x, nn.y};
    const int bi = a.bc[f];
    const int type = bi < 0 ? -1 : bct.bc[bi].type;
    double F[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const double2* fq = reinterpret_cast<const double2*>(a.fv + ((size_t)f * NQ + q) * 8);
        double cl[4], cr[4], pl[5], pr[5], Ft[4];
        {
            const double2 x0 = fq[0], x1 = fq[1];
            cl[0] = x0.x; cl[1] = x0.y; cl[2] = x1.x; cl[3] = x1.y;
        }
        if (type < 0) {
            const double2 x2 = fq[2], x3 = fq[3];
            cr[0] = x2.x; cr[1] = x2.y; cr[2] = x3.x; cr[3] = x3.y;
        }
        if (POSITIVITY) {
            if (!admissible(g, cl))
#pragma unroll
                for (int i = 0; i < 4; i++) cl[i] = a.U[(size_t)lr.x * NC + i];
            if (type < 0 && !admissible(g, cr))
#pragma unroll
                for (int i = 0; i < 4; i++) cr[i] = a.U[(size_t)lr.y * NC + i];
        }
        primitives(g, cl, pl);
        if (type == MGPU_BC_WALL_ADIABATIC) {
            Ft[0] = 0.0;
            Ft[1] = pl[2] * n[0];
            Ft[2] = pl[2] * n[1];
            Ft[3] = 0.0;
        } else {
            if (type < 0) {
                primitives(g, cr, pr);
            } else if (type == MGPU_BC_SYMMETRY) {
                // right state = left state with the velocity reflected
#pragma unroll
                for (int i = 0; i < 4; i++) cr[i] = cl[i];
#pragma unroll
                for (int i = 0; i < NPR; i++) pr[i] = pl[i];
                const double un = pl[0] * n[0] + pl[1] * n[1];
                pr[0] = pl[0] - 2.0 * un * n[0];
                pr[1] = pl[1] - 2.0 * un * n[1];
            } else if (type == MGPU_BC_EXTRAPOLATION) {
#pragma unroll
                for (int i = 0; i < 4; i++) cr[i] = cl[i];
#pragma unroll
                for (int i = 0; i < NPR; i++) pr[i] = pl[i];
            } else if (type == MGPU_BC_UPT) {
                const double* d = bct.bc[bi].data;
                cr[0] = d[0];
#pragma unroll
                for (int i = 0; i < NPR; i++) pr[i] = d[i + 1];
            } else {  // MGPU_BC_P_OUT
                const double rho_l = cl[0];
                const double um = sqrt(pl[0] * pl[0] + pl[1] * pl[1]);
                const double sos = sqrt(g.gamma * pl[2] / rho_l);
                const double po = (um < sos) ? bct.bc[bi].data[0] : pl[2];
                const double T = pl[3];
                const double rho = po / (g.R * T);
                const double e = g.cv * T;
                cr[0] = rho;
                pr[0] = pl[0];
                pr[1] = pl[1];
                pr[2] = po;
                pr[3] = T;
                pr[4] = e + po / rho;
            }
            riemann<RS>(Ft, n, cl[0], pl, pl[2], g.gamma, pl[4], cr[0], pr, pr[2], g.gamma, pr[4], a.guard != 0);
        }
#pragma unroll
        for (int i = 0; i < 4; i++) F[i] += a.qw[q] * Ft[i];
    }
    const double area = a.area[f];
    double2* Gf = reinterpret_cast<double2*>(a.G + (size_t)f * 4);
    Gf[0] = make_double2(area * (F[0] * 0.5), area * (F[1] * 0.5));
    Gf[1] = make_double2(area * (F[2] * 0.5), area * (F[3] * 0.5));
}

template <int K, int M, int NQ>
cudaError_t teno_dispatch_variant(const TenoArgs& a, int variant, const double* U, double* fv, uint8_t* masks,
                                  cudaStream_t s) {
    const long long threads = (long long)a.n_cells * 4;
    const unsigned blocks = (unsigned)((threads + 127) / 128);
    if (blocks == 0) return cudaSuccess;
    if (variant == MGPU_TENO_CORRECTED)
        teno_kernel<K, M, NQ, MGPU_TENO_CORRECTED><<<blocks, 128, 0, s>>>(a, U, fv, masks);
    else if (variant == MGPU_TENO_ROBUST)
        teno_kernel<K, M, NQ, MGPU_TENO_ROBUST><<<blocks, 128, 0, s>>>(a, U, fv, masks);
    else
        teno_kernel<K, M, NQ, MGPU_TENO_REFERENCE><<<blocks, 128, 0, s>>>(a, U, fv, masks);
    return cudaGetLastError();
}

template <int RS, int NQ>
cudaError_t flux_dispatch_pos(const FluxArgs& a, const GasParams& g, const BcTable& bct, bool pos, cudaStream_t s) {
    const unsigned blocks = (unsigned)((a.n_faces + 127) / 128);
    if (blocks == 0) return cudaSuccess;
    if (pos) flux_kernel<RS, NQ, true><<<blocks, 128, 0, s>>>(a, g, bct);
    else flux_kernel<RS, NQ, false><<<blocks, 128, 0, s>>>(a, g, bct);
    return cudaGetLastError();
}

template <int RS>
cudaError_t flux_dispatch_nq(const FluxArgs& a, const GasParams& g, const BcTable& bct, int nq, bool pos,
                             cudaStream_t s) {
    switch (nq) {
        case 1: return flux_dispatch_pos<RS, 1>(a, g, bct, pos, s);
        case 2: return flux_dispatch_pos<RS, 2>(a, g, bct, pos, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_teno(const TenoArgs& a, int K, int M, int nq, int variant, const double* U, double* fv,
                        uint8_t* masks, cudaStream_t s) {
    if (K == 10 && M == 20 && nq == 2) return teno_dispatch_variant<10, 20, 2>(a, variant, U, fv, masks, s);
    if (K == 6 && M == 12 && nq == 1) return teno_dispatch_variant<6, 12, 1>(a, variant, U, fv, masks, s);
    if (K == 3 && M == 6 && nq == 1) return teno_dispatch_variant<3, 6, 1>(a, variant, U, fv, masks, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_flux(const FluxArgs& a, const GasParams& g, const BcTable& bct, int rsolver, int nq,
                        bool positivity, cudaStream_t s) {
    switch (rsolver) {
        case MGPU_RIEMANN_RUSANOV: return flux_dispatch_nq<MGPU_RIEMANN_RUSANOV>(a, g, bct, nq, positivity, s);
        case MGPU_RIEMANN_HLL: return flux_dispatch_nq<MGPU_RIEMANN_HLL>(a, g, bct, nq, positivity, s);
        case MGPU_RIEMANN_HLLC: return flux_dispatch_nq<MGPU_RIEMANN_HLLC>(a, g, bct, nq, positivity, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace MGPU_NS
}  // namespace mgpu
