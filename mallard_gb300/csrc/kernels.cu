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

#include "device.h"

namespace mgpu {

namespace {

constexpr int NC = 4;
constexpr int NPR = 5;

// ---------------------------------------------------------------------------
// Euler physics (src/physics/physics.h:842-867)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void primitives(const GasParams& g, const double* U, double* W) {
    const double rho = U[0];
    const double u0 = U[1] / rho, u1 = U[2] / rho;
    const double E = U[3] / rho;
    const double e = E - 0.5 * (u0 * u0 + u1 * u1);
    const double p = fmax(g.p_min, fmin(g.p_max, (g.gamma - 1.0) * rho * e));
    W[0] = u0;
    W[1] = u1;
    W[2] = p;
    W[3] = e / g.cv;
    W[4] = e + p / rho;
}

// ---------------------------------------------------------------------------
// Riemann solvers (src/numerics/riemann_solver.h:205-519)
// ---------------------------------------------------------------------------

// star-region estimates; W = {rho, u_n, p, gamma}
__device__ __forceinline__ void pvrs(const double* L, const double* R, double& ps) {
    const double al = sqrt(L[3] * L[2] / L[0]);
    const double ar = sqrt(R[3] * R[2] / R[0]);
    const double rho_m = 0.5 * (L[0] + R[0]);
    const double a_m = 0.5 * (al + ar);
    ps = 0.5 * (L[2] + R[2]) + 0.5 * (L[1] - R[1]) * rho_m * a_m;
}

__device__ __noinline__ void trrs(const double* L, const double* R, double& ps) {
    const double al = sqrt(L[3] * L[2] / L[0]);
    const double ar = sqrt(R[3] * R[2] / R[0]);
    const double zl = (L[3] - 1.0) / (2.0 * L[3]);
    const double zr = (R[3] - 1.0) / (2.0 * R[3]);
    const double plr = pow((L[2] / R[2]), zl);
    const double us = (plr * L[1] / al + R[1] / ar + 2.0 * (1.0 - plr) / (L[3] - 1.0)) / (plr / al + 1.0 / ar);
    ps = 0.5 * (L[2] * pow((1.0 + (L[3] - 1.0) / (2.0 * al) * (L[1] - us)), (1.0 / zl)) +
                R[2] * pow((1.0 + (R[3] - 1.0) / (2.0 * ar) * (us - R[1])), (1.0 / zr)));
}

__device__ __noinline__ void tsrs(const double* L, const double* R, double& ps) {
    const double gl = (L[3] - 1.0) / (L[3] + 1.0);
    const double gr = (R[3] - 1.0) / (R[3] + 1.0);
    const double Al = 2.0 / (L[3] + 1.0) / L[0], Bl = gl * L[2];
    const double Ar = 2.0 / (R[3] + 1.0) / R[0], Br = gr * R[2];
    const double p0 = fmax(0.0, ps);
    const double ql = sqrt(Al / (p0 + Bl));
    const double qr = sqrt(Ar / (p0 + Br));
    ps = (ql * L[2] + qr * R[2] - (R[1] - L[1])) / (ql + qr);
}

// ANRS (riemann_solver.h:308-329); only p_star is used by HLL/HLLC.
__device__ __forceinline__ double anrs(const double* L, const double* R) {
    const double pmax = fmax(L[2], R[2]), pmin = fmin(L[2], R[2]);
    const double qmax = pmax / pmin;
    double ps;
    pvrs(L, R, ps);
    if ((qmax < 2.0) && (pmin <= ps) && (ps <= pmax)) return ps;
    if (ps < pmin) trrs(L, R, ps);
    else tsrs(L, R, ps);
    return ps;
}

template <int RS>
__device__ __forceinline__ void riemann(double* F, const double* n, double rl, const double* ul, double pl, double gl,
                                        double hl, double rr, const double* ur, double pr, double gr, double hr) {
    const double unl = ul[0] * n[0] + ul[1] * n[1];
    const double unr = ur[0] * n[0] + ur[1] * n[1];
    const double qql = ul[0] * ul[0] + ul[1] * ul[1];
    const double qqr = ur[0] * ur[0] + ur[1] * ur[1];
    const double al = sqrt(gl * pl / rl);
    const double ar = sqrt(gr * pr / rr);
    const double El = (hl + 0.5 * qql) * rl - pl;
    const double Er = (hr + 0.5 * qqr) * rr - pr;
    const double Ul[4] = {rl, rl * ul[0], rl * ul[1], El};
    const double Ur[4] = {rr, rr * ur[0], rr * ur[1], Er};
    const double Fl[4] = {rl * unl, rl * ul[0] * unl + pl * n[0], rl * ul[1] * unl + pl * n[1], (El + pl) * unl};
    const double Fr[4] = {rr * unr, rr * ur[0] * unr + pr * n[0], rr * ur[1] * unr + pr * n[1], (Er + pr) * unr};
    if (RS == MGPU_RIEMANN_RUSANOV) {
        const double smax = fmax(fabs(unl) + al, fabs(unr) + ar);
#pragma unroll
        for (int i = 0; i < 4; i++) F[i] = 0.5 * (Fl[i] + Fr[i] + smax * (Ul[i] - Ur[i]));
        return;
    }
    const double Wl[4] = {rl, unl, pl, gl}, Wr[4] = {rr, unr, pr, gr};
    const double ps = anrs(Wl, Wr);
    const double ql = (ps <= pl) ? 1.0 : sqrt(1.0 + (gl + 1.0) / (2.0 * gl) * (ps / pl - 1.0));
    const double qr = (ps <= pr) ? 1.0 : sqrt(1.0 + (gr + 1.0) / (2.0 * gr) * (ps / pr - 1.0));
    const double Sl = unl - al * ql;
    const double Sr = unr + ar * qr;
    if (RS == MGPU_RIEMANN_HLL) {
        if (0.0 <= Sl) {
#pragma unroll
            for (int i = 0; i < 4; i++) F[i] = Fl[i];
        } else if (Sr <= 0.0) {
#pragma unroll
            for (int i = 0; i < 4; i++) F[i] = Fr[i];
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) F[i] = (Sr * Fl[i] - Sl * Fr[i] + Sl * Sr * (Ur[i] - Ul[i])) / (Sr - Sl);
        }
        return;
    }
    const double Ss = (pr - pl + rl * unl * (Sl - unl) - rr * unr * (Sr - unr)) / (rl * (Sl - unl) - rr * (Sr - unr));
    if (0.0 <= Sl) {
#pragma unroll
        for (int i = 0; i < 4; i++) F[i] = Fl[i];
    } else if (Sr <= 0.0) {
#pragma unroll
        for (int i = 0; i < 4; i++) F[i] = Fr[i];
    } else {
        const double D[4] = {0.0, n[0], n[1], Ss};
        const double Plr = 0.5 * (pl + pr + rl * (Sl - unl) * (Ss - unl) + rr * (Sr - unr) * (Ss - unr));
        if (Ss >= 0.0) {
#pragma unroll
            for (int i = 0; i < 4; i++) F[i] = (Ss * (Sl * Ul[i] - Fl[i]) + Sl * Plr * D[i]) / (Sl - Ss);
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) F[i] = (Ss * (Sr * Ur[i] - Fr[i]) + Sr * Plr * D[i]) / (Sr - Ss);
        }
    }
}

// Correctly rounded x^6 (up to a 2^-100 relative window) from an exact
// double-double evaluation: x^2, x^4 = (x^2)^2, x^6 = x^4 x^2 with the
// rounding error of every product carried along (Dekker/Ogita-Rump-Oishi
// error-free products via fma).  Stands in for the reference's
// pow(x, 6.0), which its C library evaluates to within 0.52 ulp.
__device__ __forceinline__ double pow6(double x) {
    const double h2 = x * x;
    const double l2 = fma(x, x, -h2);
    const double h4 = h2 * h2;
    const double l4 = fma(h2, h2, -h4) + 2.0 * h2 * l2;
    const double h6 = h4 * h2;
    const double l6 = fma(h4, h2, -h6) + (h4 * l2 + l4 * h2);
    return h6 + l6;
}

// ---------------------------------------------------------------------------
// TENO reconstruction (face_reconstruction.cpp:866-1039)
// ---------------------------------------------------------------------------
// Four lanes per cell, one per conserved variable; eight cells per warp.
// Each lane keeps the reduced coefficients of all four stencils in
// registers until the weights are known, then writes its variable at the
// quadrature points of the cell's three faces.

template <int K, int M, int NQ, int VARIANT>
__global__ void __launch_bounds__(128) teno_kernel(const TenoArgs a, const double* __restrict__ U,
                                                   double* __restrict__ fv, uint8_t* __restrict__ masks) {
    constexpr int KR = K - 1, MR = M - 1, NF = 3, S = 4;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int cell = gt >> 2, v = gt & 3;
    if (cell >= a.n_cells) return;
    const int tile = cell >> 3, lane = cell & 7;
    const double uc = U[(size_t)cell * NC + v];
    const unsigned sm = a.smask[cell];

    double coef[S][KR];
    double w[S];
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
            const double b = __ldg(arp + j * TILE) * (__ldg(U + (size_t)nbj * NC + v) - uc);
#pragma unroll
            for (int k = 0; k < KR; ++k) coef[s][k] = coef[s][k] + __ldg(Pp + (j * KR + k) * TILE) * b;
        }
        // smoothness indicator a^T (OI a), dof 0 omitted (its coefficient is exactly zero)
        double si = 0.0;
#pragma unroll
        for (int i = 0; i < KR; ++i) {
            double oa = 0.0;
#pragma unroll
            for (int l = 0; l < KR; ++l) oa = oa + a.oi[i * KR + l] * coef[s][l];
            si = si + coef[s][i] * oa;
        }
        w[s] = 1.0 / pow6(si + 1.0e-12);
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
        if (VARIANT == MGPU_TENO_CORRECTED) {
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

    // face states at the quadrature points
#pragma unroll
    for (int fl = 0; fl < NF; ++fl) {
        const uint32_t slot = __ldg(a.cface + ((size_t)tile * NF + fl) * TILE + lane);
        const size_t f = slot >> 1;
        const unsigned side = slot & 1u;
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
                for (int k = 0; k < KR; ++k) out = out + (w[s] * coef[s][k]) * phi[k];
            }
            fv[((f * NQ + q) * 2 + side) * NC + v] = out;
        }
    }
}

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
// Face flux (flux_functor.h:124-178 and src/boundary/boundary_*.cpp)
// ---------------------------------------------------------------------------

__device__ __forceinline__ bool admissible(const GasParams& g, const double* W) {
    const double rho = W[0];
    if (!(rho > 0.0)) return false;
    const double u0 = W[1] / rho, u1 = W[2] / rho;
    const double e = W[3] / rho - 0.5 * (u0 * u0 + u1 * u1);
    return (g.gamma - 1.0) * rho * e > 0.0;
}

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
            riemann<RS>(Ft, n, cl[0], pl, pl[2], g.gamma, pl[4], cr[0], pr, pr[2], g.gamma, pr[4]);
        }
#pragma unroll
        for (int i = 0; i < 4; i++) F[i] += a.qw[q] * Ft[i];
    }
    const double area = a.area[f];
    double2* Gf = reinterpret_cast<double2*>(a.G + (size_t)f * 4);
    Gf[0] = make_double2(area * (F[0] * 0.5), area * (F[1] * 0.5));
    Gf[1] = make_double2(area * (F[2] * 0.5), area * (F[3] * 0.5));
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

template <int K, int M, int NQ>
cudaError_t teno_dispatch_variant(const TenoArgs& a, int variant, const double* U, double* fv, uint8_t* masks,
                                  cudaStream_t s) {
    const long long threads = (long long)a.n_cells * 4;
    const unsigned blocks = (unsigned)((threads + 127) / 128);
    if (blocks == 0) return cudaSuccess;
    if (variant == MGPU_TENO_CORRECTED)
        teno_kernel<K, M, NQ, MGPU_TENO_CORRECTED><<<blocks, 128, 0, s>>>(a, U, fv, masks);
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

cudaError_t launch_first_order(int n_faces, const int2* lr, const double* U, double* fv, cudaStream_t s) {
    const long long threads = (long long)n_faces * 4;
    const unsigned blocks = (unsigned)((threads + 255) / 256);
    if (blocks == 0) return cudaSuccess;
    first_order_kernel<<<blocks, 256, 0, s>>>(n_faces, lr, U, fv);
    return cudaGetLastError();
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
