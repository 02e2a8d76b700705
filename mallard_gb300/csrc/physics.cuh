// physics.cuh -- device-side Euler physics and Riemann solvers shared by the
// kernels (restating src/physics/physics.h:842-867 and
// src/numerics/riemann_solver.h:205-519), templated on the arithmetic type.
//
// Every translation unit that includes it gets its own copy (internal
// linkage); the rounding of each copy is fixed by the unit's -fmad setting.
// With T = double the expressions are the reference's, operation for
// operation.  With T = float every literal is a T, so nothing is promoted to
// FP64 (the slow unit on GB300).
#pragma once

#include <cstdint>

#include "device.h"

namespace mgpu {
namespace {

constexpr int NC = 4;
constexpr int NPR = 5;

// ---------------------------------------------------------------------------
// Euler physics (src/physics/physics.h:842-867)
// ---------------------------------------------------------------------------

// A gas constant in the arithmetic type: the FP64 value, or its FP32
// rounding made once on the host (a device F2F conversion issues on the
// FP64 unit).
template <class T>
__device__ __forceinline__ T cst(double d, float f);
template <>
__device__ __forceinline__ double cst<double>(double d, float) { return d; }
template <>
__device__ __forceinline__ float cst<float>(double, float f) { return f; }

template <class T>
__device__ __forceinline__ void primitives(const GasParams& g, const T* U, T* W) {
    const T rho = U[0];
    const T u0 = U[1] / rho, u1 = U[2] / rho;
    const T E = U[3] / rho;
    const T e = E - T(0.5) * (u0 * u0 + u1 * u1);
    const T p = fmax(cst<T>(g.p_min, g.p_min_f), fmin(cst<T>(g.p_max, g.p_max_f), (cst<T>(g.gamma, g.gamma_f) - T(1.0)) * rho * e));
    W[0] = u0;
    W[1] = u1;
    W[2] = p;
    W[3] = e / cst<T>(g.cv, g.cv_f);
    W[4] = e + p / rho;
}

// Positivity test of the corrected TENO variant's fallback.
template <class T>
__device__ __forceinline__ bool admissible(const GasParams& g, const T* W) {
    const T rho = W[0];
    if (!(rho > T(0.0))) return false;
    const T u0 = W[1] / rho, u1 = W[2] / rho;
    const T e = W[3] / rho - T(0.5) * (u0 * u0 + u1 * u1);
    return (cst<T>(g.gamma, g.gamma_f) - T(1.0)) * rho * e > T(0.0);
}

// ---------------------------------------------------------------------------
// Riemann solvers (src/numerics/riemann_solver.h:205-519)
// ---------------------------------------------------------------------------

// star-region estimates; W = {rho, u_n, p, gamma}
template <class T>
__device__ __forceinline__ void pvrs(const T* L, const T* R, T& ps) {
    const T al = sqrt(L[3] * L[2] / L[0]);
    const T ar = sqrt(R[3] * R[2] / R[0]);
    const T rho_m = T(0.5) * (L[0] + R[0]);
    const T a_m = T(0.5) * (al + ar);
    ps = T(0.5) * (L[2] + R[2]) + T(0.5) * (L[1] - R[1]) * rho_m * a_m;
}

template <class T>
__device__ __noinline__ void trrs(const T* L, const T* R, T& ps) {
    const T al = sqrt(L[3] * L[2] / L[0]);
    const T ar = sqrt(R[3] * R[2] / R[0]);
    const T zl = (L[3] - T(1.0)) / (T(2.0) * L[3]);
    const T zr = (R[3] - T(1.0)) / (T(2.0) * R[3]);
    const T plr = pow((L[2] / R[2]), zl);
    const T us = (plr * L[1] / al + R[1] / ar + T(2.0) * (T(1.0) - plr) / (L[3] - T(1.0))) / (plr / al + T(1.0) / ar);
    ps = T(0.5) * (L[2] * pow((T(1.0) + (L[3] - T(1.0)) / (T(2.0) * al) * (L[1] - us)), (T(1.0) / zl)) +
                   R[2] * pow((T(1.0) + (R[3] - T(1.0)) / (T(2.0) * ar) * (us - R[1])), (T(1.0) / zr)));
}

template <class T>
__device__ __noinline__ void tsrs(const T* L, const T* R, T& ps) {
    const T gl = (L[3] - T(1.0)) / (L[3] + T(1.0));
    const T gr = (R[3] - T(1.0)) / (R[3] + T(1.0));
    const T Al = T(2.0) / (L[3] + T(1.0)) / L[0], Bl = gl * L[2];
    const T Ar = T(2.0) / (R[3] + T(1.0)) / R[0], Br = gr * R[2];
    const T p0 = fmax(T(0.0), ps);
    const T ql = sqrt(Al / (p0 + Bl));
    const T qr = sqrt(Ar / (p0 + Br));
    ps = (ql * L[2] + qr * R[2] - (R[1] - L[1])) / (ql + qr);
}

// ANRS (riemann_solver.h:308-329); only p_star is used by HLL/HLLC.
template <class T>
__device__ __forceinline__ T anrs(const T* L, const T* R) {
    const T pmax = fmax(L[2], R[2]), pmin = fmin(L[2], R[2]);
    const T qmax = pmax / pmin;
    T ps;
    pvrs(L, R, ps);
    if ((qmax < T(2.0)) && (pmin <= ps) && (ps <= pmax)) return ps;
    if (ps < pmin) trrs(L, R, ps);
    else tsrs(L, R, ps);
    return ps;
}

// guard: a star pressure that is not a number counts as zero (the robust
// TENO variant).  The two-rarefaction estimate raises a negative base to
// the power 2 gamma / (gamma - 1), not an exact integer in floating point,
// when a strong expansion meets near-vacuum pressure; zero gives the wave
// speeds of every star pressure below both sides' pressures, so no flux the
// reference computes as a number changes.
template <int RS, class T>
__device__ __forceinline__ void riemann(T* F, const T* n, T rl, const T* ul, T pl, T gl, T hl, T rr, const T* ur, T pr,
                                        T gr, T hr, bool guard = false) {
    const T unl = ul[0] * n[0] + ul[1] * n[1];
    const T unr = ur[0] * n[0] + ur[1] * n[1];
    const T qql = ul[0] * ul[0] + ul[1] * ul[1];
    const T qqr = ur[0] * ur[0] + ur[1] * ur[1];
    const T al = sqrt(gl * pl / rl);
    const T ar = sqrt(gr * pr / rr);
    const T El = (hl + T(0.5) * qql) * rl - pl;
    const T Er = (hr + T(0.5) * qqr) * rr - pr;
    const T Ul[4] = {rl, rl * ul[0], rl * ul[1], El};
    const T Ur[4] = {rr, rr * ur[0], rr * ur[1], Er};
    const T Fl[4] = {rl * unl, rl * ul[0] * unl + pl * n[0], rl * ul[1] * unl + pl * n[1], (El + pl) * unl};
    const T Fr[4] = {rr * unr, rr * ur[0] * unr + pr * n[0], rr * ur[1] * unr + pr * n[1], (Er + pr) * unr};
    if (RS == MGPU_RIEMANN_RUSANOV) {
        const T smax = fmax(fabs(unl) + al, fabs(unr) + ar);
#pragma unroll
        for (int i = 0; i < 4; i++) F[i] = T(0.5) * (Fl[i] + Fr[i] + smax * (Ul[i] - Ur[i]));
        return;
    }
    const T Wl[4] = {rl, unl, pl, gl}, Wr[4] = {rr, unr, pr, gr};
    T ps = anrs(Wl, Wr);
    if (guard && !(ps == ps)) ps = T(0.0);
    const T ql = (ps <= pl) ? T(1.0) : sqrt(T(1.0) + (gl + T(1.0)) / (T(2.0) * gl) * (ps / pl - T(1.0)));
    const T qr = (ps <= pr) ? T(1.0) : sqrt(T(1.0) + (gr + T(1.0)) / (T(2.0) * gr) * (ps / pr - T(1.0)));
    const T Sl = unl - al * ql;
    const T Sr = unr + ar * qr;
    if (RS == MGPU_RIEMANN_HLL) {
        if (T(0.0) <= Sl) {
#pragma unroll
            for (int i = 0; i < 4; i++) F[i] = Fl[i];
        } else if (Sr <= T(0.0)) {
#pragma unroll
            for (int i = 0; i < 4; i++) F[i] = Fr[i];
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) F[i] = (Sr * Fl[i] - Sl * Fr[i] + Sl * Sr * (Ur[i] - Ul[i])) / (Sr - Sl);
        }
        return;
    }
    const T Ss = (pr - pl + rl * unl * (Sl - unl) - rr * unr * (Sr - unr)) / (rl * (Sl - unl) - rr * (Sr - unr));
    if (T(0.0) <= Sl) {
#pragma unroll
        for (int i = 0; i < 4; i++) F[i] = Fl[i];
    } else if (Sr <= T(0.0)) {
#pragma unroll
        for (int i = 0; i < 4; i++) F[i] = Fr[i];
    } else {
        const T D[4] = {T(0.0), n[0], n[1], Ss};
        const T Plr = T(0.5) * (pl + pr + rl * (Sl - unl) * (Ss - unl) + rr * (Sr - unr) * (Ss - unr));
        if constexpr (sizeof(T) == 4) {
            // FP32 form: one correctly rounded reciprocal of the shared
            // denominator instead of four divisions
            if (Ss >= T(0.0)) {
                const T r = __frcp_rn(Sl - Ss);
#pragma unroll
                for (int i = 0; i < 4; i++) F[i] = (Ss * (Sl * Ul[i] - Fl[i]) + Sl * Plr * D[i]) * r;
            } else {
                const T r = __frcp_rn(Sr - Ss);
#pragma unroll
                for (int i = 0; i < 4; i++) F[i] = (Ss * (Sr * Ur[i] - Fr[i]) + Sr * Plr * D[i]) * r;
            }
        } else if (Ss >= T(0.0)) {
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

}  // namespace
}  // namespace mgpu
