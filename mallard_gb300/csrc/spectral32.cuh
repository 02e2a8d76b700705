// spectral32.cuh -- the FP32 form's spectral radius of a cell
// (SpectralRadiusFunctor, solver.cpp:634-706, in FP32 arithmetic), computed
// from the FP32 copy of the conserved state that the stage update writes.
//
// The FP32 form carries no FP64 primitives through the step: its flux,
// viscous terms and selector all read the FP32 state copy, and the time
// step is computed from it here.  Every operation is an explicit
// round-to-nearest intrinsic, so the value does not depend on the including
// translation unit's -fmad setting: the time-step kernel (kernels_fast.cu)
// and mgpu_calc_dt_noalloc (noalloc.cu) agree bit for bit.
#pragma once

#include "device.h"
#include "fp_convert.cuh"

namespace mgpu {
namespace {

// Velocity and sound speed of one FP32 state row: FP32 recovery, or FP64
// recovery from the same FP32 values where the internal energy is a small
// remainder of the total energy (near vacuum pressure), as the FP32 flux
// does for its face states.
__device__ __forceinline__ float3 velocity_sound32(const SpecArgs& a, const float4 x) {
    const float ir = __frcp_rn(x.x);
    const float u = __fmul_rn(x.y, ir), v = __fmul_rn(x.z, ir);
    const float E = __fmul_rn(x.w, ir);
    const float e = __fsub_rn(E, __fmul_rn(0.5f, __fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v))));
    if (e > __fmul_rn(1.0e-3f, E)) {
        const float p =
            fmaxf(a.p_min_f, fminf(a.p_max_f, __fmul_rn(__fmul_rn(__fsub_rn(a.gamma_f, 1.0f), x.x), e)));
        return make_float3(u, v, __fsqrt_rn(__fmul_rn(__fmul_rn(a.gamma_f, p), ir)));
    }
    const double rho = f64_of(x.x), ird = __drcp_rn(rho);
    const double ud = __dmul_rn(f64_of(x.y), ird), vd = __dmul_rn(f64_of(x.z), ird);
    const double ed = __dsub_rn(__dmul_rn(f64_of(x.w), ird),
                                __dmul_rn(0.5, __dadd_rn(__dmul_rn(ud, ud), __dmul_rn(vd, vd))));
    const double p = fmax(a.p_min, fmin(a.p_max, __dmul_rn(__dmul_rn(__dsub_rn(a.gamma, 1.0), rho), ed)));
    return make_float3(u, v, f32_rn(__dsqrt_rn(__dmul_rn(__dmul_rn(a.gamma, p), ird))));
}

// The radius of cell c: per face the mean of the two cells' |u . n| and
// sound speeds over the face distance, the reference's 1.37 and 3 / n_faces
// factors.  IX maps a local cell index to its state row.
template <class IX>
__device__ __forceinline__ float spectral_cell32(const SpecArgs& a, int c, const IX& ix) {
    const int4 cf = a.cfaces[c];
    const int ent[4] = {cf.x, cf.y, cf.z, cf.w};
    float conv = 0.0f, acou = 0.0f;
    int nf = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (ent[k] < 0) break;
        ++nf;
        const int f = ent[k];
        const int2 lr = a.lr[f];
        const int L = lr.x, R = lr.y < 0 ? lr.x : lr.y;
        const float4 gf = a.geo32[f];
        const float nx = gf.x, ny = gf.y, idx = gf.z;
        const float3 wl = velocity_sound32(a, a.u32[ix.u(L)]);
        const float3 wr = velocity_sound32(a, a.u32[ix.u(R)]);
        const float af = __fmul_rn(0.5f, __fadd_rn(wl.z, wr.z));
        const float uf0 = __fmul_rn(0.5f, __fadd_rn(wl.x, wr.x)), uf1 = __fmul_rn(0.5f, __fadd_rn(wl.y, wr.y));
        const float un = fabsf(__fadd_rn(__fmul_rn(uf0, nx), __fmul_rn(uf1, ny)));
        conv = __fadd_rn(conv, __fmul_rn(un, idx));
        const float t = __fmul_rn(af, idx);
        acou = __fadd_rn(acou, __fmul_rn(t, t));
    }
    const float geom = nf == 3 ? 1.0f : 0.75f;  // 3 / n_faces, exactly
    conv = __fmul_rn(conv, __fmul_rn(1.37f, geom));
    acou = __fmul_rn(1.37f, __fsqrt_rn(__fmul_rn(geom, acou)));
    return __fadd_rn(conv, acou);
}

}  // namespace
}  // namespace mgpu
