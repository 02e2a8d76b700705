// selector.cuh -- the learned TENO stencil selector: features and constants
// shared by the harvest, training and inference kernels.
//
// The selector is a 96-64-64-32 MLP evaluated once per cell.  Its input is,
// for each conserved variable v (24 entries per variable):
//   [0,19)  differences U_j - U_c over the central stencil's 19 neighbours
//           (stencil order), divided by the variable's range over that
//           stencil (target included);
//   19      log10 of that range, scaled: (log10 r + 6) / 6 clamped to
//           [-1, 1]; -1 when the range is flat (at most FLAT_RANGE);
//   20..22  range over directional stencil d (target included) divided by
//           the central range, clipped to 4 and scaled by 1/4 (for a flat
//           central range: 1 if the directional one is not flat, else 0); -1
//           when the stencil does not exist (boundary face);
//   23      zero.
// Its output is 4 heads (one per variable) of 8 logits over TENO's
// decisions for that variable: class 0 = central stencil only, class
// m = 1..7 = directional stencils whose bit is set in m pass the cut-off
// (the kernels' mask >> 1).  The network has no counterpart in the
// reference; the decisions it learns are those of
// face_reconstruction.cpp:939-981 as computed by the corrected TENO form.
#pragma once

#include <cstdint>

#include "device.h"
#include "selector_params.h"

namespace mgpu {
namespace sel {

// Ranges up to this are flat: differences, log-range and directional ratios
// as for an exactly uniform stencil.  TENO itself treats such stencils as
// smooth (its smoothness indicators, ~ range^2, fall below its epsilon
// 1e-12), and the FP32 form's round-off leaves ranges of 1e-7 .. 2e-6 in
// uniform flow, which the network must read as uniform.
constexpr float FLAT_RANGE = 1.0e-5f;

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
__device__ __forceinline__ float gelu(float x) {
    const float c = 0.7978845608028654f;
    return 0.5f * x * (1.0f + tanhf(c * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float c = 0.7978845608028654f;
    const float t = tanhf(c * (x + 0.044715f * x * x * x));
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * c * (1.0f + 3.0f * 0.044715f * x * x);
}

// Neighbour j of stencil s of a cell, in either tiled layout:
// nb [tiles][4][M-1][8] (FP64 forms) or nb4 [tiles][4][ceil((M-1)/4)][8][4] (FP32 form).
template <bool NB4>
__device__ __forceinline__ uint32_t stencil_cell(const TenoArgs& a, int tile, int lane, int s, int j) {
    if (NB4) {
        constexpr int GJ = (MR + 3) / 4;
        return __ldg(a.nb4 + ((((size_t)tile * S + s) * GJ + j / 4) * TILE + lane) * 4 + (j & 3));
    }
    return __ldg(a.nb + (((size_t)tile * S + s) * MR + j) * TILE + lane);
}

// The 19 stencil values of variable v minus uc, for stencil s of a cell.
// NB4: 16-byte index loads from the FP32 form's grouped layout; nbs (not
// null): the same layout for tiles tile0.. staged in shared memory.
template <bool NB4, class T, class ToF>
__device__ __forceinline__ void stencil_diffs(const TenoArgs& a, const T* __restrict__ U, int tile, int lane, int s,
                                              int v, float uc, ToF to_f, float* d, const uint4* nbs = nullptr,
                                              int tile0 = 0) {
    if (NB4) {
        constexpr int GJ = (MR + 3) / 4;
        const uint4* p = nbs ? nbs + (((size_t)(tile - tile0) * S + s) * GJ) * TILE + lane
                             : reinterpret_cast<const uint4*>(a.nb4) + (((size_t)tile * S + s) * GJ) * TILE + lane;
        uint32_t id[GJ * 4];
#pragma unroll
        for (int g = 0; g < GJ; ++g) {
            const uint4 q = nbs ? p[g * TILE] : __ldg(p + g * TILE);
            id[4 * g] = q.x;
            id[4 * g + 1] = q.y;
            id[4 * g + 2] = q.z;
            id[4 * g + 3] = q.w;
        }
#pragma unroll
        for (int j = 0; j < MR; ++j) d[j] = to_f(__ldg(U + (size_t)id[j] * 4 + v)) - uc;
    } else {
#pragma unroll
        for (int j = 0; j < MR; ++j) d[j] = to_f(__ldg(U + (size_t)stencil_cell<false>(a, tile, lane, s, j) * 4 + v)) - uc;
    }
}

// Features of variable v of one cell, from the state U (FP64, or the FP32
// form's FP32 copy; to_f gives the FP32 value of an element, rounded to
// nearest).  Writes PER_VAR floats.
template <bool NB4, class T, class ToF>
__device__ __forceinline__ void features(const TenoArgs& a, const T* __restrict__ U, int cell, int v, unsigned smask,
                                         ToF to_f, float* x, const uint4* nbs = nullptr, int tile0 = 0) {
    const int tile = cell >> 3, lane = cell & 7;
    const float uc = to_f(__ldg(U + (size_t)cell * 4 + v));
    stencil_diffs<NB4>(a, U, tile, lane, 0, v, uc, to_f, x, nbs, tile0);
    float lo = 0.0f, hi = 0.0f;
#pragma unroll
    for (int j = 0; j < MR; ++j) {
        lo = fminf(lo, x[j]);
        hi = fmaxf(hi, x[j]);
    }
    // flat ranges count as zero
    const float r0 = hi - lo > FLAT_RANGE ? hi - lo : 0.0f;
    const float inv = r0 > 0.0f ? 1.0f / r0 : 0.0f;
#pragma unroll
    for (int j = 0; j < MR; ++j) x[j] *= inv;
    x[MR] = r0 > 0.0f ? fminf(1.0f, fmaxf(-1.0f, (log10f(r0) + 6.0f) * (1.0f / 6.0f))) : -1.0f;
#pragma unroll
    for (int s = 1; s < S; ++s) {
        float f = -1.0f;
        if ((smask >> s) & 1u) {
            float d[MR];
            stencil_diffs<NB4>(a, U, tile, lane, s, v, uc, to_f, d, nbs, tile0);
            float l = 0.0f, h = 0.0f;
#pragma unroll
            for (int j = 0; j < MR; ++j) {
                l = fminf(l, d[j]);
                h = fmaxf(h, d[j]);
            }
            const float rs = h - l;
            f = r0 > 0.0f ? fminf(rs * inv, 4.0f) * 0.25f : (rs > FLAT_RANGE ? 1.0f : 0.0f);
        }
        x[MR + s] = f;
    }
    x[PER_VAR - 1] = 0.0f;
}

}  // namespace sel
}  // namespace mgpu
