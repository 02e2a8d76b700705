// selector_params.h -- sizes and packing of the learned stencil selector,
// shared by host and device code.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#define MGPU_HD
#else
#define MGPU_HD __host__ __device__
#endif

namespace mgpu {
namespace sel {

constexpr int NV = 4;          // conserved variables
constexpr int PER_VAR = 24;    // inputs per variable
constexpr int IN = NV * PER_VAR;  // 96
constexpr int HID = 64;
constexpr int NCLS = 8;
constexpr int OUT = NV * NCLS;  // 32
constexpr int MR = 19;         // central stencil neighbours at p = 3
constexpr int S = 4;           // stencils per triangle

// packed parameters: W1 [IN][HID] | b1 [HID] | W2 [HID][HID] | b2 | W3 [HID][OUT] | b3
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + IN * HID;
constexpr int OFF_W2 = OFF_B1 + HID;
constexpr int OFF_B2 = OFF_W2 + HID * HID;
constexpr int OFF_W3 = OFF_B2 + HID;
constexpr int OFF_B3 = OFF_W3 + HID * OUT;
constexpr int N_PARAMS = OFF_B3 + OUT;  // 12448

// TENO mask (bit 0 central, bits 1..3 directional passes) <-> class
MGPU_HD inline int class_of_mask(unsigned mask) { return (mask & 1u) ? 0 : (int)((mask >> 1) & 7u); }
MGPU_HD inline unsigned mask_of_class(int c) { return c == 0 ? 1u : ((unsigned)c << 1); }

}  // namespace sel
}  // namespace mgpu
