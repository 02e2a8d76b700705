// teno_flux_exact.cu -- TENO and face-flux kernels with the reference's
// rounding (compiled with -fmad=false; see teno_flux.cuh).
#define MGPU_NS exact
#define MGPU_FAST 0
#include "teno_flux.cuh"
