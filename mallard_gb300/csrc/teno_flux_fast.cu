// teno_flux_fast.cu -- TENO and face-flux kernels with FMA contraction and
// the reduced-instruction forms (compiled with -fmad=true; see teno_flux.cuh).
#define MGPU_NS fast
#define MGPU_FAST 1
#include "teno_flux.cuh"
