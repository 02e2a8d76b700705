// device.h -- parameter blocks shared by the host context and the kernels.
//
// Device layout (cells and faces in the library's internal order):
//   U, Utmp, W        double [n_cells][4]          conserved state, AoS (32 B/cell)
//   prim              double [n_cells][5]
//   TENO tables, tiled by 8 cells so that one warp (8 cells x 4 variables)
//   reads 64 contiguous bytes per table entry:
//     nb    uint32 [tiles][4 stencils][M-1][8]     neighbour cells (target dropped)
//     ar    double [tiles][4][M-1][8]              transformed areas
//     P     double [tiles][4][M-1][K-1][8]         pseudo-inverse, dof 0 and column 0
//                                                  dropped (exact zeros in the reference)
//     phi   double [tiles][3 faces][n_q][K-1][8]   basis shape value at each face point
//     cface uint32 [tiles][3][8]                   face slot * 2 + side
//   fv    double [n_faces][n_q][2][4]             reconstructed face states
//   G     double [n_flux_faces][4]                face-area x numerical flux
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/mallard_gb300.h"

namespace mgpu {

constexpr int TILE = 8;
constexpr int MAX_BC = 16;
constexpr int KR_MAX = 9;  // K-1 for p = 3

struct GasParams {
    double gamma, R, cv, p_min, p_max;
    double icv;  // 1 / cv (fast forms)
    float gamma_f, R_f, cv_f, p_min_f, p_max_f;  // the same rounded to FP32 on the host (FP32 form)
    float icv_f, gm1_f;                          // 1 / cv and gamma - 1, rounded once (FP32 form)
};

struct BcEntry {
    int type;
    double data[6];
};

struct BcTable {
    int n;
    BcEntry bc[MAX_BC];
};

struct TenoArgs {
    int n_cells;
    const uint32_t* nb;
    const double* ar;
    const double* P;
    const double* phi;
    const uint32_t* cface;
    const uint8_t* smask;
    // FP32-bulk form: the same tables in FP32, in groups of four entries so
    // that a lane reads 16 bytes (transformed areas folded into P)
    const uint32_t* nb4;  // [tiles][4][ceil((M-1)/4)][8][4]
    const float* P4;      // [tiles][4][ceil((M-1)(K-1)/4)][8][4], entry j*(K-1)+k
    // Face shapes of the FP32 form.  Mapped into its triangle's reference
    // frame, a face's points are the Gauss points of one of the reference
    // triangle's three edges, run in one of two directions: six shape sets,
    // shared by all cells, picked per face slot by a 3-bit code.
    const uint16_t* fcode;   // [tiles][8]: per cell, bits 3f..3f+2 = code of face slot f
    const float4* phi_tab4;  // [8 codes][ceil(n_q (K-1)/4)] float4, entry q*(K-1)+k
    double oi[KR_MAX * KR_MAX];   // oscillation indicator without dof 0, row-major (K-1)^2
    double oi2[KR_MAX * KR_MAX];  // same, upper triangle with doubled off-diagonals (fast form)
    float oi2f[KR_MAX * KR_MAX];  // oi2 in FP32 (FP32-bulk form)
    unsigned* err;                // status word: bit 2 when a bounded wait ran out (staged FP32 form)
    // robust TENO variant: per cell 1 if it has a boundary face
    const uint8_t* bcell;         // null unless the variant is MGPU_TENO_ROBUST
    // Viscous gradients from the reconstruction (MGPU_VISC_GRAD_RECON): the
    // kernel differentiates each cell's polynomials at its centroid and
    // writes the cell's (u, v, T) and their gradients.  Null vgrad / vq:
    // not asked.
    const double* ji;             // [n_cells][4] inverse Jacobian of the cell's reference frame (FP64 forms)
    const float4* ji4;            // the same in FP32 (FP32 form)
    double dphi[2 * KR_MAX];      // [k][2] basis gradient (d/dxi_0, d/dxi_1) at the reference centroid, k >= 1
    float dphif[2 * KR_MAX];
    double cv;                    // specific heat at constant volume (T = e / cv)
    float inv_cv;
    double* vgrad;                // FP64 forms: [n_cells][6] du/dx, du/dy, dv/dx, dv/dy, dT/dx, dT/dy
    float4* vq;                   // FP32 form: the Visc32Args records (u, v, T, 0), (du, dv), (dT)
    float4* vga;
    float2* vgb;
};

struct FluxArgs {
    int n_faces;            // faces that carry a flux
    const int2* lr;         // internal cell ids; y = -1 on boundary faces
    const double2* nrm;     // unit normal (reference unit<2> arithmetic, precomputed)
    const float2* nrm32;    // the same rounded to FP32 once (FP32 form)
    const double* area;
    const int8_t* bc;       // -1 interior, else BcTable index
    const double* fv;
    double* G;
    const double* U;        // stage input, for the positivity fallback
    double qw[4];           // face quadrature weights
    float qw_f[4];          // the same rounded to FP32 (FP32 form)
    int guard;              // robust TENO variant: a NaN star pressure counts as zero (HLL, HLLC)
};

struct UpdateArgs {
    int n_cells;
    const int4* gat;        // per cell up to 4 (face*2 + negate) in the reference's summation order, -1 = none
    const double* G;
    const double* vol;
    const double* ivol;     // 1 / volume (fast forms)
    const double* dt;       // device scalar
    double* U;              // stage-1 base; final state after stage 3
    double* Ut;             // stage state
    double* W;              // running sum U + dt/6 k1 + dt/6 k2
    double* prim;
    double* snd;            // sound speed per cell, written with prim
    double* rhs;            // residual output (stage 0 only)
    float* u32;             // FP32 copy of the stage's output state (FP32 form), or null
    unsigned* flags;
};

// Viscous face flux (no counterpart in the reference): Green-Gauss
// gradients of (u, v, T) per cell, then per flux face the Navier-Stokes
// stress and heat flux subtracted from G.
struct ViscArgs {
    int n_cells, n_faces;   // cells, flux faces
    const int4* cfaces;     // faces of each cell, -1 = none
    const int2* lr;
    const double2* nrm;     // unit normals
    const double* area;
    const double* vol;
    const int8_t* bc;       // -1 interior, else BcTable index
    const double2* xc;      // cell centres
    const double2* xf;      // face midpoints
    double* grad;           // [n_cells][6]: du/dx, du/dy, dv/dx, dv/dy, dT/dx, dT/dy
    double* G;
    double mu_ref, T_ref, S, cp_over_pr;
    int grad_ready;         // 1: the reconstruction wrote grad (no Green-Gauss kernel)
};

// FP32 form of the viscous flux: (u, v, T) and their Green-Gauss gradients
// per cell from the FP32 stage state, then the face flux inside the FP32
// face-flux kernel.  Face geometry rounded to FP32 once, on upload.
struct Visc32Args {
    int n_cells;
    const int4* cfaces;     // faces of each cell, -1 = none
    const int2* lr;
    const int8_t* bc;       // -1 interior, else BcTable index
    const float4* fgeo;     // per flux face: unit normal (x, y), centre-line direction (x, y)
    const float2* fgeo2;    // per flux face: area, 1 / centre-line length
    const double* ivol;     // 1 / volume
    float4* q;              // per cell: u, v, T, 0
    float4* ga;             // per cell: du/dx, du/dy, dv/dx, dv/dy
    float2* gb;             // per cell: dT/dx, dT/dy
    float mu_ref, T_ref, S, cp_over_pr, inv_cv;
};

// GPU build of the TENO least-squares tables (teno_tables.cu): one warp per
// stencil of every cell, results in the tiled layout of TenoArgs.
constexpr int LSQ_MAXQ = 8;
struct LsqBuildArgs {
    int n_cells;              // cells, library numbering
    const uint32_t* cell_old; // library -> caller cell id
    const double2* nodes;     // node coordinates
    const uint3* tri;         // nodes of each cell (caller numbering)
    const uint32_t* off_st;   // [4 n_cells + 1] stencil offsets (reference layout, caller numbering)
    const uint32_t* st;       // stencil cells, target first (caller numbering)
    int M, K, nq;             // stencil size, dofs, cell quadrature points
    double qp[2 * LSQ_MAXQ], qw[LSQ_MAXQ];
    int pidx[2 * 10];
    double ipt[10];           // basis means of the target (face_reconstruction.cpp:598-602)
    double* P;                // FP64 forms: pseudo-inverse, [tiles][4][M-1][K-1][8]
    double* ar;               // FP64 forms: transformed areas, [tiles][4][M-1][8]
    float* P4;                // FP32 form (P null): pseudo-inverse x areas, grouped by four
    unsigned* err;            // 1 stencil size, 2 full-rank system, 4 singular Jacobian
};
cudaError_t launch_teno_lsq(const LsqBuildArgs& a, cudaStream_t s);

struct SpecArgs {
    int n_cells;
    const int4* cfaces;     // faces of the cell in the reference's order, -1 = none
    const int2* lr;
    const double2* nrm;
    const double* dxn;      // |s . n| with the reference's boundary rule, precomputed
    const double* idxn;     // 1 / dxn (fast forms)
    const double* U;
    const double* prim;
    const double* snd;      // sound speed per cell
    double* rho_cell;
    unsigned long long* rmax_bits;
    double gamma;
    // FP32 form: the radius comes from the FP32 state rows (spectral32.cuh)
    const float4* u32;      // null in the FP64 forms
    const float4* geo32;    // FP32 form: per face the unit normal and 1 / dxn rounded once, 0
    double p_min, p_max;
    float gamma_f, p_min_f, p_max_f;
};

// Launchers.  All return cudaGetLastError() of the launch.
// TENO and face flux exist twice: exact:: keeps the reference's rounding
// (teno_flux_exact.cu), fast:: contracts to FMA (teno_flux_fast.cu).
#define MGPU_DECLARE_TENO_FLUX                                                                              \
    cudaError_t launch_teno(const TenoArgs& a, int K, int M, int nq, int variant, const double* U, double* fv, \
                            uint8_t* masks, cudaStream_t s);                                                  \
    cudaError_t launch_flux(const FluxArgs& a, const GasParams& g, const BcTable& bct, int rsolver, int nq,  \
                            bool positivity, cudaStream_t s);
namespace exact {
MGPU_DECLARE_TENO_FLUX
}
namespace fast {
MGPU_DECLARE_TENO_FLUX
}
#undef MGPU_DECLARE_TENO_FLUX
// FP32-bulk form (fp32_fast.cu): face states in FP32, flux written in FP64.
namespace f32 {
// shape: launch shape 0..3 (128-thread blocks with at most 128, 80 or 64
// registers, or 256-thread blocks with 64; p = 3 only, other orders use
// shape 0) or 4..6, the staged form that copies each tile's table blocks
// into shared memory with cp.async.bulk; chosen by the autotuner
constexpr int TENO32_SHAPES = MGPU_AUTOTUNE_SHAPES;
// the batched reconstruction also has shapes 7 and 8: one CTA of 4 or 8
// warps per mesh tile, its tables resident in shared memory for all cases
constexpr int TENO32_BATCH_SHAPES = 9;
// U: the FP32 copy of the stage state
cudaError_t launch_teno(const TenoArgs& a, int K, int M, int nq, const float* U, float* fv, uint8_t* masks,
                        int shape, cudaStream_t s);
// with the learned selector's predictions (p = 3 only)
cudaError_t launch_teno_selected(const TenoArgs& a, int K, int M, int nq, const float* U, const uint8_t* pred,
                                 float* fv, uint8_t* masks, int shape, cudaStream_t s);
// visc: the viscous flux's arguments (after launch_visc_grad), or null
cudaError_t launch_flux(const FluxArgs& a, const float* fv, const GasParams& g, const BcTable& bct, int rsolver,
                        int nq, const Visc32Args* visc, cudaStream_t s);
// per-cell (u, v, T) and gradients of the FP32 stage state U
cudaError_t launch_visc_grad(const Visc32Args& v, const BcTable& bct, const float* U, cudaStream_t s);
}  // namespace f32
// ---------------------------------------------------------------------------
// Batched form: many cases on a few meshes in one launch per kernel.
// The cases of group g share one mesh (its tables and geometry, in the
// per-group argument blocks below); their state and face rows are
// interleaved per 8-row tile: row(c) = ubase + ((c / 8) C + case) 8 + c % 8.
// A kernel's threads run over all groups in order; group g starts at the
// thread index in the *0 arrays.  The kernels are persistent: any grid
// size works, each thread strides over the whole range.  A case whose
// status flags are set (non-finite state, invalid dt) is frozen: every
// kernel skips it from the next step on.
// ---------------------------------------------------------------------------
constexpr int MAX_GROUPS = 8;
struct BatchLaunch {
    int n_groups;
    unsigned C[MAX_GROUPS];          // cases in the group
    unsigned case0[MAX_GROUPS];      // global index of its first case
    int n_cells[MAX_GROUPS], n_faces[MAX_GROUPS];  // cells, flux faces
    unsigned long long ubase[MAX_GROUPS], fbase[MAX_GROUPS];
    long long cell0[MAX_GROUPS + 1];  // thread ranges: (case, cell)
    long long teno0[MAX_GROUPS + 1];  //                (case, cell, variable)
    long long face0[MAX_GROUPS + 1];  //                (case, flux face)
    // per-group argument blocks in device memory (tables, geometry)
    const TenoArgs* teno;
    const FluxArgs* flux;
    const UpdateArgs* upd;
    const SpecArgs* spec;
    // state of all cases
    double *U, *Ut, *W, *prim, *snd, *G;
    float *U32, *Ut32;               // FP32 copies of U and Ut
    float* fv;
    double *dt, *t;                  // per case
    unsigned long long* rmax;        // per case
    unsigned* flags;                 // per case
};

namespace f32 {
cudaError_t launch_teno_batch(const BatchLaunch& b, const float* U, int shape, int blocks_per_sm, cudaStream_t s);
cudaError_t launch_flux_batch(const BatchLaunch& b, const GasParams& g, const BcTable& bct, int rsolver, int nq,
                              const double* U, cudaStream_t s);
}  // namespace f32
cudaError_t launch_update_batch(const BatchLaunch& b, const GasParams& g, int stage, cudaStream_t s);
cudaError_t launch_spectral_batch(const BatchLaunch& b, cudaStream_t s);
cudaError_t launch_dt_batch(const BatchLaunch& b, int n_cases, double cfl, cudaStream_t s);
// caller-order rows of one case <-> its interleaved internal rows
cudaError_t launch_batch_rows(int n, int width, const uint32_t* perm_old, const double* src, double* dst,
                              unsigned long long ubase, unsigned C, unsigned cs, bool to_batch, cudaStream_t s);
cudaError_t launch_batch_prims(int n, const GasParams& g, double* U, double* prim, double* snd, float* U32,
                               unsigned long long ubase, unsigned C, unsigned cs, cudaStream_t s);
// FP32 copy of n doubles (round to nearest)
cudaError_t launch_to_f32(size_t n, const double* src, float* dst, cudaStream_t s);

// kernels.cu
cudaError_t launch_first_order(int n_faces, const int2* lr, const double* U, double* fv, cudaStream_t s);
cudaError_t launch_update(const UpdateArgs& a, const GasParams& g, int stage, int scheme, bool fast, cudaStream_t s);
cudaError_t launch_spectral(const SpecArgs& a, bool fast, cudaStream_t s);
cudaError_t launch_sound(int n, double gamma, const double* U, const double* prim, double* snd, cudaStream_t s);
// viscous: gradients of the stage input U, then the face flux into G
cudaError_t launch_viscous(const ViscArgs& a, const GasParams& g, const BcTable& bct, const double* U, cudaStream_t s);
cudaError_t launch_dt(const unsigned long long* rmax_bits, double cfl, double* dt, double* t, unsigned* flags,
                      cudaStream_t s);
cudaError_t launch_set_scalar(double* dst, double value, cudaStream_t s);
// caller-order rows of a device-addressable host array <-> internal rows
// (pos: caller row -> internal row), in one pass; load also writes the FP32
// copy when dst32 is given
cudaError_t launch_load_rows(int n, int width, const uint32_t* pos, const double* host, double* dst, float* dst32,
                             cudaStream_t s);
cudaError_t launch_store_rows(int n, int width, const uint32_t* pos, const double* src, double* host, cudaStream_t s);
cudaError_t launch_permute_rows(int n, int width, const uint32_t* idx, const double* src, double* dst, bool scatter,
                                cudaStream_t s);
// dst[idx[c]] = src[c * stride] for c < n
cudaError_t launch_permute_column(int n, int stride, const uint32_t* idx, const double* src, double* dst,
                                  cudaStream_t s);
cudaError_t launch_riemann_batch(int rsolver, uint32_t n, const double* buf_in, double* flux, cudaStream_t s);
cudaError_t launch_primitives_batch(const GasParams& g, uint32_t n, const double* U, double* W, cudaStream_t s);
cudaError_t run_fp64_probe(int device, double* gflops);
// f32_rn of n doubles and f64_of of n floats (host arrays), on the device
cudaError_t run_convert_probe(int device, const double* in64, float* out32, const float* in32, double* out64, size_t n);

}  // namespace mgpu
