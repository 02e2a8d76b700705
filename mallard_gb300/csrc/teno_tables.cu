// teno_tables.cu -- the TENO least-squares tables built on the GPU.
//
// The stencils come from the search (face_reconstruction.cpp:217-475;
// stencil_search.cu on the GPU, host_teno.cpp on the host); this kernel
// then computes what compute_reconstruction_matrices computes for every
// stencil (face_reconstruction.cpp:477-741, common_math.h:355-493): the basis
// moments of each stencil cell in the target cell's reference frame, the
// mean subtraction, the Householder QR of the reduced (M-1) x (K-1) system
// and the two triangular solves of the pseudo-inverse.  It writes the
// result straight into the reconstruction kernels' tiled layout.
//
// The tables must equal the host build's (and so the reference's) bit for
// bit: this file is compiled with -fmad=false, and every element is
// computed by one lane with the same expression and summation order as the
// host code (host_teno.cpp).  What is parallel is the independent work:
// one warp per stencil; a lane per stencil cell for the moments, a lane per
// (row, column) element for each Householder reflection, a lane per
// right-hand side for the triangular solves.  The full-rank branch of the
// reference (a first moment column that is not zero) is not built here; a
// stencil that would take it sets the error word and the host fails the
// build.
//
// Legendre basis only: the monomial basis evaluates std::pow, whose CUDA
// and C library results can differ in the last bit; the host builds those.

#include <cstdint>

#include "device.h"

namespace mgpu {
namespace {

constexpr int LSQ_MAXM = 20, LSQ_MAXK = 10, LSQ_WARPS = 4;

// basis.h: Legendre polynomials on [0, 1]^2 coordinates (the same
// expressions as the host's basis_1d)
__device__ __forceinline__ double legendre(int p, double x) {
    switch (p) {
        case 0: return 1.0 * (1.0);
        case 1: return 1.0 * (1.0 * x);
        case 2: return 0.5 * (3.0 * x * x - 1.0);
        case 3: return 0.5 * (5.0 * x * x * x - 3.0 * x);
    }
    return 0.125 * (35.0 * x * x * x * x - 30.0 * x * x + 3.0);
}

__device__ __forceinline__ void mv2(const double* A, const double* x, double* y) {
    const double t0 = A[0] * x[0] + A[1] * x[1];
    const double t1 = A[2] * x[0] + A[3] * x[1];
    y[0] = t0;
    y[1] = t1;
}

__device__ __forceinline__ void jac(const double* a, const double* b, const double* c, double* J) {
    J[0] = b[0] - a[0];
    J[1] = c[0] - a[0];
    J[2] = b[1] - a[1];
    J[3] = c[1] - a[1];
}

__device__ __forceinline__ double tarea(const double* a, const double* b, const double* c) {
    return 0.5 * fabs(a[0] * (b[1] - c[1]) + b[0] * (c[1] - a[1]) + c[0] * (a[1] - b[1]));
}

struct WarpScratch {
    double A[LSQ_MAXM * LSQ_MAXK];              // moments [M][K]
    double R[(LSQ_MAXM - 1) * (LSQ_MAXK - 1)];  // reduced system -> R
    double T[(LSQ_MAXM - 1) * (LSQ_MAXK - 1)];  // next R; later Y
    double X[(LSQ_MAXK - 1) * (LSQ_MAXM - 1)];  // solution [K-1][M-1]
    double v[LSQ_MAXM], at[LSQ_MAXM];
};

__global__ void __launch_bounds__(LSQ_WARPS * 32) teno_lsq_kernel(const LsqBuildArgs a) {
    __shared__ WarpScratch scratch[LSQ_WARPS];
    const int lane = threadIdx.x & 31;
    WarpScratch& w = scratch[threadIdx.x >> 5];
    const long long gw = (long long)blockIdx.x * LSQ_WARPS + (threadIdx.x >> 5);
    if (gw >= (long long)a.n_cells * 4) return;
    const int c = (int)(gw >> 2), s = (int)(gw & 3);
    const uint32_t o = a.cell_old[c];
    const size_t si = (size_t)o * 4 + s;
    const uint32_t so = a.off_st[si];
    const int Ms = (int)(a.off_st[si + 1] - so);
    if (Ms == 0) return;
    const int M = a.M, K = a.K;
    if (Ms != M) {
        if (lane == 0) atomicOr(a.err, 1u);
        return;
    }
    // --- moments: lane j <-> stencil cell j (stencil_moments)
    const double2* N = a.nodes;
    const uint3 tn = a.tri[o];
    const double w0[2] = {N[tn.x].x, N[tn.x].y};
    if (lane < M) {
        const int j = lane;
        double J[4], Ji[4];
        {
            const double w1[2] = {N[tn.y].x, N[tn.y].y}, w2[2] = {N[tn.z].x, N[tn.z].y};
            jac(w0, w1, w2, J);
            const double det = J[0] * J[3] - J[1] * J[2];
            if (det == 0.0) atomicOr(a.err, 4u);  // "Matrix is singular." on the host
            const double r = 1.0 / det;
            Ji[0] = J[3] * r;
            Ji[1] = -J[1] * r;
            Ji[2] = -J[2] * r;
            Ji[3] = J[0] * r;
        }
        const uint3 nn = a.tri[a.st[so + j]];
        double v[3][2], vt[3][2];
        v[0][0] = N[nn.x].x; v[0][1] = N[nn.x].y;
        v[1][0] = N[nn.y].x; v[1][1] = N[nn.y].y;
        v[2][0] = N[nn.z].x; v[2][1] = N[nn.z].y;
        double Jn[4];
        jac(v[0], v[1], v[2], Jn);
        for (int k = 0; k < 3; ++k) {
            vt[k][0] = v[k][0] - w0[0];
            vt[k][1] = v[k][1] - w0[1];
            mv2(Ji, vt[k], vt[k]);
        }
        const double atj = tarea(vt[0], vt[1], vt[2]);
        w.at[j] = atj;
        double qp[2 * LSQ_MAXQ];
        for (int q = 0; q < a.nq; ++q) {
            double x[2] = {a.qp[2 * q], a.qp[2 * q + 1]};
            mv2(Jn, x, x);
            x[0] += v[0][0];
            x[1] += v[0][1];
            x[0] -= w0[0];
            x[1] -= w0[1];
            mv2(Ji, x, x);
            qp[2 * q] = x[0];
            qp[2 * q + 1] = x[1];
        }
        for (int k = 0; k < K; ++k) {
            double acc = 0.0;
            for (int q = 0; q < a.nq; ++q)
                acc += a.qw[q] * (legendre(a.pidx[2 * k], qp[2 * q]) * legendre(a.pidx[2 * k + 1], qp[2 * q + 1]));
            acc *= atj;
            // mean subtraction (stencil_pinv)
            w.A[j * K + k] = acc - atj * a.ipt[k];
        }
    }
    __syncwarp();
    // the reduced system requires a zero first moment column (:621-627)
    const bool nz = lane < M && w.A[lane * K] > 1.0e-12;
    if (__any_sync(0xffffffffu, nz)) {
        if (lane == 0) atomicOr(a.err, 2u);
        return;
    }
    const int m = M - 1, n = K - 1;
    for (int e = lane; e < m * n; e += 32) w.R[e] = w.A[(e / n + 1) * K + (e % n + 1)];
    __syncwarp();
    // --- Householder QR (householder_upper): column jc's reflector
    for (int jc = 0; jc < n; jc++) {
        double nx = 0.0;
        for (int i = jc; i < m; i++) nx += w.R[i * n + jc] * w.R[i * n + jc];
        nx = sqrt(nx);
        if (nx < 1.0e-15) continue;
        const double sgn = (w.R[jc * n + jc] >= 0.0) ? 1.0 : -1.0;
        const double alpha = -sgn * nx;
        double nu = 0.0, mine = 0.0;
        for (int k = 0; k < m - jc; k++) {
            double vk = w.R[(jc + k) * n + jc];
            if (k == 0) vk -= alpha;
            nu += vk * vk;
            if (k == lane) mine = vk;
        }
        nu = sqrt(nu);
        __syncwarp();
        if (lane < m - jc) w.v[lane] = mine / nu;
        __syncwarp();
        const int rows = m - jc, cols = n - jc;
        for (int e = lane; e < rows * cols; e += 32) {
            const int i = jc + e / cols, cc = jc + e % cols;
            double acc = 0.0;
            for (int k = jc; k < m; k++) {
                const double q = ((i == k) ? 1.0 : 0.0) - 2.0 * w.v[i - jc] * w.v[k - jc];
                acc += q * w.R[k * n + cc];
            }
            w.T[i * n + cc] = acc;
        }
        __syncwarp();
        for (int e = lane; e < rows * cols; e += 32) {
            const int i = jc + e / cols, cc = jc + e % cols;
            w.R[i * n + cc] = w.T[i * n + cc];
        }
        __syncwarp();
    }
    // --- R^T Y = B^T (solve_rt), then R X = Y (solve_r): lane <-> column
    // of the right-hand side; B is the reduced system, kept in A
    double* Y = w.T;
    if (lane < m) {
        const int jj = lane;
        for (int i = 0; i < n; i++) {
            double acc = 0.0;
            for (int k = 0; k < i; k++) acc += w.R[k * n + i] * Y[k * m + jj];
            Y[i * m + jj] = (w.A[(jj + 1) * K + (i + 1)] - acc) / w.R[i * n + i];
        }
        for (int i = n - 1; i >= 0; i--) {
            double acc = 0.0;
            for (int k = i + 1; k < n; k++) acc += w.R[i * n + k] * w.X[k * m + jj];
            w.X[i * m + jj] = (Y[i * m + jj] - acc) / w.R[i * n + i];
        }
    }
    __syncwarp();
    // --- tiled output (the layout of host_ctx.cpp's table pack)
    const size_t tile = (size_t)c / TILE, tl = (size_t)c % TILE;
    const int KR = n, MR = m;
    if (a.P4) {
        const size_t GP = ((size_t)MR * KR + 3) / 4;
        for (int e = lane; e < MR * KR; e += 32) {
            const int jm = e / KR, k = e % KR;  // flat entry jm * (K-1) + k
            const double x = w.X[k * m + jm] * w.at[jm + 1];
            a.P4[(((tile * 4 + s) * GP + e / 4) * TILE + tl) * 4 + e % 4] = __double2float_rn(x);
        }
    } else {
        for (int e = lane; e < MR * KR; e += 32) {
            const int jm = e / KR, k = e % KR;
            a.P[(((tile * 4 + s) * MR + jm) * KR + k) * TILE + tl] = w.X[k * m + jm];
        }
        for (int jm = lane; jm < MR; jm += 32) a.ar[((tile * 4 + s) * MR + jm) * TILE + tl] = w.at[jm + 1];
    }
}

}  // namespace

cudaError_t launch_teno_lsq(const LsqBuildArgs& a, cudaStream_t s) {
    if (a.M > LSQ_MAXM || a.K > LSQ_MAXK || a.nq > LSQ_MAXQ || a.M < 2 || a.K < 2) return cudaErrorInvalidValue;
    const long long warps = (long long)a.n_cells * 4;
    const long long blocks = (warps + LSQ_WARPS - 1) / LSQ_WARPS;
    if (blocks == 0) return cudaSuccess;
    teno_lsq_kernel<<<(unsigned)blocks, LSQ_WARPS * 32, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mgpu
