// stencil_search.cu -- the TENO stencil search on the GPU
// (face_reconstruction.cpp:217-475: TENO::get_next_ring and
// compute_stencils_of_cell, with the Naive Cell Based central stencil and
// the Type 4 directional stencils).
//
// One thread per cell; each finds the cell's four stencils exactly as
// cell_stencils (host_teno.cpp) does, in the same order:
//  * rings are the layers of a breadth-first search (from the cell, or in
//    the directional fill-up from the whole stencil).  A neighbour of a
//    layer-k cell lies in layer k-1, k or k+1, so testing a candidate
//    against the two previous layers and the layer being built is the
//    reference's test against every ring so far;
//  * each ring is sorted by squared distance to the target with std::sort,
//    as the reference sorts it.  Among equal distances (everywhere on a
//    structured mesh) the order is whatever the library's sort leaves,
//    and the cells at a stencil's cut and the stencil's row order depend
//    on it.  This file calls the same std::sort template as the host
//    (libstdc++'s, constexpr since C++20 and so compiled for the device
//    under --expt-relaxed-constexpr), so ties fall as on the host;
//  * squared distances and the directional sector test are the host's
//    FP64 expressions, compiled with -fmad=false (no contraction), so every
//    comparison sees the same bits.
// A cell the kernel cannot finish -- a ring longer than RING_CAP, a
// singular face Jacobian, or a mesh too small for the stencil, where the
// reference throws -- is marked, and the host searches it again
// (host_teno.cpp), which gives the reference's error where there is one.
#include <algorithm>
#include <cstdint>
#include <string>
#include <utility>

#include <cuda_runtime.h>

#include "host.h"

namespace mgpu {
namespace {

constexpr int RING_CAP = 128;  // cells per ring held by a thread
// std::sort recurses (introsort) at most 2 lg(RING_CAP) + 1 = 15 levels
// deep; each level's frame is 80 bytes in the sm_103a build.  The stack
// limit is raised to the kernel's own frame plus this much for the search.
constexpr size_t SORT_STACK = 4096;

using DistPair = std::pair<uint32_t, double>;
struct ByDistance {
    __host__ __device__ bool operator()(const DistPair& a, const DistPair& b) const { return a.second < b.second; }
};

struct SearchArgs {
    const uint32_t *goff, *gnb;  // first-order neighbourhoods (the cell itself included), CSR
    const double *X, *nodes;     // cell centroids, node coordinates
    const uint32_t *ofc, *foc;   // faces of each cell, CSR
    const int32_t* cof;          // cells of each face (-1: boundary)
    const uint32_t *onf, *nof;   // nodes of each face, CSR
    uint32_t n_cells;
    int M;
    uint32_t* flat;   // [cell][4][M]
    uint8_t* sizes;   // [cell][4]
    uint8_t* status;  // [cell]: 0 found, 1 to be searched on the host
};

__host__ __device__ __forceinline__ bool contains(const uint32_t* l, int n, uint32_t x) {
    for (int i = 0; i < n; ++i)
        if (l[i] == x) return true;
    return false;
}

// The next layer: cells met from `front` (in its order, each cell's
// neighbours in CSR order) that are in none of `back`, `front` and the
// layer so far, then sorted by squared distance to `target`.  False when
// the layer would pass RING_CAP.
__host__ __device__ bool next_layer(const SearchArgs& a, uint32_t target, const uint32_t* back, int nb, const uint32_t* front,
                           int nf, uint32_t* out, int& no, DistPair* dist) {
    no = 0;
    for (int i = 0; i < nf; ++i) {
        const uint32_t c = front[i];
        for (uint32_t k = a.goff[c]; k < a.goff[c + 1]; ++k) {
            const uint32_t n = a.gnb[k];
            if (contains(back, nb, n) || contains(front, nf, n) || contains(out, no, n)) continue;
            if (no == RING_CAP) return false;
            out[no++] = n;
        }
    }
    for (int i = 0; i < no; ++i) {
        const uint32_t n = out[i];
        double d = 0.0;
        for (int j = 0; j < 2; j++) {
            const double t = a.X[2 * (size_t)n + j] - a.X[2 * (size_t)target + j];
            d += t * t;
        }
        dist[i] = DistPair(n, d);
    }
    std::sort(dist, dist + no, ByDistance{});
    for (int i = 0; i < no; ++i) out[i] = dist[i].first;
    return true;
}

// Per-thread scratch: three rings and the sort's (cell, distance) pairs.
struct Scratch {
    uint32_t ring[3][RING_CAP];
    DistPair dist[RING_CAP];
};

// The four stencils of cell c into a.flat, their sizes into sz; false when
// the host has to search the cell.
__host__ __device__ bool search_cell(const SearchArgs& a, uint32_t c, Scratch& w, int (&sz)[4]) {
    const int M = a.M;
    uint32_t* st = a.flat + (size_t)c * 4 * M;
    auto& ring = w.ring;
    int rn[3];
    const uint32_t f0 = a.ofc[c];
    if (a.ofc[c + 1] - f0 != 3) return false;
    // the faces' Jacobians in the cell's frame, inverted (mat2_inverse)
    double Ji[3][4];
    bool bnd[3];
    for (int s = 0; s < 3; ++s) {
        const uint32_t f = a.foc[f0 + s];
        const uint32_t n0 = a.nof[a.onf[f]], n1 = a.nof[a.onf[f] + 1];
        const double* x = a.X + 2 * (size_t)c;
        const double J[4] = {a.nodes[2 * (size_t)n0] - x[0], a.nodes[2 * (size_t)n1] - x[0],
                             a.nodes[2 * (size_t)n0 + 1] - x[1], a.nodes[2 * (size_t)n1 + 1] - x[1]};
        const double det = J[0] * J[3] - J[1] * J[2];
        if (det == 0.0) return false;
        const double r = 1.0 / det;
        Ji[s][0] = J[3] * r;
        Ji[s][1] = -J[1] * r;
        Ji[s][2] = -J[2] * r;
        Ji[s][3] = J[0] * r;
        bnd[s] = a.cof[2 * (size_t)f + 1] == -1;
    }
    for (int s = 0; s < 4; ++s) {
        st[s * M] = c;
        sz[s] = 1;
    }
    // central and directional stencils from the rings around the cell
    int ib = 0, ifr = 1, io = 2;
    rn[ib] = 0;
    ring[ifr][0] = c;
    rn[ifr] = 1;
    bool cen_full = M <= 1, dir_done = false;
    while (!cen_full || !dir_done) {
        if (!next_layer(a, c, ring[ib], rn[ib], ring[ifr], rn[ifr], ring[io], rn[io], w.dist)) return false;
        const uint32_t* L = ring[io];
        const int nL = rn[io];
        if (!cen_full) {
            for (int i = 0; i < nL && sz[0] < M; ++i) st[sz[0]++] = L[i];
            if (sz[0] == M) cen_full = true;
            else if (nL == 0) return false;  // the mesh is exhausted
        }
        if (!dir_done) {
            bool grew[3] = {false, false, false};
            for (int s = 0; s < 3; ++s) {
                uint32_t* d = st + (1 + s) * M;
                for (int i = 0; i < nL; ++i) {
                    if (sz[1 + s] == M) break;
                    const uint32_t n = L[i];
                    const double dx[2] = {a.X[2 * (size_t)n] - a.X[2 * (size_t)c],
                                          a.X[2 * (size_t)n + 1] - a.X[2 * (size_t)c + 1]};
                    const double t0 = Ji[s][0] * dx[0] + Ji[s][1] * dx[1];
                    const double t1 = Ji[s][2] * dx[0] + Ji[s][3] * dx[1];
                    if (!(t0 < 0.0) && !(t1 < 0.0)) {
                        d[sz[1 + s]++] = n;
                        grew[s] = true;
                    }
                }
            }
            dir_done = true;
            for (int s = 0; s < 3; ++s)
                if (!bnd[s] && sz[1 + s] < M && grew[s]) dir_done = false;
        }
        const int t = ib;
        ib = ifr;
        ifr = io;
        io = t;
    }
    // fill-up: layers around the whole directional stencil
    for (int s = 0; s < 3; ++s) {
        if (bnd[s]) {
            sz[1 + s] = 0;
            continue;
        }
        if (sz[1 + s] >= M) continue;
        if (sz[1 + s] > RING_CAP) return false;
        uint32_t* d = st + (1 + s) * M;
        ib = 0;
        ifr = 1;
        io = 2;
        rn[ib] = 0;
        for (int i = 0; i < sz[1 + s]; ++i) ring[ifr][i] = d[i];
        rn[ifr] = sz[1 + s];
        while (sz[1 + s] < M) {
            if (!next_layer(a, c, ring[ib], rn[ib], ring[ifr], rn[ifr], ring[io], rn[io], w.dist) || rn[io] == 0)
                return false;
            for (int i = 0; i < rn[io] && sz[1 + s] < M; ++i) d[sz[1 + s]++] = ring[io][i];
            const int t = ib;
            ib = ifr;
            ifr = io;
            io = t;
        }
    }
    for (int s = 0; s < 4; ++s)
        if (sz[s] < M && sz[s] != 0) return false;
    return true;
}

__global__ void __launch_bounds__(128) stencil_search_kernel(const SearchArgs a) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    Scratch w;
    int sz[4] = {0, 0, 0, 0};
    const bool ok = search_cell(a, c, w, sz);
    for (int s = 0; s < 4; ++s) a.sizes[(size_t)c * 4 + s] = ok ? (uint8_t)sz[s] : 0;
    a.status[c] = ok ? 0 : 1;
}

// Device buffers freed on every path.
struct Buffers {
    void* p[16] = {};
    int n = 0;
    template <class T>
    cudaError_t get(T** out, size_t count) {
        void* q = nullptr;
        const cudaError_t e = cudaMalloc(&q, count ? count * sizeof(T) : 1);
        if (e == cudaSuccess) p[n++] = q;
        *out = static_cast<T*>(q);
        return e;
    }
    template <class T>
    cudaError_t put(T** out, const T* src, size_t count) {
        cudaError_t e = get(out, count);
        if (e == cudaSuccess && count) e = cudaMemcpy(*out, src, count * sizeof(T), cudaMemcpyHostToDevice);
        return e;
    }
    ~Buffers() {
        for (int i = 0; i < n; ++i) cudaFree(p[i]);
    }
};

}  // namespace

bool gpu_stencil_search(const mgpu_mesh& m, const uint32_t* goff, const uint32_t* gnb, int M, uint32_t* flat,
                        uint8_t* sizes, uint8_t* status, std::string& msg) {
    const uint32_t N = m.n_cells;
    if (N == 0) return true;
    Buffers b;
    SearchArgs a{};
    a.n_cells = N;
    a.M = M;
    uint32_t *goff_d, *gnb_d, *ofc_d, *foc_d, *onf_d, *nof_d;
    double *X_d, *nodes_d;
    int32_t* cof_d;
    cudaError_t e = cudaSuccess;
    auto step = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    step(b.put(&goff_d, goff, (size_t)N + 1));
    if (e == cudaSuccess) step(b.put(&gnb_d, gnb, (size_t)goff[N]));
    step(b.put(&X_d, m.cell_coords, 2 * (size_t)N));
    step(b.put(&nodes_d, m.node_coords, 2 * (size_t)m.n_nodes));
    step(b.put(&ofc_d, m.offsets_faces_of_cell, (size_t)N + 1));
    if (e == cudaSuccess) step(b.put(&foc_d, m.faces_of_cell, (size_t)m.offsets_faces_of_cell[N]));
    step(b.put(&cof_d, m.cells_of_face, 2 * (size_t)m.n_faces));
    step(b.put(&onf_d, m.offsets_nodes_of_face, (size_t)m.n_faces + 1));
    if (e == cudaSuccess) step(b.put(&nof_d, m.nodes_of_face, (size_t)m.offsets_nodes_of_face[m.n_faces]));
    step(b.get(&a.flat, (size_t)N * 4 * M));
    step(b.get(&a.sizes, (size_t)N * 4));
    step(b.get(&a.status, (size_t)N));
    a.goff = goff_d;
    a.gnb = gnb_d;
    a.X = X_d;
    a.nodes = nodes_d;
    a.ofc = ofc_d;
    a.foc = foc_d;
    a.cof = cof_d;
    a.onf = onf_d;
    a.nof = nof_d;
    // stack for std::sort's recursion on top of the kernel's own frame
    size_t stack_prev = 0, stack_need = 0;
    bool raised = false;
    if (e == cudaSuccess) {
        cudaFuncAttributes fa{};
        step(cudaFuncGetAttributes(&fa, stencil_search_kernel));
        step(cudaDeviceGetLimit(&stack_prev, cudaLimitStackSize));
        stack_need = fa.localSizeBytes + SORT_STACK;
        if (e == cudaSuccess && stack_need > stack_prev) {
            step(cudaDeviceSetLimit(cudaLimitStackSize, stack_need));
            raised = e == cudaSuccess;
        }
    }
    if (e == cudaSuccess) {
        stencil_search_kernel<<<(N + 127) / 128, 128>>>(a);
        step(cudaGetLastError());
        step(cudaDeviceSynchronize());
    }
    if (e == cudaSuccess) step(cudaMemcpy(flat, a.flat, (size_t)N * 4 * M * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (e == cudaSuccess) step(cudaMemcpy(sizes, a.sizes, (size_t)N * 4, cudaMemcpyDeviceToHost));
    if (e == cudaSuccess) step(cudaMemcpy(status, a.status, (size_t)N, cudaMemcpyDeviceToHost));
    if (raised) {
        const cudaError_t r = cudaDeviceSetLimit(cudaLimitStackSize, stack_prev);
        if (e == cudaSuccess) e = r;
    }
    if (e != cudaSuccess) {
        msg = std::string("stencil search on the GPU: ") + cudaGetErrorString(e);
        return false;
    }
    return true;
}

}  // namespace mgpu
