// host_ctx.cpp -- the solver context behind the C ABI: device layout,
// reordering, launch sequencing and the parity hooks.
//
// Boundary semantics follow the reference's classes:
//   mgpu_finalize        ~ TENO::init + Solver::allocate_memory
//   mgpu_calc_face_values~ FaceReconstruction::calc_face_values
//   mgpu_calc_rhs        ~ Solver::calc_rhs (solver_rhs.cpp:44-115)
//   mgpu_take_step       ~ SSPRK3::take_step + update_primitives
//   mgpu_calc_dt         ~ Solver::calc_dt (solver.cpp:580-590)
// Errors never cross the ABI as exceptions: every entry point returns a
// status and records a message for mgpu_last_error().
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <queue>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#include <chrono>
#endif

#include "host_ctx.h"

namespace mgpu {

namespace {
thread_local std::string g_error;

// reverse Cuthill-McKee over the face-neighbour graph; returns old_of_new
std::vector<uint32_t> rcm_order(uint32_t n, const std::vector<std::vector<uint32_t>>& adj) {
    std::vector<uint32_t> order;
    order.reserve(n);
    std::vector<char> seen(n, 0);
    std::vector<uint32_t> by_degree(n);
    std::iota(by_degree.begin(), by_degree.end(), 0u);
    std::stable_sort(by_degree.begin(), by_degree.end(),
                     [&](uint32_t a, uint32_t b) { return adj[a].size() < adj[b].size(); });
    std::vector<uint32_t> nb;
    for (uint32_t start : by_degree) {
        if (seen[start]) continue;
        size_t head = order.size();
        order.push_back(start);
        seen[start] = 1;
        while (head < order.size()) {
            const uint32_t c = order[head++];
            nb.clear();
            for (uint32_t x : adj[c])
                if (!seen[x]) nb.push_back(x);
            std::sort(nb.begin(), nb.end(), [&](uint32_t a, uint32_t b) {
                return adj[a].size() != adj[b].size() ? adj[a].size() < adj[b].size() : a < b;
            });
            for (uint32_t x : nb) {
                seen[x] = 1;
                order.push_back(x);
            }
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

}  // namespace

void set_error(const std::string& msg) { g_error = msg; }

}  // namespace mgpu

using namespace mgpu;


// ---------------------------------------------------------------------------
// mgpu_finalize: numbering, geometry precomputation, TENO tables, upload
// ---------------------------------------------------------------------------

// The least-squares tables of every stencil on the device (teno_tables.cu),
// into P / ar (FP64 forms) or P4 (FP32 form), already allocated and zeroed.
void mgpu_ctx::build_lsq_on_device(const TenoTables& t) {
    const mgpu_mesh mv = mesh.view();
    std::vector<uint3> h_tri(mv.n_cells);
    for (uint32_t c = 0; c < mv.n_cells; ++c) {
        const uint32_t* nc = mv.nodes_of_cell + mv.offsets_nodes_of_cell[c];
        h_tri[c] = make_uint3(nc[0], nc[1], nc[2]);
    }
    std::vector<double2> h_nodes(mv.n_nodes);
    for (uint32_t i = 0; i < mv.n_nodes; ++i) h_nodes[i] = make_double2(mv.node_coords[2 * (size_t)i], mv.node_coords[2 * (size_t)i + 1]);
    DevArray<uint3> d_tri;
    DevArray<double2> d_nodes;
    DevArray<uint32_t> d_cold, d_off, d_st, d_err;
    d_tri.upload(h_tri);
    d_nodes.upload(h_nodes);
    d_cold.upload(cell_old);
    d_off.upload(t.off_stencils);
    d_st.upload(t.stencils);
    d_err.alloc(1);
    LsqBuildArgs a{};
    a.n_cells = (int)N;
    a.cell_old = d_cold.p;
    a.nodes = d_nodes.p;
    a.tri = d_tri.p;
    a.off_st = d_off.p;
    a.st = d_st.p;
    a.M = t.M;
    a.K = t.K;
    a.nq = t.qcell.n();
    if (a.nq > LSQ_MAXQ || t.K > 10) throw Unsupported("GPU table build: cell quadrature or basis too large");
    for (int q = 0; q < a.nq; ++q) {
        a.qp[2 * q] = t.qcell.pts[2 * q];
        a.qp[2 * q + 1] = t.qcell.pts[2 * q + 1];
        a.qw[q] = t.qcell.wts[q];
    }
    for (int k = 0; k < t.K; ++k) {
        a.pidx[2 * k] = t.pidx[2 * k];
        a.pidx[2 * k + 1] = t.pidx[2 * k + 1];
        a.ipt[k] = t.ipt[k];
    }
    a.P = single() ? nullptr : P.p;
    a.ar = single() ? nullptr : ar.p;
    a.P4 = single() ? P4.p : nullptr;
    a.err = d_err.p;
    ck(launch_teno_lsq(a, stream), "GPU table build");
    unsigned err = 0;
    ck(cudaMemcpyAsync(&err, d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, stream), "D2H");
    ck(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    if (err & 4u) throw ArgFail("Matrix is singular.");
    if (err & 2u) throw Unsupported("least-squares system took the full-rank branch");
    if (err & 1u) throw Unsupported("unexpected stencil shape");
}

void mgpu_ctx::build() {
    const auto t_start = std::chrono::steady_clock::now();
    auto lap = [&, t = t_start](int phase) mutable {
        const auto now = std::chrono::steady_clock::now();
        build_s[phase] += std::chrono::duration<double>(now - t).count();
        t = now;
    };
    const mgpu_mesh mv = mesh.view();
    N = mv.n_cells;
    if (N == 0) throw ArgFail("mesh has no cells");
    if (mv.n_zones < 1) throw ArgFail("mesh has no interior zone");

    // --- real faces: the union of all zones; flux faces: interior + applied BCs
    std::vector<int> zone_bc(mv.n_zones, -2);  // -2 unused zone, -1 interior, else bc index
    zone_bc[0] = -1;
    for (size_t i = 0; i < bcs.size(); ++i) {
        if (zone_bc[bcs[i].zone] != -2) throw ArgFail("a face zone carries more than one boundary condition");
        zone_bc[bcs[i].zone] = (int)i;
    }
    std::vector<int> face_bc(mv.n_faces, -3);  // -3 not real
    for (uint32_t z = 0; z < mv.n_zones; ++z)
        for (uint32_t k = mv.zone_offsets[z]; k < mv.zone_offsets[z + 1]; ++k) {
            const uint32_t f = mv.zone_faces[k];
            if (face_bc[f] != -3) throw ArgFail("a face belongs to more than one zone");
            face_bc[f] = zone_bc[z];
            // interior faces join two cells, boundary faces have none on side 1
            const int32_t right = mv.cells_of_face[2 * (size_t)f + 1];
            if ((z == 0) != (right >= 0)) throw ArgFail("zone and cells_of_face disagree on a boundary face");
            if (mv.cells_of_face[2 * (size_t)f] < 0) throw ArgFail("a face has no cell on side 0");
        }
    for (uint32_t c = 0; c < N; ++c) {
        const uint32_t nf = mv.offsets_faces_of_cell[c + 1] - mv.offsets_faces_of_cell[c];
        if (nf < 3 || nf > 4) throw Unsupported("cells must have 3 or 4 faces");
        for (uint32_t k = mv.offsets_faces_of_cell[c]; k < mv.offsets_faces_of_cell[c + 1]; ++k)
            if (face_bc[mv.faces_of_cell[k]] == -3) throw ArgFail("a face of a cell belongs to no zone");
    }

    // --- cell order
    cell_old.resize(N);
    if (cfg.reorder) {
        std::vector<std::vector<uint32_t>> adj(N);
        for (uint32_t f = 0; f < mv.n_faces; ++f) {
            if (face_bc[f] == -3) continue;
            const int32_t a = mv.cells_of_face[2 * (size_t)f], b = mv.cells_of_face[2 * (size_t)f + 1];
            if (b >= 0) {
                adj[a].push_back((uint32_t)b);
                adj[b].push_back((uint32_t)a);
            }
        }
        cell_old = rcm_order(N, adj);
    } else {
        std::iota(cell_old.begin(), cell_old.end(), 0u);
    }
    cell_new.assign(N, 0);
    for (uint32_t c = 0; c < N; ++c) cell_new[cell_old[c]] = c;

    // --- face order: flux faces by internal left cell, then the rest
    std::vector<uint32_t> flux_faces, other_faces;
    for (uint32_t f = 0; f < mv.n_faces; ++f) {
        if (face_bc[f] == -3) continue;
        (face_bc[f] == -2 ? other_faces : flux_faces).push_back(f);
    }
    auto key = [&](uint32_t f) {
        const int32_t a = mv.cells_of_face[2 * (size_t)f], b = mv.cells_of_face[2 * (size_t)f + 1];
        return std::make_pair(cell_new[a], b >= 0 ? cell_new[b] : 0xffffffffu);
    };
    std::stable_sort(flux_faces.begin(), flux_faces.end(), [&](uint32_t x, uint32_t y) { return key(x) < key(y); });
    F_flux = (uint32_t)flux_faces.size();
    F_real = F_flux + (uint32_t)other_faces.size();
    face_old = flux_faces;
    face_old.insert(face_old.end(), other_faces.begin(), other_faces.end());
    face_new.assign(mv.n_faces, -1);
    for (uint32_t i = 0; i < F_real; ++i) face_new[face_old[i]] = (int32_t)i;

    lap(0);
    // --- per-face geometry (reference unit<2>, spectral-radius distance)
    std::vector<int2> h_lr(F_real);
    std::vector<double2> h_nrm(F_real);
    std::vector<double> h_area(F_real), h_dxn(F_real);
    std::vector<int8_t> h_bc(F_real, -1);
    for (uint32_t i = 0; i < F_real; ++i) {
        const uint32_t f = face_old[i];
        const int32_t a = mv.cells_of_face[2 * (size_t)f], b = mv.cells_of_face[2 * (size_t)f + 1];
        h_lr[i] = make_int2((int)cell_new[a], b >= 0 ? (int)cell_new[b] : -1);
        const double* nv = mv.face_normals + 2 * (size_t)f;
        const double inv = 1 / std::sqrt(nv[0] * nv[0] + nv[1] * nv[1]);
        const double n0 = nv[0] * inv, n1 = nv[1] * inv;
        h_nrm[i] = make_double2(n0, n1);
        h_area[i] = mv.face_area[f];
        double s0, s1;
        if (b == -1) {
            s0 = 2.0 * std::pow(mv.cell_volume[a], 1.0 / 2);
            s1 = 2.0 * std::pow(mv.cell_volume[a], 1.0 / 2);
        } else {
            s0 = mv.cell_coords[2 * (size_t)b] - mv.cell_coords[2 * (size_t)a];
            s1 = mv.cell_coords[2 * (size_t)b + 1] - mv.cell_coords[2 * (size_t)a + 1];
        }
        h_dxn[i] = std::fabs(s0 * n0 + s1 * n1);
        if (i < F_flux && face_bc[f] >= 0) h_bc[i] = (int8_t)face_bc[f];
    }

    // --- per-cell gather list in the reference's summation order
    std::vector<int4> h_gat(N, make_int4(-1, -1, -1, -1)), h_cf(N, make_int4(-1, -1, -1, -1));
    std::vector<int> fill(N, 0);
    auto push = [&](uint32_t cold, int val) {
        const uint32_t c = cell_new[cold];
        if (fill[c] >= 4) throw Unsupported("a cell receives more than 4 face fluxes");
        int* e = &h_gat[c].x;
        e[fill[c]++] = val;
    };
    for (uint32_t k = mv.zone_offsets[0]; k < mv.zone_offsets[1]; ++k) {
        const uint32_t f = mv.zone_faces[k];
        const int fn = face_new[f];
        const int32_t a = mv.cells_of_face[2 * (size_t)f], b = mv.cells_of_face[2 * (size_t)f + 1];
        push((uint32_t)a, fn * 2 + 1);
        if (b >= 0) push((uint32_t)b, fn * 2);
    }
    for (const BcHost& bc : bcs)
        for (uint32_t k = mv.zone_offsets[bc.zone]; k < mv.zone_offsets[bc.zone + 1]; ++k) {
            const uint32_t f = mv.zone_faces[k];
            push((uint32_t)mv.cells_of_face[2 * (size_t)f], face_new[f] * 2 + 1);
        }
    for (uint32_t cold = 0; cold < N; ++cold) {
        int* e = &h_cf[cell_new[cold]].x;
        int j = 0;
        for (uint32_t k = mv.offsets_faces_of_cell[cold]; k < mv.offsets_faces_of_cell[cold + 1]; ++k)
            e[j++] = face_new[mv.faces_of_cell[k]];
    }
    std::vector<double> h_vol(N);
    for (uint32_t c = 0; c < N; ++c) h_vol[c] = mv.cell_volume[cell_old[c]];

    // --- quadrature
    QuadRule qf;
    if (cfg.recon == MGPU_RECON_FO) {
        gauss_legendre_rule(1, qf);
    } else {
        const int order = cfg.quadrature_order_face > 0 ? cfg.quadrature_order_face : (cfg.poly_order + 1) / 2;
        if (!gauss_legendre_rule(order, qf)) throw ArgFail("Gauss-Legendre quadrature rule not implemented.");
    }
    nq = qf.n();
    if (nq > 2) throw Unsupported("the GPU path supports 1 or 2 face quadrature points");
    for (int q = 0; q < nq; ++q) qw[q] = qf.wts[q];

    lap(1);
    // --- TENO tables straight into the tiled layout
    const size_t tiles = (N + TILE - 1) / TILE;
    if (cfg.recon == MGPU_RECON_TENO) {
        TenoTables t;
        build_teno_stencils(mv, cfg.basis, cfg.poly_order, cfg.max_stencil_size_factor, cfg.quadrature_order_cell,
                            cfg.quadrature_order_face, t, cfg.table_build == MGPU_TABLES_GPU);
        lap(2);
        K = t.K;
        M = t.M;
        if (!((K == 10 && M == 20 && nq == 2) || (K == 6 && M == 12 && nq == 1) || (K == 3 && M == 6 && nq == 1)))
            throw Unsupported("GPU TENO kernels exist for p = 1..3 with stencil factor 2 and default face quadrature");
        const int KR = K - 1, MR = M - 1, S = 4, NF = 3;
        // FP32-bulk form: FP32 tables only, in groups of four for 16-byte
        // loads (flat index j*(K-1)+k for P), with the transformed areas
        // folded into P; face shapes as a per-cell code into one shared table
        const bool f32 = single();
        // least squares on the GPU (teno_tables.cu) unless asked for the host
        // build or the basis is monomial (std::pow)
        const bool gpu_lsq = cfg.table_build == MGPU_TABLES_GPU && cfg.basis == MGPU_BASIS_LEGENDRE;
        const size_t GJ = (MR + 3) / 4, GP = ((size_t)MR * KR + 3) / 4, GT = ((size_t)nq * KR + 3) / 4;
        auto at4 = [](size_t group, size_t lane, size_t e) { return (group * TILE + lane) * 4 + e; };
        std::vector<uint32_t> h_cface(tiles * NF * TILE, 0), h_nb, h_nb4;
        std::vector<double> h_ar, h_P, h_phi;
        std::vector<float> h_P4, h_tab;
        std::vector<uint16_t> h_fcode;
        // The FP32 form's face shapes.  In a triangle's reference frame (its
        // nodes 0, 1, 2 at (0,0), (1,0), (0,1)) the face from node i0 to node
        // i1 is a reference edge: code 2 i0 for i1 = i0 + 1 (mod 3), 2 i0 + 1
        // for i1 = i0 + 2, so six shape sets serve every cell (codes 6 and 7
        // stay zero).  Each cell's own shapes are still evaluated below and
        // must equal its codes' entries.
        const double ref[3][2] = {{0.0, 0.0}, {1.0, 0.0}, {0.0, 1.0}};
        auto edge_point = [&](int code, int q, double* x) {
            const int i0 = code / 2, i1 = (code & 1) ? (i0 + 2) % 3 : (i0 + 1) % 3;
            for (int i = 0; i < 2; i++) x[i] = (qf.pts[q] + 1.0) * 0.5 * (ref[i1][i] - ref[i0][i]) + ref[i0][i];
        };
        if (f32) {
            h_nb4.assign(tiles * S * GJ * TILE * 4, 0);
            if (!gpu_lsq) h_P4.assign(tiles * S * GP * TILE * 4, 0.0f);
            h_fcode.assign(tiles * TILE, 0x1ff);  // code 7 (zero shapes) until the cell's faces are seen
            h_tab.assign(8 * GT * 4, 0.0f);
            for (int code = 0; code < 6; ++code)
                for (int q = 0; q < nq; ++q) {
                    double xq[2];
                    edge_point(code, q, xq);
                    for (int k = 1; k < K; ++k)
                        h_tab[(size_t)code * GT * 4 + (size_t)q * KR + (k - 1)] =
                            (float)(basis_2d(t.basis, t.pidx[2 * k], t.pidx[2 * k + 1], xq[0], xq[1]) - t.ipt[k]);
                }
        } else {
            h_nb.assign(tiles * S * MR * TILE, 0);
            if (!gpu_lsq) {
                h_ar.assign(tiles * S * MR * TILE, 0.0);
                h_P.assign(tiles * S * MR * KR * TILE, 0.0);
            }
            h_phi.assign(tiles * NF * nq * KR * TILE, 0.0);
        }
        std::vector<uint8_t> h_sm(N, 0);
        std::string err;
        int nthreads = 1;
#ifdef _OPENMP
        nthreads = omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nthreads)
        {
            LsqWork* w = lsq_work_new();
            std::vector<double> pinv((size_t)K * M), ars(M);
#pragma omp for schedule(dynamic, 128)
            for (int64_t ci = 0; ci < (int64_t)N; ++ci) {
                try {
                    const uint32_t c = (uint32_t)ci, o = cell_old[c];
                    const size_t tile = c / TILE, lane = c % TILE;
                    uint8_t sm = 0;
                    for (int s = 0; s < S; ++s) {
                        const size_t si = (size_t)o * S + s;
                        const uint32_t so = t.off_stencils[si];
                        const int Ms = (int)(t.off_stencils[si + 1] - so);
                        if (Ms == 0) continue;
                        if (Ms != M || t.stencils[so] != o) throw Unsupported("unexpected stencil shape");
                        sm |= (uint8_t)(1u << s);
                        if (gpu_lsq) {
                            for (int j = 1; j < M; ++j) {
                                const size_t jj = j - 1;
                                if (f32) h_nb4[at4((tile * S + s) * GJ + jj / 4, lane, jj % 4)] = cell_new[t.stencils[so + j]];
                                else h_nb[((tile * S + s) * MR + jj) * TILE + lane] = cell_new[t.stencils[so + j]];
                            }
                            if (s == 0) ars[0] = teno_target_area(mv, t, o, *w);
                        } else {
                            teno_stencil_lsq(mv, t, si, *w, pinv.data(), ars.data());
                            for (int j = 0; j < M; ++j)
                                if (pinv[j] != 0.0) throw Unsupported("least-squares system took the full-rank branch");
                            for (int k = 0; k < K; ++k)
                                if (pinv[(size_t)k * M] != 0.0) throw Unsupported("least-squares system took the full-rank branch");
                        }
                        for (int j = 1; j < M && !gpu_lsq; ++j) {
                            if (f32) {
                                const size_t jj = j - 1;
                                h_nb4[at4((tile * S + s) * GJ + jj / 4, lane, jj % 4)] = cell_new[t.stencils[so + j]];
                                for (int k = 1; k < K; ++k) {
                                    const size_t fl = jj * KR + (k - 1);
                                    h_P4[at4((tile * S + s) * GP + fl / 4, lane, fl % 4)] =
                                        (float)(pinv[(size_t)k * M + j] * ars[j]);
                                }
                                continue;
                            }
                            const size_t b = ((tile * S + s) * MR + (j - 1)) * TILE + lane;
                            h_nb[b] = cell_new[t.stencils[so + j]];
                            h_ar[b] = ars[j];
                            for (int k = 1; k < K; ++k)
                                h_P[(((tile * S + s) * MR + (j - 1)) * KR + (k - 1)) * TILE + lane] = pinv[(size_t)k * M + j];
                        }
                        if (s == 0) {
                            // basis shape values at the face quadrature points, in the
                            // target cell's reference frame (face_reconstruction.cpp:985-1031)
                            const double area0 = ars[0];
                            const uint32_t* nc = mv.nodes_of_cell + mv.offsets_nodes_of_cell[o];
                            const double* w0 = mv.node_coords + 2 * (size_t)nc[0];
                            double J[4], Ji[4];
                            tri_jacobian(w0, mv.node_coords + 2 * (size_t)nc[1], mv.node_coords + 2 * (size_t)nc[2], J);
                            mat2_inverse(J, Ji);
                            uint32_t fcode = 0;
                            for (int fl = 0; fl < NF; ++fl) {
                                const uint32_t f = mv.faces_of_cell[mv.offsets_faces_of_cell[o] + fl];
                                const int side = mv.cells_of_face[2 * (size_t)f] == (int32_t)o ? 0 : 1;
                                h_cface[(tile * NF + fl) * TILE + lane] = (uint32_t)face_new[f] * 2u + (uint32_t)side;
                                int code = 0;
                                if (f32) {
                                    const uint32_t* fn = mv.nodes_of_face + mv.offsets_nodes_of_face[f];
                                    int i0 = -1, i1 = -1;
                                    for (int i = 0; i < 3; ++i) {
                                        if (nc[i] == fn[0]) i0 = i;
                                        if (nc[i] == fn[1]) i1 = i;
                                    }
                                    if (i0 < 0 || i1 < 0 || i0 == i1) throw Unsupported("a face is not an edge of its cell");
                                    code = i1 == (i0 + 1) % 3 ? 2 * i0 : 2 * i0 + 1;
                                    fcode |= (uint32_t)code << (3 * fl);
                                }
                                const double* p0 = mv.node_coords + 2 * (size_t)mv.nodes_of_face[mv.offsets_nodes_of_face[f]];
                                const double* p1 = mv.node_coords + 2 * (size_t)mv.nodes_of_face[mv.offsets_nodes_of_face[f] + 1];
                                double x0[2], x1[2];
                                for (int i = 0; i < 2; i++) {
                                    x0[i] = p0[i] - w0[i];
                                    x1[i] = p1[i] - w0[i];
                                }
                                mat2_vec(Ji, x0, x0);
                                mat2_vec(Ji, x1, x1);
                                for (int q = 0; q < nq; ++q) {
                                    double xq[2];
                                    for (int i = 0; i < 2; i++) xq[i] = (qf.pts[q] + 1.0) * 0.5 * (x1[i] - x0[i]) + x0[i];
                                    for (int k = 1; k < K; ++k) {
                                        const double b = basis_2d(t.basis, t.pidx[2 * k], t.pidx[2 * k + 1], xq[0], xq[1]);
                                        const double shape = cfg.teno_variant != MGPU_TENO_REFERENCE ? b - t.ipt[k]
                                                                                                   : b + (t.ipt[k] / area0);
                                        if (f32) {
                                            // the cell's own shape against its code's table entry
                                            const float own = (float)shape;
                                            const float tab = h_tab[(size_t)code * GT * 4 + (size_t)q * KR + (k - 1)];
                                            if (!(std::fabs(own - tab) <= 1e-5f * (1.0f + std::fabs(tab))))
                                                throw Unsupported("face shapes of a cell differ from its reference edge's");
                                        } else {
                                            h_phi[(((tile * NF + fl) * nq + q) * KR + (k - 1)) * TILE + lane] = shape;
                                        }
                                    }
                                }
                            }
                            if (f32) h_fcode[c] = (uint16_t)fcode;
                        }
                    }
                    h_sm[c] = sm;
                } catch (const std::exception& e) {
#pragma omp critical
                    err = e.what();
                }
            }
            lsq_work_free(w);
        }
        if (!err.empty()) throw Unsupported(err);
        teno.n_cells = (int)N;
        for (int i = 0; i < KR; ++i)
            for (int l = 0; l < KR; ++l) {
                teno.oi[i * KR + l] = t.oi[(size_t)(i + 1) * K + (l + 1)];
                teno.oi2[i * KR + l] = l < i ? 0.0 : (l == i ? 1.0 : 2.0) * t.oi[(size_t)(i + 1) * K + (l + 1)];
                teno.oi2f[i * KR + l] = (float)teno.oi2[i * KR + l];
            }
        // basis gradients at the reference centroid (1/3, 1/3), for the
        // viscous gradients from the reconstruction (the monomial basis with
        // the plain derivative p x^(p-1), not the (p+1) factor the reference
        // uses in its oscillation indicator)
        auto d1 = [&](int p, double x) {
            if (t.basis == MGPU_BASIS_MONOMIAL) return p == 0 ? 0.0 : (double)p * std::pow(x, (double)(p - 1));
            return basis_1d_deriv(t.basis, 1, p, x);
        };
        for (int k = 1; k < K; ++k) {
            const int px = t.pidx[2 * k], py = t.pidx[2 * k + 1];
            const double x = 1.0 / 3.0;
            teno.dphi[2 * (k - 1)] = d1(px, x) * basis_1d(t.basis, py, x);
            teno.dphi[2 * (k - 1) + 1] = basis_1d(t.basis, px, x) * d1(py, x);
            teno.dphif[2 * (k - 1)] = (float)teno.dphi[2 * (k - 1)];
            teno.dphif[2 * (k - 1) + 1] = (float)teno.dphi[2 * (k - 1) + 1];
        }
        if (f32) {
            nb4.upload(h_nb4);
            if (gpu_lsq) P4.alloc(tiles * S * GP * TILE * 4);
            else P4.upload(h_P4);
            fcode.upload(h_fcode);
            std::vector<float4> tab4(8 * GT);
            std::memcpy(tab4.data(), h_tab.data(), h_tab.size() * sizeof(float));
            phi_tab4.upload(tab4);
        } else {
            nb.upload(h_nb);
            if (gpu_lsq) {
                ar.alloc(tiles * S * MR * TILE);
                P.alloc(tiles * S * MR * KR * TILE);
            } else {
                ar.upload(h_ar);
                P.upload(h_P);
            }
            phi.upload(h_phi);
        }
        lap(3);
        if (gpu_lsq) build_lsq_on_device(t);
        lap(4);
        cface.upload(h_cface);
        smask.upload(h_sm);
        if (cfg.teno_variant == MGPU_TENO_ROBUST) {
            // the robust variant's first-order cells: those with a boundary face
            std::vector<uint8_t> h_bc(N, 0);
            for (uint32_t c = 0; c < N; ++c) {
                const uint32_t o = cell_old[c];
                for (uint32_t k = mv.offsets_faces_of_cell[o]; k < mv.offsets_faces_of_cell[o + 1]; ++k)
                    if (mv.cells_of_face[2 * (size_t)mv.faces_of_cell[k] + 1] < 0) h_bc[c] = 1;
            }
            bcell.upload(h_bc);
            teno.bcell = bcell.p;
        }
        teno.nb = nb.p;
        teno.ar = ar.p;
        teno.P = P.p;
        teno.phi = phi.p;
        teno.nb4 = nb4.p;
        teno.P4 = P4.p;
        teno.fcode = fcode.p;
        teno.phi_tab4 = phi_tab4.p;
        teno.cface = cface.p;
        teno.smask = smask.p;
        // compulsory bytes of one reconstruction launch: tables, shapes (the
        // FP32 form: a 2-byte code per cell), face slots, the state gathered
        // once per cell, face states written
        double tb = 0;
        const double per_row = f32 ? 4 + 4.0 * KR : 4 + 8 + 8.0 * KR, fw = f32 ? 4 : 8;
        for (uint32_t c = 0; c < N; ++c) tb += __builtin_popcount(h_sm[c]) * (double)MR * per_row;
        const double shapes = f32 ? 2.0 : NF * nq * KR * fw;
        recon_bytes = tb + (double)N * (shapes + NF * 4 + 1 + 32) + (double)N * NF * nq * 4 * fw;
    } else {
        recon_bytes = (double)F_flux * (8 + 64) + (double)N * 32;
    }

    lap(5);
    // --- BCs
    bct.n = (int)bcs.size();
    for (size_t i = 0; i < bcs.size(); ++i) {
        bct.bc[i].type = bcs[i].type;
        for (int k = 0; k < 6; ++k) bct.bc[i].data[k] = bcs[i].data[k];
    }

    // --- upload the rest
    lr.upload(h_lr);
    nrm.upload(h_nrm);
    if (single()) {
        // round to nearest once, as the kernels' FP64 -> FP32 conversion does
        std::vector<float2> h_n32(F_real);
        for (uint32_t i = 0; i < F_real; ++i) h_n32[i] = make_float2((float)h_nrm[i].x, (float)h_nrm[i].y);
        nrm32.upload(h_n32);
    }
    area.upload(h_area);
    dxn.upload(h_dxn);
    if (rcp()) {
        std::vector<double> h_idxn(F_real), h_ivol(N);
        for (uint32_t i = 0; i < F_real; ++i) h_idxn[i] = 1.0 / h_dxn[i];
        for (uint32_t c = 0; c < N; ++c) h_ivol[c] = 1.0 / h_vol[c];
        idxn.upload(h_idxn);
        ivol.upload(h_ivol);
        if (single()) {
            // rounded to nearest once, as the kernels' FP64 -> FP32 conversion does
            std::vector<float4> h_g(F_real);
            for (uint32_t i = 0; i < F_real; ++i)
                h_g[i] = make_float4((float)h_nrm[i].x, (float)h_nrm[i].y, (float)h_idxn[i], 0.0f);
            geo32.upload(h_g);
        }
    }
    bcidx.upload(h_bc);
    gat.upload(h_gat);
    cfaces.upload(h_cf);
    vol.upload(h_vol);
    U.alloc((size_t)N * 4);
    Ut.alloc((size_t)N * 4);
    W.alloc((size_t)N * 4);
    rhs.alloc((size_t)N * 4);
    prim.alloc((size_t)N * 5);
    snd.alloc(N);
    rho_cell.alloc(N);
    if (cfg.precision == MGPU_PREC_FP32) {
        fv32.alloc((size_t)F_real * nq * 8);
        U32.alloc((size_t)N * 4);
        Ut32.alloc((size_t)N * 4);
    }
    else fv.alloc((size_t)F_real * nq * 8);
    G.alloc((size_t)F_flux * 4);
    scal.alloc(2);
    flags.alloc(1);
    teno.err = flags.p;
    rmax.alloc(1);
    masks.alloc((size_t)N * 4);
    staging.alloc((size_t)N * 5);
    perm_old.upload(cell_old);
    {
        std::vector<uint32_t> cell_new(N);
        for (uint32_t c = 0; c < N; ++c) cell_new[cell_old[c]] = c;
        perm_new.upload(cell_new);
    }
    if (cfg.viscous) {
        std::vector<double2> h_xc(N), h_xf(F_real);
        for (uint32_t c = 0; c < N; ++c)
            h_xc[c] = make_double2(mv.cell_coords[2 * (size_t)cell_old[c]], mv.cell_coords[2 * (size_t)cell_old[c] + 1]);
        for (uint32_t i = 0; i < F_real; ++i) {
            const uint32_t f = face_old[i];
            const double* p0 = mv.node_coords + 2 * (size_t)mv.nodes_of_face[mv.offsets_nodes_of_face[f]];
            const double* p1 = mv.node_coords + 2 * (size_t)mv.nodes_of_face[mv.offsets_nodes_of_face[f] + 1];
            h_xf[i] = make_double2(0.5 * (p0[0] + p1[0]), 0.5 * (p0[1] + p1[1]));
        }
        xc.upload(h_xc);
        xf.upload(h_xf);
        grad.alloc((size_t)N * 6);
        visc.n_cells = (int)N;
        visc.n_faces = (int)F_flux;
        visc.cfaces = cfaces.p;
        visc.lr = lr.p;
        visc.nrm = nrm.p;
        visc.area = area.p;
        visc.vol = vol.p;
        visc.bc = bcidx.p;
        visc.xc = xc.p;
        visc.xf = xf.p;
        visc.grad = grad.p;
        visc.G = G.p;
        visc.mu_ref = cfg.mu_ref;
        visc.T_ref = cfg.T_mu_ref;
        visc.S = cfg.sutherland_S;
        const double cp = gas.R * cfg.gamma / (cfg.gamma - 1.0);
        visc.cp_over_pr = cp / cfg.prandtl;
        if (single()) {
            // face geometry of the FP32 viscous flux, derived in FP64 and
            // rounded once: normal, centre-line direction, area, 1 / length
            std::vector<float4> g0(F_real);
            std::vector<float2> g1(F_real);
            for (uint32_t i = 0; i < F_real; ++i) {
                const int2 e = h_lr[i];
                const double2 a = h_xc[e.x], b = e.y >= 0 ? h_xc[e.y] : h_xf[i];
                const double dx = b.x - a.x, dy = b.y - a.y, dl = std::sqrt(dx * dx + dy * dy);
                g0[i] = make_float4((float)h_nrm[i].x, (float)h_nrm[i].y, (float)(dx / dl), (float)(dy / dl));
                g1[i] = make_float2((float)h_area[i], (float)(1.0 / dl));
            }
            vgeo.upload(g0);
            vgeo2.upload(g1);
            vq.alloc(N);
            vga.alloc(N);
            vgb.alloc(N);
            visc32.n_cells = (int)N;
            visc32.cfaces = cfaces.p;
            visc32.lr = lr.p;
            visc32.bc = bcidx.p;
            visc32.fgeo = vgeo.p;
            visc32.fgeo2 = vgeo2.p;
            visc32.ivol = ivol.p;
            visc32.q = vq.p;
            visc32.ga = vga.p;
            visc32.gb = vgb.p;
            visc32.mu_ref = (float)cfg.mu_ref;
            visc32.T_ref = (float)cfg.T_mu_ref;
            visc32.S = (float)cfg.sutherland_S;
            visc32.cp_over_pr = (float)visc.cp_over_pr;
            visc32.inv_cv = (float)(1.0 / gas.cv);
        }
        if (recon_grads()) {
            // per cell the inverse Jacobian of its TENO reference frame
            // (nodes 0, 1, 2 at (0,0), (1,0), (0,1)), as the tables use it
            std::vector<double> h_ji((size_t)N * 4);
            for (uint32_t c = 0; c < N; ++c) {
                const uint32_t* nc = mv.nodes_of_cell + mv.offsets_nodes_of_cell[cell_old[c]];
                double J[4];
                tri_jacobian(mv.node_coords + 2 * (size_t)nc[0], mv.node_coords + 2 * (size_t)nc[1],
                             mv.node_coords + 2 * (size_t)nc[2], J);
                mat2_inverse(J, &h_ji[4 * (size_t)c]);
            }
            teno.cv = gas.cv;
            teno.inv_cv = (float)(1.0 / gas.cv);
            if (single()) {
                std::vector<float4> h4(N);
                for (uint32_t c = 0; c < N; ++c)
                    h4[c] = make_float4((float)h_ji[4 * (size_t)c], (float)h_ji[4 * (size_t)c + 1],
                                        (float)h_ji[4 * (size_t)c + 2], (float)h_ji[4 * (size_t)c + 3]);
                ji4.upload(h4);
                teno.ji4 = ji4.p;
                teno.vq = vq.p;
                teno.vga = vga.p;
                teno.vgb = vgb.p;
            } else {
                ji.upload(h_ji);
                teno.ji = ji.p;
                teno.vgrad = grad.p;
                visc.grad_ready = 1;
            }
        }
    }
    // compulsory bytes of one stage: reconstruction + flux (face states in,
    // G out, face geometry) + update (G gathered, state in/out)
    const double flux_b = (double)F_flux * (nq * 64 + 32 + 8 + 16 + 8 + 1);
    const double upd_b = (double)N * (16 + 8 + 32 * 4) + (double)F_flux * 32 * 2;
    stage_bytes = recon_bytes + flux_b + upd_b;
    lap(6);
    finalized = true;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

const char* mgpu_last_error(void) { return g_error.c_str(); }
int mgpu_version(void) { return 100; }

void mgpu_config_defaults(mgpu_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->recon = MGPU_RECON_TENO;
    c->basis = MGPU_BASIS_LEGENDRE;
    c->poly_order = 3;
    c->max_stencil_size_factor = 2.0;
    c->riemann_solver = MGPU_RIEMANN_HLLC;
    c->time_integrator = MGPU_INTEGRATOR_SSPRK3;
    c->gamma = 1.4;
    c->p_ref = 101325.0;
    c->T_ref = 298.15;
    c->rho_ref = 1.225;
    c->p_min = -1e20;
    c->p_max = 1e20;
    c->teno_variant = MGPU_TENO_REFERENCE;
    c->precision = MGPU_PREC_FP64;
    c->reorder = 1;
    c->device = 0;
    c->viscous = 0;
    c->mu_ref = 0.0;
    c->T_mu_ref = 1.0;
    c->sutherland_S = 0.0;
    c->prandtl = 0.72;
    c->table_build = MGPU_TABLES_GPU;
    c->viscous_gradients = MGPU_VISC_GRAD_RECON;
}

int mgpu_create(const mgpu_mesh* mesh, const mgpu_config* cfg, mgpu_ctx** out) {
    return guarded([&] {
        if (!mesh || !cfg || !out) throw ArgFail("mgpu_create: null argument");
        if (cfg->recon != MGPU_RECON_FO && cfg->recon != MGPU_RECON_TENO) throw ArgFail("Unknown face reconstruction type.");
        if (cfg->riemann_solver < 0 || cfg->riemann_solver > 2) throw ArgFail("Unknown Riemann solver type.");
        if (cfg->time_integrator != MGPU_INTEGRATOR_SSPRK3 && cfg->time_integrator != MGPU_INTEGRATOR_FE &&
            cfg->time_integrator != MGPU_INTEGRATOR_RK4)
            throw ArgFail("Unknown time integrator type.");
        if (cfg->precision != MGPU_PREC_FP64 && cfg->precision != MGPU_PREC_FP64_FAST &&
            cfg->precision != MGPU_PREC_FP32)
            throw Unsupported("unknown precision mode");
        if (cfg->table_build != MGPU_TABLES_GPU && cfg->table_build != MGPU_TABLES_HOST)
            throw ArgFail("table_build: MGPU_TABLES_GPU or MGPU_TABLES_HOST");
        if (cfg->viscous_gradients != MGPU_VISC_GRAD_RECON && cfg->viscous_gradients != MGPU_VISC_GRAD_GREEN_GAUSS)
            throw ArgFail("viscous_gradients: MGPU_VISC_GRAD_RECON or MGPU_VISC_GRAD_GREEN_GAUSS");
        if (cfg->viscous && !(cfg->mu_ref >= 0.0 && cfg->prandtl > 0.0 && (cfg->sutherland_S <= 0.0 || cfg->T_mu_ref > 0.0)))
            throw ArgFail("viscous flux: mu_ref >= 0, prandtl > 0 and, with Sutherland's law, T_mu_ref > 0");
        if (cfg->precision == MGPU_PREC_FP32 &&
            (cfg->recon != MGPU_RECON_TENO || cfg->teno_variant == MGPU_TENO_REFERENCE))
            throw Unsupported("the FP32 form implements TENO with the corrected or robust weighting");
        if (cfg->teno_variant != MGPU_TENO_REFERENCE && cfg->teno_variant != MGPU_TENO_CORRECTED &&
            cfg->teno_variant != MGPU_TENO_ROBUST)
            throw ArgFail("unknown TENO variant");
        if (cfg->basis != MGPU_BASIS_LEGENDRE && cfg->basis != MGPU_BASIS_MONOMIAL) throw ArgFail("Unknown basis type.");
        if (!(cfg->gamma > 1.0) || !(cfg->p_ref > 0) || !(cfg->T_ref > 0) || !(cfg->rho_ref > 0))
            throw ArgFail("invalid physics constants");
        auto ctx = std::make_unique<mgpu_ctx>();
        ctx->cfg = *cfg;
        HostMesh& m = ctx->mesh;
        m.n_nodes = mesh->n_nodes;
        m.n_cells = mesh->n_cells;
        m.n_faces = mesh->n_faces;
        auto cp = [](auto& dst, const auto* src, size_t n) {
            if (!src && n) throw ArgFail("mgpu_create: null mesh array");
            dst.assign(src, src + n);
        };
        cp(m.node_coords, mesh->node_coords, 2 * (size_t)m.n_nodes);
        cp(m.cell_coords, mesh->cell_coords, 2 * (size_t)m.n_cells);
        cp(m.cell_volume, mesh->cell_volume, m.n_cells);
        cp(m.face_area, mesh->face_area, m.n_faces);
        cp(m.face_normals, mesh->face_normals, 2 * (size_t)m.n_faces);
        cp(m.off_noc, mesh->offsets_nodes_of_cell, (size_t)m.n_cells + 1);
        cp(m.noc, mesh->nodes_of_cell, m.off_noc.back());
        cp(m.off_foc, mesh->offsets_faces_of_cell, (size_t)m.n_cells + 1);
        cp(m.foc, mesh->faces_of_cell, m.off_foc.back());
        cp(m.off_nof, mesh->offsets_nodes_of_face, (size_t)m.n_faces + 1);
        cp(m.nof, mesh->nodes_of_face, m.off_nof.back());
        cp(m.cof, mesh->cells_of_face, 2 * (size_t)m.n_faces);
        cp(m.zone_off, mesh->zone_offsets, (size_t)mesh->n_zones + 1);
        cp(m.zone_faces, mesh->zone_faces, m.zone_off.back());
        for (uint32_t f : m.foc)
            if (f >= m.n_faces) throw ArgFail("mesh: face index out of range");
        for (uint32_t f : m.zone_faces)
            if (f >= m.n_faces) throw ArgFail("mesh: zone face out of range");
        for (uint32_t n : m.noc)
            if (n >= m.n_nodes) throw ArgFail("mesh: node index out of range");
        for (uint32_t n : m.nof)
            if (n >= m.n_nodes) throw ArgFail("mesh: node index out of range");
        for (size_t i = 0; i < m.cof.size(); ++i)
            if (m.cof[i] >= (int32_t)m.n_cells || m.cof[i] < -1) throw ArgFail("mesh: cells_of_face out of range");
        // Euler::set_R_cp_cv (physics.cpp:69-73)
        const double R = cfg->p_ref / (cfg->T_ref * cfg->rho_ref);
        const double cp_ = R * cfg->gamma / (cfg->gamma - 1.0);
        ctx->gas.gamma = cfg->gamma;
        ctx->gas.R = R;
        ctx->gas.cv = cp_ / cfg->gamma;
        ctx->gas.p_min = cfg->p_min;
        ctx->gas.p_max = cfg->p_max;
        ctx->gas.icv = 1.0 / ctx->gas.cv;
        ctx->gas.gamma_f = (float)ctx->gas.gamma;
        ctx->gas.R_f = (float)ctx->gas.R;
        ctx->gas.cv_f = (float)ctx->gas.cv;
        ctx->gas.icv_f = (float)(1.0 / ctx->gas.cv);
        ctx->gas.gm1_f = (float)(ctx->gas.gamma - 1.0);
        ctx->gas.p_min_f = (float)ctx->gas.p_min;
        ctx->gas.p_max_f = (float)ctx->gas.p_max;
        ck(cudaSetDevice(cfg->device), "cudaSetDevice");
        ck(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        ctx->own_stream = true;
        *out = ctx.release();
        return MGPU_OK;
    });
}

int mgpu_add_boundary(mgpu_ctx* ctx, uint32_t zone, int bc_type, const double* data, int n_data) {
    return guarded([&] {
        if (!ctx) throw ArgFail("null context");
        if (ctx->finalized) throw ArgFail("boundaries must be added before mgpu_finalize");
        if (zone == 0 || zone + 1 >= ctx->mesh.zone_off.size()) throw ArgFail("Boundary name not found in mesh.");
        if (ctx->bcs.size() >= (size_t)MAX_BC) throw Unsupported("too many boundary conditions");
        BcHost b{};
        b.zone = zone;
        b.type = bc_type;
        if (bc_type == MGPU_BC_UPT) {
            // BoundaryUPT::init (boundary_upt.cpp:38-73): data = (u, v, p, T)
            if (!data || n_data < 4) throw ArgFail("Missing u, p or T for boundary.");
            const double u0 = data[0], u1 = data[1], p = data[2], T = data[3];
            const double rho = p / (ctx->gas.R * T);
            const double e = ctx->gas.cv * T;
            const double h = e + p / rho;
            const double d[6] = {rho, u0, u1, p, T, h};
            std::memcpy(b.data, d, sizeof(d));
        } else if (bc_type == MGPU_BC_P_OUT) {
            if (!data || n_data < 1) throw ArgFail("Missing p for boundary.");
            b.data[0] = data[0];
        } else if (bc_type < 0 || bc_type > MGPU_BC_P_OUT) {
            throw ArgFail("Unknown boundary type.");
        }
        ctx->bcs.push_back(b);
        return MGPU_OK;
    });
}

int mgpu_finalize(mgpu_ctx* ctx) {
    return guarded([&] {
        if (!ctx) throw ArgFail("null context");
        if (ctx->finalized) return MGPU_OK;
        ck(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
        ctx->build();
        return MGPU_OK;
    });
}

int mgpu_destroy(mgpu_ctx* ctx) {
    if (ctx) {
        cudaSetDevice(ctx->cfg.device);
        if (ctx->stream) cudaStreamSynchronize(ctx->stream);
        delete ctx;
    }
    return MGPU_OK;
}

int mgpu_set_stream(mgpu_ctx* ctx, void* stream) {
    return guarded([&] {
        if (!ctx) throw ArgFail("null context");
        if (ctx->stream) ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
        if (stream) {
            ctx->stream = (cudaStream_t)stream;
            ctx->own_stream = false;
        } else {
            ck(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
            ctx->own_stream = true;
        }
        ctx->drop_graphs();
        return MGPU_OK;
    });
}

int mgpu_synchronize(mgpu_ctx* ctx) {
    return guarded([&] {
        if (!ctx) throw ArgFail("null context");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        return MGPU_OK;
    });
}

int mgpu_set_state(mgpu_ctx* ctx, const double* Uh, const double* primh) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (!Uh) throw ArgFail("null state");
        ctx->upload_cells(ctx->U.p, Uh, 4, ctx->single() ? ctx->U32.p : nullptr);
        if (ctx->single() && !primh) {
            // the FP32 form's step reads neither the FP64 primitives nor the
            // sound speeds: they are recovered from U when a caller asks
            ctx->prim_stale = true;
        } else {
            if (primh) {
                ctx->upload_cells(ctx->prim.p, primh, 5);
            } else {
                ck(launch_primitives_batch(ctx->gas, ctx->N, ctx->U.p, ctx->prim.p, ctx->stream), "primitives");
            }
            ck(launch_sound((int)ctx->N, ctx->gas.gamma, ctx->U.p, ctx->prim.p, ctx->snd.p, ctx->stream),
               "sound speed");
            ctx->prim_stale = false;
        }
        ck(cudaMemsetAsync(ctx->flags.p, 0, sizeof(unsigned), ctx->stream), "cudaMemsetAsync");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        return MGPU_OK;
    });
}

int mgpu_get_state(mgpu_ctx* ctx, double* Uh, double* primh) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (Uh) ctx->download_cells(ctx->U.p, Uh, 4);
        if (primh) {
            ctx->refresh_prims();
            ctx->download_cells(ctx->prim.p, primh, 5);
        }
        return MGPU_OK;
    });
}

int mgpu_calc_face_values(mgpu_ctx* ctx, const double* Uh, double* face, uint8_t* tmask) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (!Uh || !face) throw ArgFail("null argument");
        ctx->upload_cells(ctx->Ut.p, Uh, 4);
        const bool sgl = ctx->single();
        if (sgl) ck(cudaMemsetAsync(ctx->fv32.p, 0, ctx->fv32.bytes(), ctx->stream), "cudaMemsetAsync");
        else ck(cudaMemsetAsync(ctx->fv.p, 0, ctx->fv.bytes(), ctx->stream), "cudaMemsetAsync");
        if (ctx->single()) ck(launch_to_f32((size_t)ctx->N * 4, ctx->Ut.p, ctx->Ut32.p, ctx->stream), "FP32 copy");
        ctx->reconstruct(ctx->Ut.p, ctx->masks.p);
        const int nq = ctx->nq;
        std::vector<double> tmp((size_t)ctx->F_real * nq * 8);
        if (sgl) {
            std::vector<float> t32(tmp.size());
            ck(cudaMemcpyAsync(t32.data(), ctx->fv32.p, t32.size() * sizeof(float), cudaMemcpyDeviceToHost,
                               ctx->stream),
               "D2H");
            ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
            for (size_t i = 0; i < t32.size(); ++i) tmp[i] = t32[i];
        } else {
            ck(cudaMemcpyAsync(tmp.data(), ctx->fv.p, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream),
               "D2H");
        }
        std::vector<uint8_t> mk((size_t)ctx->N * 4);
        if (tmask)
            ck(cudaMemcpyAsync(mk.data(), ctx->masks.p, mk.size(), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        std::memset(face, 0, (size_t)ctx->mesh.n_faces * nq * 8 * sizeof(double));
        for (uint32_t i = 0; i < ctx->F_real; ++i)
            std::memcpy(face + (size_t)ctx->face_old[i] * nq * 8, &tmp[(size_t)i * nq * 8], nq * 8 * sizeof(double));
        if (tmask)
            for (uint32_t c = 0; c < ctx->N; ++c) std::memcpy(tmask + (size_t)ctx->cell_old[c] * 4, &mk[(size_t)c * 4], 4);
        return MGPU_OK;
    });
}

int mgpu_calc_rhs(mgpu_ctx* ctx, const double* Uh, double* rhsh) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (!Uh || !rhsh) throw ArgFail("null argument");
        ctx->upload_cells(ctx->Ut.p, Uh, 4);
        if (ctx->single()) ck(launch_to_f32((size_t)ctx->N * 4, ctx->Ut.p, ctx->Ut32.p, ctx->stream), "FP32 copy");
        ctx->reconstruct(ctx->Ut.p, nullptr);
        ctx->flux(ctx->Ut.p);
        ctx->viscous(ctx->Ut.p);
        UpdateArgs a = ctx->update_args();
        ck(launch_update(a, ctx->gas, 0, MGPU_INTEGRATOR_SSPRK3, ctx->rcp(), ctx->stream), "update");
        ctx->download_cells(ctx->rhs.p, rhsh, 4);
        return MGPU_OK;
    });
}

int mgpu_calc_dt(mgpu_ctx* ctx, double cfl, double* dt, double* cfl_local) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (!dt) throw ArgFail("null argument");
        ctx->spectral_and_dt(cfl, false);
        double h = 0;
        ck(cudaMemcpyAsync(&h, ctx->dt_ptr(), sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        *dt = h;
        if (cfl_local) {
            ctx->download_cells(ctx->rho_cell.p, cfl_local, 1);
            for (uint32_t c = 0; c < ctx->N; ++c) cfl_local[c] = h * cfl_local[c];
        }
        if (h < 0.0) {
            set_error("dt negative: " + std::to_string(h) + ".");
            return MGPU_ERR_NAN;
        }
        return MGPU_OK;
    });
}

int mgpu_take_step(mgpu_ctx* ctx, double dt) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        ck(launch_set_scalar(ctx->dt_ptr(), dt, ctx->stream), "set dt");
        for (int k = 1; k <= ctx->n_stages(); ++k) ctx->stage(k);
        ctx->prim_stale = ctx->single();
        return MGPU_OK;
    });
}

int mgpu_run(mgpu_ctx* ctx, double cfl, uint32_t n_steps, double* t_out) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        ck(launch_set_scalar(ctx->t_ptr(), 0.0, ctx->stream), "set t");
        if (n_steps > 0 && ctx->single()) ctx->prim_stale = true;
        // a prediction step every sel_interval steps, counted from this call
        const uint32_t every = ctx->sel_on ? ctx->sel_interval : 1;
        if (ctx->timing) {
            for (uint32_t s = 0; s < n_steps; ++s) ctx->cfl_step(cfl, s % every == 0);
        } else {
            if (ctx->step_cfl != cfl) ctx->drop_graphs();
            auto capture = [&](bool predict, cudaGraphExec_t* exec) {
                cudaGraph_t g = nullptr;
                ck(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
                try {
                    ctx->cfl_step(cfl, predict);
                } catch (...) {
                    cudaStreamEndCapture(ctx->stream, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                ck(cudaStreamEndCapture(ctx->stream, &g), "cudaStreamEndCapture");
                cudaError_t e = cudaGraphInstantiate(exec, g, 0);
                cudaGraphDestroy(g);
                ck(e, "cudaGraphInstantiate");
            };
            if (!ctx->step_exec) capture(true, &ctx->step_exec);
            if (every > 1 && !ctx->step_exec_np) capture(false, &ctx->step_exec_np);
            ctx->step_cfl = cfl;
            for (uint32_t s = 0; s < n_steps; ++s)
                ck(cudaGraphLaunch(s % every == 0 ? ctx->step_exec : ctx->step_exec_np, ctx->stream), "cudaGraphLaunch");
        }
        if (t_out) {
            double h = 0;
            ck(cudaMemcpyAsync(&h, ctx->t_ptr(), sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
            ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
            *t_out = h;
        }
        return MGPU_OK;
    });
}

int mgpu_status(mgpu_ctx* ctx, uint32_t* flags) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        unsigned h = 0;
        ck(cudaMemcpyAsync(&h, ctx->flags.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        if (flags) *flags = h;
        if (h & 4u) {
            set_error("a bounded device wait ran out");
            return MGPU_ERR_TIMEOUT;
        }
        return h ? MGPU_ERR_NAN : MGPU_OK;
    });
}

int mgpu_enable_kernel_timing(mgpu_ctx* ctx, int enable) {
    return guarded([&] {
        if (!ctx) throw ArgFail("null context");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        ctx->timing = enable != 0;
        ctx->marks_used = 0;
        return MGPU_OK;
    });
}

int mgpu_kernel_times(mgpu_ctx* ctx, double* ms, uint32_t* launches) {
    return guarded([&] {
        if (!ctx || !ms || !launches) throw ArgFail("null argument");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        for (int i = 0; i < 5; ++i) {
            ms[i] = 0.0;
            launches[i] = 0;
        }
        for (size_t i = 0; i < ctx->marks_used; ++i) {
            float t = 0.f;
            ck(cudaEventElapsedTime(&t, ctx->marks[i].a, ctx->marks[i].b), "cudaEventElapsedTime");
            ms[ctx->marks[i].cls] += t;
            launches[ctx->marks[i].cls] += 1;
        }
        ctx->marks_used = 0;
        return MGPU_OK;
    });
}

int mgpu_autotune(mgpu_ctx* ctx, double* ms, int* best) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        const int n = ctx->single() && ctx->K == 10 ? f32::TENO32_SHAPES : 1;
        std::vector<double> t(f32::TENO32_SHAPES, 0.0);
        cudaEvent_t a, b;
        ck(cudaEventCreate(&a), "cudaEventCreate");
        ck(cudaEventCreate(&b), "cudaEventCreate");
        const bool timing = ctx->timing;
        ctx->timing = false;
        int choice = 0;
        double tbest = 1e300;
        try {
            for (int sh = 0; sh < n; ++sh) {
                ctx->teno_shape = sh;
                ctx->reconstruct(ctx->U.p, nullptr, true);  // warm-up (and the selector's predictions)
                ck(cudaEventRecord(a, ctx->stream), "cudaEventRecord");
                for (int r = 0; r < 3; ++r) ctx->reconstruct(ctx->U.p, nullptr, false);
                ck(cudaEventRecord(b, ctx->stream), "cudaEventRecord");
                ck(cudaEventSynchronize(b), "cudaEventSynchronize");
                float f = 0.f;
                ck(cudaEventElapsedTime(&f, a, b), "cudaEventElapsedTime");
                t[sh] = f / 3.0;
                if (t[sh] < tbest) {
                    tbest = t[sh];
                    choice = sh;
                }
            }
        } catch (...) {
            ctx->timing = timing;
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            throw;
        }
        ctx->timing = timing;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        ctx->teno_shape = choice;
        ctx->drop_graphs();  // recapture with the chosen shape
        if (ms)
            for (int i = 0; i < f32::TENO32_SHAPES; ++i) ms[i] = t[i];
        if (best) *best = choice;
        return MGPU_OK;
    });
}

int mgpu_set_launch_shape(mgpu_ctx* ctx, int shape) {
    if (int rc = need_ready(ctx)) return rc;
    const int n = ctx->single() && ctx->K == 10 ? f32::TENO32_SHAPES : 1;
    if (shape < 0 || shape >= n) {
        set_error("launch shape out of range for this form");
        return MGPU_ERR_ARG;
    }
    ctx->teno_shape = shape;
    ctx->drop_graphs();
    return MGPU_OK;
}

int mgpu_traffic_model(mgpu_ctx* ctx, double* recon_bytes, double* stage_bytes) {
    if (int rc = need_ready(ctx)) return rc;
    if (recon_bytes) *recon_bytes = ctx->recon_bytes;
    if (stage_bytes) *stage_bytes = ctx->stage_bytes;
    return MGPU_OK;
}

int mgpu_build_times(mgpu_ctx* ctx, double* seconds) {
    if (int rc = need_ready(ctx)) return rc;
    if (!seconds) return MGPU_ERR_ARG;
    for (int i = 0; i < 7; ++i) seconds[i] = ctx->build_s[i];
    return MGPU_OK;
}

int mgpu_get_table(mgpu_ctx* ctx, int field, void* dst, uint64_t* bytes) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (!bytes) throw ArgFail("null argument");
        const void* src = nullptr;
        size_t n = 0;
        switch (field) {
            case MGPU_TABLE_P: src = ctx->P.p; n = ctx->P.bytes(); break;
            case MGPU_TABLE_AREAS: src = ctx->ar.p; n = ctx->ar.bytes(); break;
            case MGPU_TABLE_P32: src = ctx->P4.p; n = ctx->P4.bytes(); break;
            case MGPU_TABLE_NB: src = ctx->nb.p; n = ctx->nb.bytes(); break;
            case MGPU_TABLE_NB32: src = ctx->nb4.p; n = ctx->nb4.bytes(); break;
            case MGPU_TABLE_PHI: src = ctx->phi.p; n = ctx->phi.bytes(); break;
            case MGPU_TABLE_PHI32: src = ctx->fcode.p; n = ctx->fcode.bytes(); break;
            default: throw ArgFail("unknown table");
        }
        if (!src) throw ArgFail("this form holds no such table");
        *bytes = n;
        if (dst) {
            ck(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
            ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        }
        return MGPU_OK;
    });
}

uint32_t mgpu_n_cells(const mgpu_ctx* ctx) { return ctx ? ctx->mesh.n_cells : 0; }

int mgpu_riemann_flux_batch(int solver, uint32_t n, const double* n_unit, const double* rho_l, const double* u_l,
                            const double* p_l, const double* gamma_l, const double* h_l, const double* rho_r,
                            const double* u_r, const double* p_r, const double* gamma_r, const double* h_r,
                            double* flux) {
    return guarded([&] {
        if ((solver & ~MGPU_RIEMANN_GUARD) < 0 || (solver & ~MGPU_RIEMANN_GUARD) > 2)
            throw ArgFail("Unknown Riemann solver type.");
        if (n == 0) return MGPU_OK;
        if (!n_unit || !rho_l || !u_l || !p_l || !gamma_l || !h_l || !rho_r || !u_r || !p_r || !gamma_r || !h_r || !flux)
            throw ArgFail("null argument");
        std::vector<double> in((size_t)n * 14);
        for (uint32_t i = 0; i < n; ++i) {
            double* b = &in[(size_t)i * 14];
            b[0] = n_unit[2 * i]; b[1] = n_unit[2 * i + 1];
            b[2] = rho_l[i]; b[3] = u_l[2 * i]; b[4] = u_l[2 * i + 1]; b[5] = p_l[i]; b[6] = gamma_l[i]; b[7] = h_l[i];
            b[8] = rho_r[i]; b[9] = u_r[2 * i]; b[10] = u_r[2 * i + 1]; b[11] = p_r[i]; b[12] = gamma_r[i]; b[13] = h_r[i];
        }
        DevArray<double> din, dout;
        din.upload(in);
        dout.alloc((size_t)n * 4);
        ck(launch_riemann_batch(solver, n, din.p, dout.p, 0), "riemann launch");
        ck(cudaMemcpy(flux, dout.p, (size_t)n * 4 * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
        return MGPU_OK;
    });
}

int mgpu_primitives_batch(double gamma, double p_ref, double T_ref, double rho_ref, double p_min, double p_max,
                          uint32_t n, const double* Uh, double* Wh) {
    return guarded([&] {
        if (n == 0) return MGPU_OK;
        if (!Uh || !Wh) throw ArgFail("null argument");
        GasParams g{};
        const double R = p_ref / (T_ref * rho_ref);
        const double cp_ = R * gamma / (gamma - 1.0);
        g.gamma = gamma;
        g.R = R;
        g.cv = cp_ / gamma;
        g.p_min = p_min;
        g.p_max = p_max;
        std::vector<double> u(Uh, Uh + (size_t)n * 4);
        DevArray<double> du, dw;
        du.upload(u);
        dw.alloc((size_t)n * 5);
        ck(launch_primitives_batch(g, n, du.p, dw.p, 0), "primitives launch");
        ck(cudaMemcpy(Wh, dw.p, (size_t)n * 5 * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
        return MGPU_OK;
    });
}

int mgpu_probe_conversions(int device, const double* in64, float* out32, const float* in32, double* out64, uint64_t n) {
    return guarded([&] {
        if (n && (!in64 || !out32 || !in32 || !out64)) throw ArgFail("null argument");
        ck(run_convert_probe(device, in64, out32, in32, out64, (size_t)n), "conversion probe");
        return MGPU_OK;
    });
}

int mgpu_probe_fp64_gflops(int device, double* gflops) {
    return guarded([&] {
        if (!gflops) throw ArgFail("null argument");
        ck(run_fp64_probe(device, gflops), "fp64 probe");
        return MGPU_OK;
    });
}

}  // extern "C"

namespace mgpu {

// The spectral-radius inputs of a finalized context, for entry points that
// live in other translation units (noalloc.cu).  Allocates nothing.
bool ctx_spectral_view(mgpu_ctx* ctx, SpecArgs* s, const uint32_t** cell_old, cudaStream_t* stream, int* device,
                       unsigned** flags) {
    if (!ctx || !ctx->finalized || !s || !cell_old || !stream || !device || !flags) return false;
    *s = SpecArgs{};
    s->n_cells = (int)ctx->N;
    s->cfaces = ctx->cfaces.p;
    s->lr = ctx->lr.p;
    s->nrm = ctx->nrm.p;
    s->dxn = ctx->dxn.p;
    s->U = ctx->U.p;
    s->prim = ctx->prim.p;
    ctx->spec_fp32(*s);
    *cell_old = ctx->perm_old.p;
    *stream = ctx->stream;
    *device = ctx->cfg.device;
    *flags = ctx->flags.p;
    return true;
}

}  // namespace mgpu
