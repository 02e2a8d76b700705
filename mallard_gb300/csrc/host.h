// host.h -- host-side data structures of the GB300 Mallard path (C++17).
//
// The host side prepares everything the kernels read: the mesh (when the
// library generates it), the TENO stencil and least-squares tables, the
// reordered device layout.  It mirrors the reference's host initialisation
// (Mesh::init_*, TENO::init) so that the GPU sees the same inputs as the
// reference's Kokkos functors would.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mallard_gb300.h"

namespace mgpu {

constexpr int NCONS = 4;  // rho, rho u, rho v, rho E
constexpr int NPRIM = 5;  // u, v, p, T, h

// An owning mesh with the reference Mesh's arrays (mesh.h:228-253).
struct HostMesh {
    uint32_t n_nodes = 0, n_cells = 0, n_faces = 0;
    std::vector<double> node_coords, cell_coords, cell_volume, face_area, face_normals;
    std::vector<uint32_t> off_noc, noc, off_foc, foc, off_nof, nof;
    std::vector<int32_t> cof;
    std::vector<uint32_t> zone_off, zone_faces;
    mgpu_mesh view() const;
};

// Derived geometry with the reference's formulas (mesh.cpp:167-261).
void derive_geometry(HostMesh& m);
HostMesh make_cartesian(uint32_t nx, uint32_t ny, double Lx, double Ly);
HostMesh make_cartesian_tri(uint32_t nx, uint32_t ny, double Lx, double Ly);
HostMesh make_wedge(uint32_t nx, uint32_t ny, double Lx, double Ly);
HostMesh make_ramp_channel(uint32_t nx, uint32_t ny, double Lx, double Ly, double x0, double ramp_deg, double jitter,
                           uint64_t seed);

// Quadrature rules (quadrature.cpp:23-273): points [n][dim], weights [n].
struct QuadRule {
    int dim = 1;
    std::vector<double> pts, wts;
    int n() const { return (int)wts.size(); }
};
bool gauss_legendre_rule(int order, QuadRule& r);
bool dunavant_rule(int order, QuadRule& r);

// Basis functions of the reference (basis.h:65-221).  Expression shapes
// follow the reference so that the tables come out bit-identical.
double basis_1d(int type, int p, double x);
double basis_1d_deriv(int type, int n, int p, double x);
inline double basis_2d(int type, int px, int py, double x, double y) { return basis_1d(type, px, x) * basis_1d(type, py, y); }

// TENO tables in the reference's layout (face_reconstruction.h:195-260).
struct TenoTables {
    int basis = MGPU_BASIS_LEGENDRE, p = 3, K = 10, M = 20;
    QuadRule qcell, qface;
    std::vector<int> pidx;                        // [K][2] polynomial powers
    std::vector<uint32_t> off_groups;             // [n_cells+1]
    std::vector<uint32_t> off_stencils;           // [n_stencils+1]
    std::vector<uint32_t> stencils;               // cells, target first
    std::vector<uint32_t> off_mats;               // [n_stencils+1]
    std::vector<double> mats;                     // K x M_s row-major per stencil
    std::vector<double> areas;                    // per stencil cell
    std::vector<double> ipt;                      // [K] mean of basis k on target
    std::vector<double> oi;                       // [K][K] oscillation indicator
};

// Throws std::runtime_error with the reference's messages on failure.
// build_teno_stencils fills everything but mats/areas; teno_stencil_lsq then
// computes one stencil's pseudo-inverse (K x M_s) and transformed areas,
// so callers can write them straight into their own layout.  gpu_search:
// the stencils are found on the current CUDA device (gpu_stencil_search),
// the cells it could not finish again on the host; same result.
void build_teno_stencils(const mgpu_mesh& m, int basis, int p, double factor, int q_cell, int q_face, TenoTables& t,
                         bool gpu_search = false);
// The stencil search on the current CUDA device (stencil_search.cu): the
// four stencils of every triangle, [cell][4][M], with their sizes, as the
// host search finds them; status[c] = 1 marks a cell the device did not
// finish (its sizes are 0).  goff/gnb: each cell's first-order
// neighbourhood, itself included, sorted.  False, with msg, on a CUDA error.
bool gpu_stencil_search(const mgpu_mesh& m, const uint32_t* goff, const uint32_t* gnb, int M, uint32_t* flat,
                        uint8_t* sizes, uint8_t* status, std::string& msg);
struct LsqWork;
LsqWork* lsq_work_new();
void lsq_work_free(LsqWork* w);
void teno_stencil_lsq(const mgpu_mesh& m, const TenoTables& t, size_t stencil, LsqWork& w, double* pinv, double* areas);
// Transformed area of cell c in its own reference frame (the first entry of
// teno_stencil_lsq's areas for any stencil of c).
double teno_target_area(const mgpu_mesh& m, const TenoTables& t, uint32_t c, LsqWork& w);
// Complete tables in the reference layout.
void build_teno_tables(const mgpu_mesh& m, int basis, int p, double factor, int q_cell, int q_face, TenoTables& t);

// Small dense helpers with the reference's arithmetic (common_math.h).
inline void mat2_vec(const double* A, const double* x, double* y) {
    double t0 = A[0] * x[0] + A[1] * x[1];
    double t1 = A[2] * x[0] + A[3] * x[1];
    y[0] = t0;
    y[1] = t1;
}
void mat2_inverse(const double* A, double* Ai);
inline void tri_jacobian(const double* a, const double* b, const double* c, double* J) {
    J[0] = b[0] - a[0];
    J[1] = c[0] - a[0];
    J[2] = b[1] - a[1];
    J[3] = c[1] - a[1];
}
double tri_area(const double* a, const double* b, const double* c);

void set_error(const std::string& msg);

}  // namespace mgpu

struct mgpu_mesh_buf {
    mgpu::HostMesh m;
    std::vector<std::string> zone_names;  // [n_zones]; zone 0 "interior"
};

namespace mgpu {
// Names of the zones of a buffer without names of its own: the generators'
// (right, top, left, bottom), else zone<i>.
void default_zone_names(mgpu_mesh_buf& b);
// Faces, cells_of_face and zones of a mesh given by its nodes and cells
// (host_mesh_io.cpp): one face per distinct cell edge, numbered in order of
// first appearance (cells in order, edges k -> k+1), nodes as in the cell
// that meets it first, which is its side-0 cell.  Boundary faces go to the
// zone of the boundary edge listed with the same two nodes (edge_zone,
// 1-based into names), else to a zone "boundary".
void build_faces(mgpu_mesh_buf& b, const std::vector<std::pair<uint64_t, uint32_t>>& edge_zone,
                 const std::vector<std::string>& names);
}  // namespace mgpu
