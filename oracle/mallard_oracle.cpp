// mallard_oracle.cpp -- CPU oracle for the Mallard residual-and-update hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is a plain C++ restatement of the
// reference solver's algorithm (MatthewBonanni/Mallard, src/...), used as the
// checker for the GPU path and as the timed CPU baseline.  Nothing in the
// product (mallard_gb300/) links, loads or calls it; only tests/, the
// smoke() entry and bench.py's CPU leg do.
//
// The reference itself cannot be compiled here: it depends on Kokkos,
// KokkosKernels and toml11, which are absent.  Every routine below therefore
// restates the reference routine named in its comment, keeping the same
// arithmetic order (the file is compiled with -ffp-contract=off and without
// -ffast-math so that x86 and aarch64 hosts produce identical bits).  The
// restatement is pinned by the reference's own unit-test golden values
// (test/riemann_solver_test.cpp, test/physics_test.cpp,
// test/time_integrator_test.cpp, test/common_math_test.cpp).
//
// Layouts follow the reference's host views (LayoutRight):
//   U          [n_cells][4]            (rho, rho u, rho v, rho E)
//   primitives [n_cells][5]            (u, v, p, T, h)
//   face       [n_faces][n_q][2][4]    (side 0 = cells_of_face(f,0))
// Threads: orc_set_threads(1) (default) reproduces Kokkos::Serial order
// exactly; more threads use OpenMP with atomic scatter like Kokkos::OpenMP.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <random>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int NC = 4;   // conservative variables (common_typedef.h:20)
constexpr int NP = 5;   // primitive variables   (common_typedef.h:21)

int g_threads = 1;
std::string g_last_error;

// ---------------------------------------------------------------------------
// Small dense algebra -- restates src/common/common_math.h
// ---------------------------------------------------------------------------

// gemv<2> (common_math.h:207-213): temporaries first, so in-place is allowed.
inline void mv2(const double* A, const double* x, double* y) {
    double t0 = A[0] * x[0] + A[1] * x[1];
    double t1 = A[2] * x[0] + A[3] * x[1];
    y[0] = t0;
    y[1] = t1;
}

// invert_matrix<2> (common_math.h:145-159)
inline void inv2(const double* A, double* Ai) {
    double det = A[0] * A[3] - A[1] * A[2];
    if (det == 0.0) throw std::runtime_error("Matrix is singular.");
    double r = 1.0 / det;
    Ai[0] = A[3] * r;
    Ai[1] = -A[1] * r;
    Ai[2] = -A[2] * r;
    Ai[3] = A[0] * r;
}

// triangle_J (common_math.h:533-542): columns are the two edge vectors.
inline void tri_jac(const double* a, const double* b, const double* c, double* J) {
    J[0] = b[0] - a[0];
    J[1] = c[0] - a[0];
    J[2] = b[1] - a[1];
    J[3] = c[1] - a[1];
}

// triangle_area<2> (common_math.h:509-516)
inline double tri_area(const double* a, const double* b, const double* c) {
    return 0.5 * std::fabs(a[0] * (b[1] - c[1]) + b[0] * (c[1] - a[1]) + c[0] * (a[1] - b[1]));
}

// gemm, no transposes (common_math.h:240-272): C[m x q] = A[m x n] B[n x q].
void mm(const double* A, const double* B, double* C, int m, int n, int q) {
    std::vector<double> out((size_t)m * q);
    for (int i = 0; i < m; i++)
        for (int j = 0; j < q; j++) {
            double s = 0.0;
            for (int k = 0; k < n; k++) s += A[i * n + k] * B[k * q + j];
            out[(size_t)i * q + j] = s;
        }
    std::copy(out.begin(), out.end(), C);
}

// QR_householder_noQ (common_math.h:355-422): R <- Q_n..Q_1 A with explicit
// m x m reflectors applied by a full gemm, exactly as the reference does.
void householder_r(const double* A, double* R, int m, int n) {
    for (int i = 0; i < m * n; i++) R[i] = A[i];
    std::vector<double> v(m), Q((size_t)m * m);
    for (int j = 0; j < n; j++) {
        double nx = 0.0;
        for (int i = j; i < m; i++) nx += R[i * n + j] * R[i * n + j];
        nx = std::sqrt(nx);
        if (nx < 1.0e-15) continue;
        double sgn = (R[j * n + j] >= 0.0) ? 1.0 : -1.0;
        double alpha = -sgn * nx;
        double nu = 0.0;
        for (int k = 0; k < m - j; k++) {
            v[k] = R[(j + k) * n + j];
            if (k == 0) v[k] -= alpha;
            nu += v[k] * v[k];
        }
        nu = std::sqrt(nu);
        for (int k = 0; k < m - j; k++) v[k] /= nu;
        for (int i = 0; i < m; i++)
            for (int k = 0; k < m; k++) Q[(size_t)i * m + k] = (i == k) ? 1.0 : 0.0;
        for (int i = j; i < m; i++)
            for (int k = j; k < m; k++) Q[(size_t)i * m + k] -= 2.0 * v[i - j] * v[k - j];
        mm(Q.data(), R, R, m, m, n);
    }
}

// forward_substitution (common_math.h:436-457)
void fwd_subst(const double* L, const double* B, double* X, int m, int n, int p, bool tL, bool tB) {
    for (int i = 0; i < m; i++)
        for (int j = 0; j < p; j++) {
            double s = 0.0;
            for (int k = 0; k < i; k++) {
                int iL = tL ? k * m + i : i * n + k;
                s += L[iL] * X[k * p + j];
            }
            int iB = tB ? j * n + i : i * p + j;
            int iD = tL ? i * m + i : i * n + i;
            X[i * p + j] = (B[iB] - s) / L[iD];
        }
}

// back_substitution (common_math.h:471-493)
void back_subst(const double* U, const double* B, double* X, int m, int n, int p, bool tU, bool tB) {
    for (int i = m - 1; i >= 0; i--)
        for (int j = 0; j < p; j++) {
            double s = 0.0;
            int end = tU ? n : m;
            for (int k = i + 1; k < end; k++) {
                int iU = tU ? k * m + i : i * n + k;
                s += U[iU] * X[k * p + j];
            }
            int iB = tB ? j * n + i : i * p + j;
            int iD = tU ? i * m + i : i * n + i;
            X[i * p + j] = (B[iB] - s) / U[iD];
        }
}

// ---------------------------------------------------------------------------
// Basis functions -- restates src/numerics/basis.h:65-221 (p <= 4 needed)
// ---------------------------------------------------------------------------

enum { BASIS_MONOMIAL = 0, BASIS_LEGENDRE = 1 };

double legendre(int p, double x) {  // LegendreTraits::compute_1D (basis.h:83-94)
    switch (p) {
        case 0: return 1.0 * (1.0);
        case 1: return 1.0 * (1.0 * x);
        case 2: return 0.5 * (3.0 * x * x - 1.0);
        case 3: return 0.5 * (5.0 * x * x * x - 3.0 * x);
        case 4: return 0.125 * (35.0 * x * x * x * x - 30.0 * x * x + 3.0);
        case 5: return 0.125 * (63.0 * x * x * x * x * x - 70.0 * x * x * x + 15.0 * x);
        default: throw std::runtime_error("oracle: Legendre order > 5 not restated");
    }
}

// LegendreTraits::derivative_1D (basis.h:110-184), orders used for p <= 4.
double legendre_d(int n, int p, double x) {
    if (n > p) return 0.0;
    if (n == 0) return legendre(p, x);
    if (n == 1) {
        switch (p) {
            case 1: return 1.0 * (1.0 * 1.0);
            case 2: return 0.5 * (3.0 * 2.0 * x);
            case 3: return 0.5 * (5.0 * 3.0 * x * x - 3.0 * 1.0);
            case 4: return 0.125 * (35.0 * 4.0 * x * x * x - 30.0 * 2.0 * x);
        }
    } else if (n == 2) {
        switch (p) {
            case 2: return 0.5 * (3.0 * 2.0 * 1.0);
            case 3: return 0.5 * (5.0 * 3.0 * 2.0 * x);
            case 4: return 0.125 * (35.0 * 4.0 * 3.0 * x * x - 30.0 * 2.0 * 1.0);
        }
    } else if (n == 3) {
        switch (p) {
            case 3: return 0.5 * (5.0 * 3.0 * 2.0 * 1.0);
            case 4: return 0.125 * (35.0 * 4.0 * 3.0 * 2.0 * x);
        }
    } else if (n == 4) {
        if (p == 4) return 0.125 * (35.0 * 4.0 * 3.0 * 2.0 * 1.0);
    }
    throw std::runtime_error("oracle: Legendre derivative order not restated");
}

// MonomialTraits (basis.h:65-79), including its (p - k + 1) factor.
double monomial(int p, double x) { return std::pow(x, (double)p); }
double monomial_d(int n, int p, double x) {
    double r = std::pow(x, (double)(p - n));
    for (int k = 0; k < n; ++k) r *= (double)(p - k + 1);
    return r;
}

inline double basis1(int type, int p, double x) {
    return type == BASIS_LEGENDRE ? legendre(p, x) : monomial(p, x);
}
inline double basis1_d(int type, int n, int p, double x) {
    return type == BASIS_LEGENDRE ? legendre_d(n, p, x) : monomial_d(n, p, x);
}
inline double basis2(int type, int px, int py, double x, double y) {
    return basis1(type, px, x) * basis1(type, py, y);
}

// ---------------------------------------------------------------------------
// Quadrature -- restates src/numerics/quadrature.cpp:23-273
// ---------------------------------------------------------------------------

struct Rule {
    std::vector<double> pts;  // [n][dim]
    std::vector<double> wts;  // [n]
    int dim = 1;
    int n() const { return (int)wts.size(); }
};

Rule gauss_legendre(int order) {
    Rule r;
    r.dim = 1;
    switch (order) {
        case 1: r.pts = {0.0}; r.wts = {2.0}; break;
        case 2:
            r.pts = {-0.577350269189625764509149, 0.577350269189625764509149};
            r.wts = {1.0, 1.0};
            break;
        case 3:
            r.pts = {-0.774596669241483377035853, 0.0, 0.774596669241483377035853};
            r.wts = {0.55555555555555555555556, 0.88888888888888888888889, 0.55555555555555555555556};
            break;
        case 4:
            r.pts = {-0.861136311594052575223946, -0.339981043584856264802666,
                     0.339981043584856264802666, 0.861136311594052575223946};
            r.wts = {0.34785484513745385737306, 0.65214515486254614262694,
                     0.65214515486254614262694, 0.34785484513745385737306};
            break;
        default: throw std::runtime_error("Gauss-Legendre quadrature rule of order " + std::to_string(order) + " not implemented.");
    }
    return r;
}

Rule dunavant(int order) {
    Rule r;
    r.dim = 2;
    switch (order) {
        case 1: r.pts = {1.0 / 3.0, 1.0 / 3.0}; r.wts = {1.0}; break;
        case 2:
            r.pts = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
            r.wts = {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0};
            break;
        case 3:
            r.pts = {1.0 / 3.0, 1.0 / 3.0, 0.6, 0.2, 0.2, 0.6, 0.2, 0.2};
            r.wts = {-0.5625, 0.52083333333333333333333333333333, 0.52083333333333333333333333333333,
                     0.52083333333333333333333333333333};
            break;
        case 4:
            r.pts = {0.108103018168070, 0.445948490915965, 0.445948490915965, 0.108103018168070,
                     0.445948490915965, 0.445948490915965, 0.816847572980459, 0.091576213509771,
                     0.091576213509771, 0.816847572980459, 0.091576213509771, 0.091576213509771};
            r.wts = {0.223381589678011, 0.223381589678011, 0.223381589678011,
                     0.109951743655322, 0.109951743655322, 0.109951743655322};
            break;
        case 5:
            r.pts = {0.333333333333333, 0.333333333333333, 0.059715871789770, 0.470142064105115,
                     0.470142064105115, 0.059715871789770, 0.470142064105115, 0.470142064105115,
                     0.797426985353087, 0.101286507323456, 0.101286507323456, 0.797426985353087,
                     0.101286507323456, 0.101286507323456};
            r.wts = {0.225000000000000, 0.132394152788506, 0.132394152788506, 0.132394152788506,
                     0.125939180544827, 0.125939180544827, 0.125939180544827};
            break;
        default: throw std::runtime_error("Triangle Dunavant quadrature rule of order " + std::to_string(order) + " not implemented.");
    }
    return r;
}

// ---------------------------------------------------------------------------
// Mesh -- restates src/mesh/mesh.cpp (generators + derived geometry)
// ---------------------------------------------------------------------------

struct OMesh {
    uint32_t n_nodes = 0, n_cells = 0, n_faces = 0;
    std::vector<double> node_coords, cell_coords, cell_volume, face_area, face_normals;
    std::vector<uint32_t> off_noc, noc, off_foc, foc, off_nof, nof;
    std::vector<int32_t> cof;
    std::vector<std::string> zone_names;
    std::vector<uint32_t> zone_off, zone_faces;  // zone 0 is "interior"

    uint32_t n_nodes_of_cell(uint32_t c) const { return off_noc[c + 1] - off_noc[c]; }
    uint32_t n_faces_of_cell(uint32_t c) const { return off_foc[c + 1] - off_foc[c]; }
    uint32_t node_of_cell(uint32_t c, int i) const { return noc[off_noc[c] + i]; }
    uint32_t face_of_cell(uint32_t c, int i) const { return foc[off_foc[c] + i]; }
    uint32_t node_of_face(uint32_t f, int i) const { return nof[off_nof[f] + i]; }
    const double* nc(uint32_t n) const { return &node_coords[2 * (size_t)n]; }
    const double* cc(uint32_t c) const { return &cell_coords[2 * (size_t)c]; }
};

// Mesh::compute_face_areas (mesh.cpp:218-227)
void geom_face_areas(OMesh& m) {
    for (uint32_t f = 0; f < m.n_faces; ++f) {
        const double* a = m.nc(m.node_of_face(f, 0));
        const double* b = m.nc(m.node_of_face(f, 1));
        double dx = b[0] - a[0], dy = b[1] - a[1];
        m.face_area[f] = std::sqrt(dx * dx + dy * dy);
    }
}

// Mesh::compute_cell_volumes (mesh.cpp:181-216)
void geom_cell_volumes(OMesh& m) {
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        uint32_t nn = m.n_nodes_of_cell(c);
        if (nn == 3) {
            m.cell_volume[c] = tri_area(m.nc(m.node_of_cell(c, 0)), m.nc(m.node_of_cell(c, 1)), m.nc(m.node_of_cell(c, 2)));
        } else if (nn == 4) {
            double a1 = tri_area(m.nc(m.node_of_cell(c, 0)), m.nc(m.node_of_cell(c, 1)), m.nc(m.node_of_cell(c, 2)));
            double a2 = tri_area(m.nc(m.node_of_cell(c, 0)), m.nc(m.node_of_cell(c, 2)), m.nc(m.node_of_cell(c, 3)));
            m.cell_volume[c] = a1 + a2;
        } else {
            throw std::runtime_error("Unknown cell type.");
        }
    }
}

// Mesh::compute_cell_centroids (mesh.cpp:167-179): vertex average.
void geom_centroids(OMesh& m) {
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        double x = 0.0, y = 0.0;
        uint32_t nn = m.n_nodes_of_cell(c);
        for (uint32_t i = 0; i < nn; ++i) {
            x += m.nc(m.node_of_cell(c, i))[0];
            y += m.nc(m.node_of_cell(c, i))[1];
        }
        m.cell_coords[2 * (size_t)c] = x / nn;
        m.cell_coords[2 * (size_t)c + 1] = y / nn;
    }
}

// Mesh::compute_face_normals (mesh.cpp:229-261): area-weighted, pointing out of cell 0.
void geom_normals(OMesh& m) {
    for (uint32_t f = 0; f < m.n_faces; ++f) {
        const double* a = m.nc(m.node_of_face(f, 0));
        const double* b = m.nc(m.node_of_face(f, 1));
        double dx = b[0] - a[0], dy = b[1] - a[1];
        double mag = std::sqrt(dx * dx + dy * dy);
        double nx = dy / mag * m.face_area[f];
        double ny = -dx / mag * m.face_area[f];
        int32_t c0 = m.cof[2 * (size_t)f];
        double ox = 0.5 * (a[0] + b[0]) - m.cc(c0)[0];
        double oy = 0.5 * (a[1] + b[1]) - m.cc(c0)[1];
        if (ox * nx + oy * ny < 0) {
            nx *= -1;
            ny *= -1;
        }
        m.face_normals[2 * (size_t)f] = nx;
        m.face_normals[2 * (size_t)f + 1] = ny;
    }
}

void geom_all(OMesh& m) {
    m.face_area.assign(m.n_faces, 0.0);
    m.cell_volume.assign(m.n_cells, 0.0);
    m.cell_coords.assign(2 * (size_t)m.n_cells, 0.0);
    m.face_normals.assign(2 * (size_t)m.n_faces, 0.0);
    geom_face_areas(m);
    geom_cell_volumes(m);
    geom_centroids(m);
    geom_normals(m);
}

void pack_csr(const std::vector<std::vector<uint32_t>>& lists, std::vector<uint32_t>& off, std::vector<uint32_t>& flat) {
    off.assign(lists.size() + 1, 0);
    flat.clear();
    for (size_t i = 0; i < lists.size(); ++i) {
        off[i + 1] = off[i] + (uint32_t)lists[i].size();
        flat.insert(flat.end(), lists[i].begin(), lists[i].end());
    }
}

void set_zones(OMesh& m, std::vector<uint32_t> fi, const std::vector<uint32_t>& fr, const std::vector<uint32_t>& ft,
               const std::vector<uint32_t>& fl, const std::vector<uint32_t>& fb) {
    std::sort(fi.begin(), fi.end());
    fi.erase(std::unique(fi.begin(), fi.end()), fi.end());
    m.zone_names = {"interior", "right", "top", "left", "bottom"};
    std::vector<std::vector<uint32_t>> z = {fi, fr, ft, fl, fb};
    pack_csr(z, m.zone_off, m.zone_faces);
}

// Mesh::init_cart (mesh.cpp:305-557)
OMesh gen_cart(uint32_t nx, uint32_t ny, double Lx, double Ly) {
    OMesh m;
    m.n_cells = nx * ny;
    m.n_nodes = (nx + 1) * (ny + 1);
    m.n_faces = 2 * m.n_cells + nx + ny;
    m.node_coords.assign(2 * (size_t)m.n_nodes, 0.0);
    m.cof.assign(2 * (size_t)m.n_faces, 0);
    std::vector<std::vector<uint32_t>> noc(m.n_cells, std::vector<uint32_t>(4)), foc(m.n_cells, std::vector<uint32_t>(4)),
        nof(m.n_faces, std::vector<uint32_t>(2, 0));
    double dx = Lx / nx, dy = Ly / ny;
    for (uint32_t i = 0; i < nx + 1; ++i)
        for (uint32_t j = 0; j < ny + 1; ++j) {
            uint32_t n = i * (ny + 1) + j;
            m.node_coords[2 * (size_t)n] = i * dx;
            m.node_coords[2 * (size_t)n + 1] = j * dy;
        }
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        uint32_t ic = c / ny, jc = c % ny;
        uint32_t ntr = (ic + 1) * (ny + 1) + jc + 1, ntl = ic * (ny + 1) + jc + 1;
        uint32_t nbl = ic * (ny + 1) + jc, nbr = (ic + 1) * (ny + 1) + jc;
        uint32_t fr = (2 * ny + 1) * (ic + 1) + jc, ft = (2 * ny + 1) * ic + jc + ny + 1;
        uint32_t fl = (2 * ny + 1) * ic + jc, fb = (2 * ny + 1) * ic + jc + ny;
        noc[c] = {ntr, ntl, nbl, nbr};
        foc[c] = {fr, ft, fl, fb};
        m.cof[2 * fr] = c; m.cof[2 * fr + 1] = ic == nx - 1 ? -1 : (int32_t)(c + ny);
        m.cof[2 * ft] = c; m.cof[2 * ft + 1] = jc == ny - 1 ? -1 : (int32_t)(c + 1);
        m.cof[2 * fl] = c; m.cof[2 * fl + 1] = ic == 0 ? -1 : (int32_t)(c - ny);
        m.cof[2 * fb] = c; m.cof[2 * fb + 1] = jc == 0 ? -1 : (int32_t)(c - 1);
        nof[fr] = {nbr, ntr};
        nof[ft] = {ntr, ntl};
        nof[fl] = {ntl, nbl};
        nof[fb] = {nbl, nbr};
    }
    std::vector<uint32_t> zi, zr, zt, zl, zb;
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        uint32_t ic = c / ny, jc = c % ny;
        (ic == nx - 1 ? zr : zi).push_back(foc[c][0]);
        (jc == ny - 1 ? zt : zi).push_back(foc[c][1]);
        (ic == 0 ? zl : zi).push_back(foc[c][2]);
        (jc == 0 ? zb : zi).push_back(foc[c][3]);
    }
    set_zones(m, zi, zr, zt, zl, zb);
    pack_csr(noc, m.off_noc, m.noc);
    pack_csr(foc, m.off_foc, m.foc);
    pack_csr(nof, m.off_nof, m.nof);
    geom_all(m);
    return m;
}

// Mesh::init_cart_tri (mesh.cpp:559-826).  Allocates 3*n_cells+nx+ny faces of
// which only 1.5*n_cells+nx+ny are used; the rest keep zero nodes and cells
// (Kokkos zero-initialises views) and NaN normals, and belong to no zone.
OMesh gen_cart_tri(uint32_t nx, uint32_t ny, double Lx, double Ly) {
    OMesh m;
    m.n_cells = 2 * nx * ny;
    m.n_nodes = (nx + 1) * (ny + 1);
    m.n_faces = 3 * m.n_cells + nx + ny;
    m.node_coords.assign(2 * (size_t)m.n_nodes, 0.0);
    m.cof.assign(2 * (size_t)m.n_faces, 0);
    std::vector<std::vector<uint32_t>> noc(m.n_cells, std::vector<uint32_t>(3)), foc(m.n_cells, std::vector<uint32_t>(3)),
        nof(m.n_faces, std::vector<uint32_t>(2, 0));
    double dx = Lx / nx, dy = Ly / ny;
    for (uint32_t i = 0; i < nx + 1; ++i)
        for (uint32_t j = 0; j < ny + 1; ++j) {
            uint32_t n = i * (ny + 1) + j;
            m.node_coords[2 * (size_t)n] = i * dx;
            m.node_coords[2 * (size_t)n + 1] = j * dy;
        }
    for (uint32_t q = 0; q < nx * ny; ++q) {
        uint32_t ic = q / ny, jc = q % ny;
        uint32_t ccr = 2 * q, ccl = ccr + 1;
        uint32_t ntr = (ic + 1) * (ny + 1) + jc + 1, ntl = ic * (ny + 1) + jc + 1;
        uint32_t nbl = ic * (ny + 1) + jc, nbr = (ic + 1) * (ny + 1) + jc;
        uint32_t col = (3 * ny + 1) * ic;
        uint32_t fr = (3 * ny + 1) * (ic + 1) + jc, ft = col + 2 * jc + ny + 2;
        uint32_t fl = col + jc, fb = col + 2 * jc + ny, fd = col + 2 * jc + ny + 1;
        noc[ccr] = {nbr, ntr, nbl};
        noc[ccl] = {ntl, nbl, ntr};
        foc[ccr] = {fb, fr, fd};
        foc[ccl] = {ft, fl, fd};
        m.cof[2 * fr] = ccr; m.cof[2 * fr + 1] = ic == nx - 1 ? -1 : (int32_t)(ccl + 2 * ny);
        m.cof[2 * ft] = ccl; m.cof[2 * ft + 1] = jc == ny - 1 ? -1 : (int32_t)(ccl + 1);
        m.cof[2 * fl] = ccl; m.cof[2 * fl + 1] = ic == 0 ? -1 : (int32_t)(ccr - 2 * ny);
        m.cof[2 * fb] = ccr; m.cof[2 * fb + 1] = jc == 0 ? -1 : (int32_t)(ccr - 1);
        m.cof[2 * fd] = ccr; m.cof[2 * fd + 1] = ccl;
        nof[fr] = {nbr, ntr};
        nof[ft] = {ntr, ntl};
        nof[fl] = {ntl, nbl};
        nof[fb] = {nbl, nbr};
        nof[fd] = {nbl, ntr};
    }
    std::vector<uint32_t> zi, zr, zt, zl, zb;
    for (uint32_t q = 0; q < nx * ny; ++q) {
        uint32_t ic = q / ny, jc = q % ny;
        uint32_t ccr = 2 * q, ccl = ccr + 1;
        (ic == nx - 1 ? zr : zi).push_back(foc[ccr][1]);
        (jc == ny - 1 ? zt : zi).push_back(foc[ccl][0]);
        (ic == 0 ? zl : zi).push_back(foc[ccl][1]);
        (jc == 0 ? zb : zi).push_back(foc[ccr][0]);
        zi.push_back(foc[ccr][2]);
    }
    set_zones(m, zi, zr, zt, zl, zb);
    pack_csr(noc, m.off_noc, m.noc);
    pack_csr(foc, m.off_foc, m.foc);
    pack_csr(nof, m.off_nof, m.nof);
    geom_all(m);
    return m;
}

// Mesh::init_wedge (mesh.cpp:828-848): cartesian quads, nodes past x=0.5
// sheared onto an 8-degree ramp, geometry recomputed.
OMesh gen_wedge(uint32_t nx, uint32_t ny, double Lx, double Ly) {
    OMesh m = gen_cart(nx, ny, Lx, Ly);
    const double pi = 3.14159265358979323846;
    double theta = 8 * pi / 180.0, xw = 0.5;
    for (uint32_t n = 0; n < m.n_nodes; ++n) {
        double x = m.node_coords[2 * (size_t)n], y = m.node_coords[2 * (size_t)n + 1];
        if (x > xw) {
            double yb = (x - xw) * std::tan(theta);
            m.node_coords[2 * (size_t)n + 1] = (y / Ly) * (Ly - yb) + yb;
        }
    }
    geom_all(m);
    return m;
}

// ---------------------------------------------------------------------------
// TENO tables -- restates src/numerics/face_reconstruction.cpp:109-788
// ---------------------------------------------------------------------------

struct Teno {
    int basis = BASIS_LEGENDRE;
    int p = 3;
    int K = 10;   // n_dof
    int M = 20;   // max_cells_per_stencil
    Rule qcell, qface;
    std::vector<int> pidx;  // [K][2]
    std::vector<uint32_t> off_groups, off_stencils, stencils, off_mats;
    std::vector<double> mats, areas, ipt, oi;
};

// Mesh::h_neighbors_of_cell with n_order = 1 (mesh.cpp:127-165)
void neighbours1(const OMesh& m, uint32_t c, std::vector<uint32_t>& out) {
    out.clear();
    out.push_back(c);
    for (uint32_t k = 0; k < m.n_faces_of_cell(c); ++k) {
        uint32_t f = m.face_of_cell(c, k);
        int32_t c0 = m.cof[2 * (size_t)f], c1 = m.cof[2 * (size_t)f + 1];
        if (c1 == -1) continue;
        out.push_back(c0 == (int32_t)c ? (uint32_t)c1 : (uint32_t)c0);
    }
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
}

// TENO::get_next_ring (face_reconstruction.cpp:217-265)
void next_ring(const OMesh& m, std::vector<std::vector<uint32_t>>& rings, uint32_t target) {
    std::vector<uint32_t> ring, nb;
    for (uint32_t c : rings.back()) {
        neighbours1(m, c, nb);
        for (uint32_t n : nb) {
            bool seen = false;
            for (const auto& r : rings)
                if (std::find(r.begin(), r.end(), n) != r.end()) { seen = true; break; }
            if (!seen && std::find(ring.begin(), ring.end(), n) == ring.end()) ring.push_back(n);
        }
    }
    std::vector<std::pair<uint32_t, double>> d;
    for (uint32_t n : ring) {
        double s = 0.0;
        for (int i = 0; i < 2; i++) {
            double t = m.cc(n)[i] - m.cc(target)[i];
            s += t * t;
        }
        d.push_back(std::make_pair(n, s));
    }
    std::sort(d.begin(), d.end(), [](auto& a, auto& b) { return a.second < b.second; });
    ring.clear();
    for (auto& pr : d) ring.push_back(pr.first);
    rings.push_back(ring);
}

// TENO::compute_stencil_of_cell_centered (face_reconstruction.cpp:267-286)
std::vector<uint32_t> stencil_central(const OMesh& m, int M, uint32_t c) {
    std::vector<uint32_t> st = {c};
    std::vector<std::vector<uint32_t>> rings = {st};
    while ((int)st.size() < M) {
        next_ring(m, rings, c);
        for (uint32_t n : rings.back()) {
            if ((int)st.size() == M) break;
            st.push_back(n);
        }
    }
    return st;
}

// TENO::compute_stencils_of_cell_directional (face_reconstruction.cpp:288-404)
std::vector<std::vector<uint32_t>> stencils_directional(const OMesh& m, int M, uint32_t c) {
    int ns = (int)m.n_faces_of_cell(c);
    std::vector<std::vector<uint32_t>> st(ns);
    std::vector<bool> grew(ns);
    std::vector<std::vector<double>> Jinv(ns, std::vector<double>(4));
    for (int s = 0; s < ns; ++s) {
        uint32_t f = m.face_of_cell(c, s);
        double J[4];
        tri_jac(m.cc(c), m.nc(m.node_of_face(f, 0)), m.nc(m.node_of_face(f, 1)), J);
        inv2(J, Jinv[s].data());
    }
    for (auto& x : st) x.push_back(c);
    std::vector<std::vector<uint32_t>> rings = {{c}};
    bool done = false;
    while (!done) {
        next_ring(m, rings, c);
        std::fill(grew.begin(), grew.end(), false);
        for (int s = 0; s < ns; ++s) {
            for (uint32_t n : rings.back()) {
                if ((int)st[s].size() == M) break;
                double d[2] = {m.cc(n)[0] - m.cc(c)[0], m.cc(n)[1] - m.cc(c)[1]};
                double t[2];
                mv2(Jinv[s].data(), d, t);
                if (!(t[0] < 0.0) && !(t[1] < 0.0)) {
                    st[s].push_back(n);
                    grew[s] = true;
                }
            }
        }
        done = true;
        for (int s = 0; s < ns; ++s) {
            if (m.cof[2 * (size_t)m.face_of_cell(c, s) + 1] != -1 && (int)st[s].size() < M && grew[s]) {
                done = false;
                break;
            }
        }
    }
    for (int s = 0; s < ns; ++s) {
        if (m.cof[2 * (size_t)m.face_of_cell(c, s) + 1] == -1) {
            st[s].clear();
            continue;
        }
        rings.clear();
        rings.push_back(st[s]);
        while ((int)st[s].size() < M) {
            next_ring(m, rings, c);
            for (uint32_t n : rings.back()) {
                if ((int)st[s].size() == M) break;
                st[s].push_back(n);
            }
        }
    }
    return st;
}

// TENO::calc_max_stencil_size + calc_polynomial_indices (face_reconstruction.cpp:170-215)
void teno_sizes(Teno& t, double factor) {
    int nd = 1, den = 1;
    for (int i = 1; i <= 2; ++i) {
        den *= i;
        nd *= t.p + i;
    }
    t.K = nd / den;
    t.M = (int)(uint16_t)(factor * t.K);
    t.pidx.clear();
    for (int ip = 0; ip <= t.p; ip++) {
        int a = ip, b = 0;
        t.pidx.push_back(a);
        t.pidx.push_back(b);
        while (b < ip) {
            if (a > 0) { a -= 1; b += 1; }
            t.pidx.push_back(a);
            t.pidx.push_back(b);
        }
    }
}

// TENO::compute_stencils (face_reconstruction.cpp:406-475).  Each cell's
// stencils depend on the mesh alone, so with more than one oracle thread
// they are searched in parallel and then concatenated in cell order (the
// same tables as the serial loop).
void teno_stencils(Teno& t, const OMesh& m) {
    t.off_groups = {0};
    t.off_stencils = {0};
    t.stencils.clear();
    std::vector<std::vector<std::vector<uint32_t>>> per(m.n_cells);
    std::string err;
#pragma omp parallel for schedule(dynamic, 256) if (g_threads > 1) num_threads(g_threads)
    for (int64_t ci = 0; ci < (int64_t)m.n_cells; ++ci) {
        try {
            const uint32_t c = (uint32_t)ci;
            per[c].push_back(stencil_central(m, t.M, c));
            for (auto& s : stencils_directional(m, t.M, c)) per[c].push_back(std::move(s));
        } catch (const std::exception& e) {
#pragma omp critical
            err = e.what();
        }
    }
    if (!err.empty()) throw std::runtime_error(err);
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        std::vector<std::vector<uint32_t>> all;
        all.swap(per[c]);
        for (auto& s : all) {
            if ((int)s.size() < t.M && s.size() > 0) throw std::runtime_error("Stencil is not full.");
            t.stencils.insert(t.stencils.end(), s.begin(), s.end());
            t.off_stencils.push_back((uint32_t)t.stencils.size());
        }
        t.off_groups.push_back((uint32_t)t.off_stencils.size() - 1);
    }
}

// TENO::compute_reconstruction_matrices (face_reconstruction.cpp:477-741),
// one stencil: its transformed areas and pseudo-inverse into at/A.  set_ipt:
// the basis means of the target (from cell 0, stencil 0, :598-602) are
// taken from this stencil first.
void stencil_matrix(Teno& t, const OMesh& m, uint32_t c, int sl, bool set_ipt, double* at, double* A) {
    const int K = t.K;
    const int nq = t.qcell.n();
    const double* w0 = m.nc(m.node_of_cell(c, 0));
    double J[4], Ji[4];
    tri_jac(w0, m.nc(m.node_of_cell(c, 1)), m.nc(m.node_of_cell(c, 2)), J);
    inv2(J, Ji);
    const uint32_t s = t.off_groups[c] + sl;
    const uint32_t so = t.off_stencils[s];
    const int M = (int)(t.off_stencils[s + 1] - so);
    std::vector<double> R((size_t)M * K), Y((size_t)K * M);
    for (int j = 0; j < M; ++j) {
        uint32_t nb = t.stencils[so + j];
        double v[3][2];
        for (int k = 0; k < 3; ++k) {
            v[k][0] = m.nc(m.node_of_cell(nb, k))[0];
            v[k][1] = m.nc(m.node_of_cell(nb, k))[1];
        }
        double Jn[4];
        tri_jac(v[0], v[1], v[2], Jn);
        double vt[3][2];
        for (int k = 0; k < 3; ++k) {
            vt[k][0] = v[k][0] - w0[0];
            vt[k][1] = v[k][1] - w0[1];
            mv2(Ji, vt[k], vt[k]);
        }
        at[j] = tri_area(vt[0], vt[1], vt[2]);
        std::vector<double> qp(2 * (size_t)nq);
        for (int q = 0; q < nq; ++q) {
            double x[2] = {t.qcell.pts[2 * q], t.qcell.pts[2 * q + 1]};
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
            double& a = A[(size_t)j * K + k];
            a = 0.0;
            for (int q = 0; q < nq; ++q)
                a += t.qcell.wts[q] * basis2(t.basis, t.pidx[2 * k], t.pidx[2 * k + 1], qp[2 * q], qp[2 * q + 1]);
            a *= at[j];
        }
    }
    if (set_ipt)
        for (int k = 0; k < K; ++k) t.ipt[k] = A[k] / at[0];
    for (int j = 0; j < M; ++j)
        for (int k = 0; k < K; ++k) A[(size_t)j * K + k] -= at[j] * t.ipt[k];
    bool col0_zero = true;
    for (int j = 0; j < M; ++j)
        if (A[(size_t)j * K] > 1.0e-12) { col0_zero = false; break; }
    if (col0_zero) {
        std::vector<double> B((size_t)(M - 1) * (K - 1));
        for (int j = 1; j < M; ++j)
            for (int k = 1; k < K; ++k) B[(size_t)(j - 1) * (K - 1) + (k - 1)] = A[(size_t)j * K + k];
        householder_r(B.data(), R.data(), M - 1, K - 1);
        fwd_subst(R.data(), B.data(), Y.data(), K - 1, K - 1, M - 1, true, true);
        back_subst(R.data(), Y.data(), B.data(), K - 1, K - 1, M - 1, false, false);
        for (int k = 0; k < K; ++k)
            for (int j = 0; j < M; ++j)
                A[(size_t)k * M + j] = (k == 0 || j == 0) ? 0.0 : B[(size_t)(k - 1) * (M - 1) + (j - 1)];
    } else {
        householder_r(A, R.data(), M, K);
        fwd_subst(R.data(), A, Y.data(), K, K, M, true, true);
        back_subst(R.data(), Y.data(), A, K, K, M, false, false);
    }
}

// All stencils: offsets first, then every stencil's matrix in place (in
// parallel with more than one oracle thread; each stencil's arithmetic is
// its own, so the tables equal the serial build's).
void teno_matrices(Teno& t, const OMesh& m) {
    const int K = t.K;
    t.ipt.assign(K, 0.0);
    std::vector<size_t> mo(t.off_stencils.size()), ao(t.off_stencils.size());
    size_t nm = 0, na = 0;
    t.off_mats = {0};
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        if (m.n_nodes_of_cell(c) != 3) throw std::runtime_error("TENO has only been implemented for triangular cells.");
        for (uint32_t s = t.off_groups[c]; s < t.off_groups[c + 1]; ++s) {
            const size_t M = t.off_stencils[s + 1] - t.off_stencils[s];
            if (M == 0 && s == t.off_groups[c])
                throw std::runtime_error("Central stencil is empty for cell " + std::to_string(c) + ".");
            mo[s] = nm;
            ao[s] = na;
            nm += (size_t)K * M;
            na += M;
            t.off_mats.push_back((uint32_t)nm);
        }
    }
    t.mats.assign(nm, 0.0);
    t.areas.assign(na, 0.0);
    if (m.n_cells == 0) return;
    stencil_matrix(t, m, 0, 0, true, &t.areas[ao[0]], &t.mats[mo[0]]);
    std::string err;
#pragma omp parallel for schedule(dynamic, 256) if (g_threads > 1) num_threads(g_threads)
    for (int64_t ci = 0; ci < (int64_t)m.n_cells; ++ci) {
        try {
            const uint32_t c = (uint32_t)ci;
            const uint32_t g0 = t.off_groups[c];
            for (uint32_t s = g0; s < t.off_groups[c + 1]; ++s) {
                if (t.off_stencils[s + 1] == t.off_stencils[s] || (c == 0 && s == g0)) continue;
                stencil_matrix(t, m, c, (int)(s - g0), false, &t.areas[ao[s]], &t.mats[mo[s]]);
            }
        } catch (const std::exception& e) {
#pragma omp critical
            err = e.what();
        }
    }
    if (!err.empty()) throw std::runtime_error(err);
}

// TENO::compute_oscillation_indicator (face_reconstruction.cpp:743-788)
void teno_oscillation(Teno& t) {
    const int K = t.K, nq = t.qcell.n();
    t.oi.assign((size_t)K * K, 0.0);
    for (int i = 0; i < K; i++)
        for (int j = 0; j < K; j++) {
            double acc = 0.0;
            for (int k = 1; k < K; k++)
                for (int q = 0; q < nq; ++q) {
                    double di = 1.0, dj = 1.0;
                    for (int d = 0; d < 2; d++) di *= basis1_d(t.basis, t.pidx[2 * k + d], t.pidx[2 * i + d], t.qcell.pts[2 * q + d]);
                    for (int d = 0; d < 2; d++) dj *= basis1_d(t.basis, t.pidx[2 * k + d], t.pidx[2 * j + d], t.qcell.pts[2 * q + d]);
                    acc += t.qcell.wts[q] * di * dj;
                }
            t.oi[(size_t)i * K + j] = acc;
        }
}

// ---------------------------------------------------------------------------
// Physics and Riemann solvers -- restates src/physics/physics.h,
// src/physics/physics.cpp and src/numerics/riemann_solver.h
// ---------------------------------------------------------------------------

struct Gas {
    double gamma = 1.4, p_ref = 101325.0, T_ref = 298.15, rho_ref = 1.225, p_min = -1e20, p_max = 1e20;
    double R = 0, cp = 0, cv = 0;
    // Euler::set_R_cp_cv (physics.cpp:69-73)
    void derive() {
        R = p_ref / (T_ref * rho_ref);
        cp = R * gamma / (gamma - 1.0);
        cv = cp / gamma;
    }
    // Euler::compute_primitives_from_conservatives_impl (physics.h:852-867)
    void prims(const double* U, double* W) const {
        double rho = U[0];
        double u0 = U[1] / rho, u1 = U[2] / rho;
        double E = U[3] / rho;
        double e = E - 0.5 * (u0 * u0 + u1 * u1);
        double p = std::fmax(p_min, std::fmin(p_max, (gamma - 1.0) * rho * e));
        double T = e / cv;
        double h = e + p / rho;
        W[0] = u0; W[1] = u1; W[2] = p; W[3] = T; W[4] = h;
    }
    double sos(double p, double rho) const { return std::sqrt(gamma * p / rho); }
};

enum { RS_RUSANOV = 0, RS_HLL = 1, RS_HLLC = 2 };

// PVRS, average form (riemann_solver.h:205-240)
void star_pvrs(const double* L, const double* R, double& ps, double& rls, double& rrs) {
    double al = std::sqrt(L[3] * L[2] / L[0]);
    double ar = std::sqrt(R[3] * R[2] / R[0]);
    double rho_m = 0.5 * (L[0] + R[0]);
    double a_m = 0.5 * (al + ar);
    double us = 0.5 * (L[1] + R[1]) + 0.5 * (L[2] - R[2]) / (rho_m * a_m);
    ps = 0.5 * (L[2] + R[2]) + 0.5 * (L[1] - R[1]) * rho_m * a_m;
    rls = L[0] + (L[1] - us) * rho_m / a_m;
    rrs = R[0] - (R[1] - us) * rho_m / a_m;
}

// TRRS (riemann_solver.h:242-271)
void star_trrs(const double* L, const double* R, double& ps, double& rls, double& rrs) {
    double al = std::sqrt(L[3] * L[2] / L[0]);
    double ar = std::sqrt(R[3] * R[2] / R[0]);
    double zl = (L[3] - 1.0) / (2.0 * L[3]);
    double zr = (R[3] - 1.0) / (2.0 * R[3]);
    double plr = std::pow((L[2] / R[2]), zl);
    double us = (plr * L[1] / al + R[1] / ar + 2.0 * (1.0 - plr) / (L[3] - 1.0)) / (plr / al + 1.0 / ar);
    ps = 0.5 * (L[2] * std::pow((1.0 + (L[3] - 1.0) / (2.0 * al) * (L[1] - us)), (1.0 / zl)) +
                R[2] * std::pow((1.0 + (R[3] - 1.0) / (2.0 * ar) * (us - R[1])), (1.0 / zr)));
    rls = L[0] * std::pow(ps / L[2], 1.0 / L[3]);
    rrs = R[0] * std::pow(ps / R[2], 1.0 / R[3]);
}

// TSRS (riemann_solver.h:273-306); p_star enters holding the PVRS estimate.
void star_tsrs(const double* L, const double* R, double& ps, double& rls, double& rrs) {
    double gl = (L[3] - 1.0) / (L[3] + 1.0);
    double gr = (R[3] - 1.0) / (R[3] + 1.0);
    double Al = 2.0 / (L[3] + 1.0) / L[0], Bl = gl * L[2];
    double Ar = 2.0 / (R[3] + 1.0) / R[0], Br = gr * R[2];
    double p0 = std::fmax(0.0, ps);
    double ql = std::sqrt(Al / (p0 + Bl));
    double qr = std::sqrt(Ar / (p0 + Br));
    ps = (ql * L[2] + qr * R[2] - (R[1] - L[1])) / (ql + qr);
    rls = L[0] * (ps / L[2] + gl) / (gl * ps / L[2] + 1.0);
    rrs = R[0] * (ps / R[2] + gr) / (gr * ps / R[2] + 1.0);
}

// ANRS (riemann_solver.h:308-329)
void star_anrs(const double* L, const double* R, double& ps, double& rls, double& rrs) {
    double pmax = std::fmax(L[2], R[2]), pmin = std::fmin(L[2], R[2]);
    double qmax = pmax / pmin;
    star_pvrs(L, R, ps, rls, rrs);
    if ((qmax < 2.0) && (pmin <= ps) && (ps <= pmax)) return;
    if (ps < pmin) star_trrs(L, R, ps, rls, rrs);
    else star_tsrs(L, R, ps, rls, rrs);
}

// Rusanov / HLL / HLLC ::calc_flux (riemann_solver.h:331-519).
// guard (the robust TENO variant): a star pressure that is not a number
// counts as zero.  The reference's two-rarefaction estimate raises a
// negative base to the power 2 gamma / (gamma - 1), which is not an exact
// integer in floating point, when a strong expansion meets a near-vacuum
// pressure; its NaN then reaches the wave speeds and the flux.  A zero star
// pressure gives the same wave speeds as any star pressure below both
// pressures, so the guard changes no flux that the reference computes as a
// number.
void riemann(int kind, double* F, const double* n, double rl, const double* ul, double pl, double gl, double hl,
             double rr, const double* ur, double pr, double gr, double hr, bool guard = false) {
    double unl = ul[0] * n[0] + ul[1] * n[1];
    double unr = ur[0] * n[0] + ur[1] * n[1];
    double qql = ul[0] * ul[0] + ul[1] * ul[1];
    double qqr = ur[0] * ur[0] + ur[1] * ur[1];
    double al = std::sqrt(gl * pl / rl);
    double ar = std::sqrt(gr * pr / rr);
    double El = (hl + 0.5 * qql) * rl - pl;
    double Er = (hr + 0.5 * qqr) * rr - pr;
    double Ul[4] = {rl, rl * ul[0], rl * ul[1], El};
    double Ur[4] = {rr, rr * ur[0], rr * ur[1], Er};
    double Fl[4] = {rl * unl, rl * ul[0] * unl + pl * n[0], rl * ul[1] * unl + pl * n[1], (El + pl) * unl};
    double Fr[4] = {rr * unr, rr * ur[0] * unr + pr * n[0], rr * ur[1] * unr + pr * n[1], (Er + pr) * unr};
    if (kind == RS_RUSANOV) {
        double smax = std::fmax(std::fabs(unl) + al, std::fabs(unr) + ar);
        for (int i = 0; i < 4; i++) F[i] = 0.5 * (Fl[i] + Fr[i] + smax * (Ul[i] - Ur[i]));
        return;
    }
    double Wl[4] = {rl, unl, pl, gl}, Wr[4] = {rr, unr, pr, gr};
    double ps, rls, rrs;
    star_anrs(Wl, Wr, ps, rls, rrs);
    if (guard && !(ps == ps)) ps = 0.0;
    double ql = (ps <= pl) ? 1.0 : std::sqrt(1.0 + (gl + 1.0) / (2.0 * gl) * (ps / pl - 1.0));
    double qr = (ps <= pr) ? 1.0 : std::sqrt(1.0 + (gr + 1.0) / (2.0 * gr) * (ps / pr - 1.0));
    double Sl = unl - al * ql;
    double Sr = unr + ar * qr;
    if (kind == RS_HLL) {
        if (0.0 <= Sl) for (int i = 0; i < 4; i++) F[i] = Fl[i];
        else if (Sr <= 0.0) for (int i = 0; i < 4; i++) F[i] = Fr[i];
        else for (int i = 0; i < 4; i++) F[i] = (Sr * Fl[i] - Sl * Fr[i] + Sl * Sr * (Ur[i] - Ul[i])) / (Sr - Sl);
        return;
    }
    double Ss = (pr - pl + rl * unl * (Sl - unl) - rr * unr * (Sr - unr)) / (rl * (Sl - unl) - rr * (Sr - unr));
    if (0.0 <= Sl) {
        for (int i = 0; i < 4; i++) F[i] = Fl[i];
    } else if (Sr <= 0.0) {
        for (int i = 0; i < 4; i++) F[i] = Fr[i];
    } else {
        double D[4] = {0.0, n[0], n[1], Ss};
        double Plr = 0.5 * (pl + pr + rl * (Sl - unl) * (Ss - unl) + rr * (Sr - unr) * (Ss - unr));
        if (Ss >= 0.0) for (int i = 0; i < 4; i++) F[i] = (Ss * (Sl * Ul[i] - Fl[i]) + Sl * Plr * D[i]) / (Sl - Ss);
        else for (int i = 0; i < 4; i++) F[i] = (Ss * (Sr * Ur[i] - Fr[i]) + Sr * Plr * D[i]) / (Sr - Ss);
    }
}

// unit<2> (common_math.h:101-106)
inline void unit2(const double* v, double* u) {
    double inv = 1 / std::sqrt(v[0] * v[0] + v[1] * v[1]);
    u[0] = v[0] * inv;
    u[1] = v[1] * inv;
}

// ---------------------------------------------------------------------------
// Boundary conditions -- restates src/boundary/boundary_*.cpp
// ---------------------------------------------------------------------------

enum { BC_SYMMETRY = 0, BC_EXTRAPOLATION = 1, BC_WALL_ADIABATIC = 2, BC_UPT = 3, BC_P_OUT = 4 };

struct Bc {
    uint32_t zone;
    int type;
    double data[6] = {0, 0, 0, 0, 0, 0};
};

// ---------------------------------------------------------------------------
// The case: one mesh + numerics + state, with the Solver's hot-path methods
// ---------------------------------------------------------------------------

enum { RECON_FO = 0, RECON_TENO = 1 };

struct Case {
    const OMesh* mesh = nullptr;
    Gas gas;
    int recon = RECON_TENO;
    int rsolver = RS_HLLC;
    Teno teno;
    Rule qface;
    int nq = 1;
    // 0: the reference's TENO weighting (face_reconstruction.cpp:947-981),
    //    including its directional-branch quirks.
    // 1: corrected: in the directional branch the central stencil and the
    //    directional stencils that fail CT2 get weight 0 and the passing ones
    //    share equal weight (the cut-off the reference's comments describe),
    //    and the polynomial is evaluated in the zero-mean basis
    //    psi_k(x) - mean(psi_k) that the least-squares tables were built in.
    //    Same decisions and same work per cell as variant 0.  The face flux
    //    then replaces a reconstructed face state whose density or pressure
    //    is not positive by the owning cell's average (first-order fallback).
    // 2: robust: variant 1, then per cell (robust_cell below):
    //    a cell with a boundary face takes its average at all its face
    //    points; otherwise each variable's polynomial is scaled toward the
    //    cell average so that its face values stay within the range of the
    //    cell's central stencil, and if a face state is still not admissible
    //    the cell takes its average at all its face points.  HLL/HLLC count a
    //    star pressure that is not a number as zero (riemann, guard).
    int teno_variant = 0;
    int integrator = 0;  // 0 SSPRK3, 1 FE, 2 RK4 (time_integrator.h)
    std::vector<Bc> bcs;
    std::vector<double> U, Utmp, prim, face, r1, r2, r3, r4, cfl_local;
    // viscous face flux (no reference counterpart; restated from the GPU
    // library's definition): Sutherland viscosity; cell gradients from the
    // reconstructed polynomials (visc_grad 0, with TENO) or Green-Gauss
    bool viscous = false;
    int visc_grad = 0;
    double mu_ref = 0.0, T_mu_ref = 1.0, sutherland_S = 0.0, cp_over_pr = 0.0;
    std::vector<double> grad;       // [n_cells][6]
    std::vector<double> cgrad;      // [n_cells][4][2]: conserved variables' polynomial gradients
    std::vector<signed char> wall;  // per face: 1 on a wall_adiabatic zone
    // diagnostics: TENO decision per [cell][var]: bit0 central, bit s = stencil s passed CT2
    std::vector<uint8_t> masks;
};

// FirstOrderFunctor (face_reconstruction.cpp:59-99), interior+boundary faces
// (the reference also loops over phantom faces; their values are never read).
void recon_fo(Case& cs, const double* U, double* face) {
    const OMesh& m = *cs.mesh;
#pragma omp parallel for if (g_threads > 1) num_threads(g_threads)
    for (int64_t f = 0; f < (int64_t)m.n_faces; ++f) {
        int32_t l = m.cof[2 * f], r = m.cof[2 * f + 1];
        for (int v = 0; v < NC; v++) {
            face[((size_t)f * 1 + 0) * 2 * NC + 0 * NC + v] = U[(size_t)l * NC + v];
            face[((size_t)f * 1 + 0) * 2 * NC + 1 * NC + v] = r >= 0 ? U[(size_t)r * NC + v] : 0.0;
        }
    }
}

bool admissible(const Gas& g, const double* W);

// The robust variant's per-cell step after the TENO face values of all four
// variables are known (no reference counterpart):
//  1. a cell with a boundary face takes its average at every face point
//     (its one-sided stencils, extrapolated onto transmissive boundaries,
//     let a boundary mode grow);
//  2. otherwise, per variable, the face-point deviations from the average
//     d_p = w_p - u are scaled by one theta = min over the points of
//     dhi / d_p (d_p > dhi) or dlo / d_p (d_p < dlo), where [dlo, dhi] is
//     the range of the central stencil's averages minus u;
//  3. if a face state is then not admissible (density positive and
//     2 rho E > |rho u|^2, i.e. pressure positive), the cell takes its
//     average at every face point.
// Admissible face state for the robust variant's fallback: density
// positive and 2 rho E > |rho u|^2, which for rho > 0 is pressure positive
// (gamma > 1), without divisions.
inline bool robust_admissible(const double* W) {
    const double m2 = W[1] * W[1] + W[2] * W[2];
    return W[0] > 0.0 && 2.0 * W[0] * W[3] > m2;
}

// keep[v]: the factor variable v's polynomial was scaled by (1 kept, 0
// replaced by the average).
void robust_cell(Case& cs, uint32_t c, const double* U, double* face, const double* dlo, const double* dhi,
                 double* keep) {
    const OMesh& m = *cs.mesh;
    const int nq = cs.nq;
    const uint32_t fo = m.off_foc[c];
    const int nf = (int)(m.off_foc[c + 1] - fo);
    auto at = [&](int fl, int q) -> double* {
        const uint32_t f = m.foc[fo + fl];
        const int side = m.cof[2 * (size_t)f] == (int32_t)c ? 0 : 1;
        return &face[(((size_t)f * nq + q) * 2 + side) * NC];
    };
    bool first_order = false;
    for (int fl = 0; fl < nf; fl++)
        if (m.cof[2 * (size_t)m.foc[fo + fl] + 1] < 0) first_order = true;
    for (int v = 0; v < NC; ++v) keep[v] = 1.0;
    if (!first_order) {
        for (int v = 0; v < NC; ++v) {
            const double u = U[(size_t)c * NC + v];
            double th = 1.0;
            for (int fl = 0; fl < nf; fl++)
                for (int q = 0; q < nq; q++) {
                    const double d = at(fl, q)[v] - u;
                    if (d > dhi[v]) th = std::fmin(th, dhi[v] / d);
                    else if (d < dlo[v]) th = std::fmin(th, dlo[v] / d);
                }
            if (th < 1.0)
                for (int fl = 0; fl < nf; fl++)
                    for (int q = 0; q < nq; q++) {
                        double& w = at(fl, q)[v];
                        w = u + th * (w - u);
                    }
            keep[v] = th;
        }
        for (int fl = 0; fl < nf && !first_order; fl++)
            for (int q = 0; q < nq; q++)
                if (!robust_admissible(at(fl, q))) {
                    first_order = true;
                    break;
                }
    }
    if (first_order) {
        for (int fl = 0; fl < nf; fl++)
            for (int q = 0; q < nq; q++)
                for (int v = 0; v < NC; ++v) at(fl, q)[v] = U[(size_t)c * NC + v];
        for (int v = 0; v < NC; ++v) keep[v] = 0.0;
    }
}

// Derivative of a 1D basis function for the polynomials' gradients: the
// Legendre derivatives of basis.h, and p x^(p-1) for the monomial basis
// (not the (p+1) factor the oscillation indicator's derivative carries).
inline double grad1(int type, int p, double x) {
    if (type == BASIS_LEGENDRE) return legendre_d(1, p, x);
    return p == 0 ? 0.0 : (double)p * std::pow(x, (double)(p - 1));
}

// TENOFunctor::operator() (face_reconstruction.cpp:866-1039)
void recon_teno_cell(Case& cs, uint32_t c, const double* U, double* face) {
    const OMesh& m = *cs.mesh;
    const Teno& t = cs.teno;
    const int K = t.K, nq = cs.nq;
    uint32_t fo = m.off_foc[c];
    int nf = (int)(m.off_foc[c + 1] - fo);
    uint32_t g0 = t.off_groups[c];
    int gs = (int)(t.off_groups[c + 1] - g0);
    std::vector<double> sw((size_t)gs * NC), dw((size_t)gs * K * NC);
    // range of the central stencil around the cell average, per variable
    // (the robust variant's bounds; the target cell itself gives 0)
    double dlo[NC] = {0.0, 0.0, 0.0, 0.0}, dhi[NC] = {0.0, 0.0, 0.0, 0.0};
    const double* w0 = m.nc(m.node_of_cell(c, 0));
    double J[4], Ji[4];
    tri_jac(w0, m.nc(m.node_of_cell(c, 1)), m.nc(m.node_of_cell(c, 2)), J);
    inv2(J, Ji);
    for (int sl = 0; sl < gs; ++sl) {
        uint32_t s = g0 + sl;
        uint32_t so = t.off_stencils[s];
        int M = (int)(t.off_stencils[s + 1] - so);
        uint32_t mo = t.off_mats[s];
        if (M == 0) {
            for (int v = 0; v < NC; v++) sw[(size_t)sl * NC + v] = 0.0;
            continue;
        }
        std::vector<double> b((size_t)M * NC);
        for (int j = 0; j < M; ++j) {
            uint32_t nb = t.stencils[so + j];
            for (int v = 0; v < NC; ++v) {
                const double d = U[(size_t)nb * NC + v] - U[(size_t)c * NC + v];
                b[(size_t)j * NC + v] = t.areas[so + j] * d;
                if (sl == 0) {
                    dlo[v] = std::fmin(dlo[v], d);
                    dhi[v] = std::fmax(dhi[v], d);
                }
            }
        }
        double* a = &dw[(size_t)sl * K * NC];
        mm(&t.mats[mo], b.data(), a, K, M, NC);
        std::vector<double> oia((size_t)K * NC);
        mm(t.oi.data(), a, oia.data(), K, K, NC);
        for (int v = 0; v < NC; ++v) {
            double si = 0.0;
            for (int k = 0; k < K; ++k) si += a[(size_t)k * NC + v] * oia[(size_t)k * NC + v];
            sw[(size_t)sl * NC + v] = 1.0 / std::pow(si + 1.0e-12, 6.0);
        }
    }
    for (int v = 0; v < NC; ++v) {
        uint8_t mask = 0;
        double sd = 0.0;
        for (int sl = 1; sl < gs; ++sl) sd += sw[(size_t)sl * NC + v];
        if (sw[v] / (sd + sw[v]) > 1.0e-7) {
            sw[v] = 1.0;
            for (int sl = 1; sl < gs; ++sl) sw[(size_t)sl * NC + v] = 0.0;
            mask = 1;
        } else {
            for (int sl = 1; sl < gs; ++sl)
                if (sw[(size_t)sl * NC + v] / sd > 1.0e-5) {
                    sw[(size_t)sl * NC + v] = (1.0 / K);
                    mask |= (uint8_t)(1u << sl);
                }
            if (cs.teno_variant >= 1) {
                sw[v] = 0.0;
                for (int sl = 1; sl < gs; ++sl)
                    if (!(mask & (1u << sl))) sw[(size_t)sl * NC + v] = 0.0;
            }
            sd = 0.0;
            for (int sl = 1; sl < gs; ++sl) sd += sw[(size_t)sl * NC + v];
            for (int sl = 1; sl < gs; ++sl) sw[(size_t)sl * NC + v] /= sd;
        }
        if (!cs.masks.empty()) cs.masks[(size_t)c * NC + v] = mask;
        if (!cs.cgrad.empty()) {
            // the polynomial's gradient at the centroid (1/3, 1/3) of the
            // reference frame, then x = Ji^T: summed in the face values' order
            double g0 = 0.0, g1 = 0.0;
            const double x = 1.0 / 3.0;
            for (int sl = 0; sl < gs; sl++) {
                if (sw[(size_t)sl * NC + v] == 0.0) continue;
                for (int k = 1; k < K; k++) {
                    const int px = t.pidx[2 * k], py = t.pidx[2 * k + 1];
                    const double d0 = grad1(t.basis, px, x) * basis1(t.basis, py, x);
                    const double d1 = basis1(t.basis, px, x) * grad1(t.basis, py, x);
                    const double ck = sw[(size_t)sl * NC + v] * dw[(size_t)sl * K * NC + (size_t)k * NC + v];
                    g0 = g0 + ck * d0;
                    g1 = g1 + ck * d1;
                }
            }
            cs.cgrad[((size_t)c * NC + v) * 2] = Ji[0] * g0 + Ji[2] * g1;
            cs.cgrad[((size_t)c * NC + v) * 2 + 1] = Ji[1] * g0 + Ji[3] * g1;
        }
        for (int fl = 0; fl < nf; fl++) {
            uint32_t f = m.foc[fo + fl];
            int side = m.cof[2 * (size_t)f] == (int32_t)c ? 0 : 1;
            double x0[2], x1[2];
            const double* n0 = m.nc(m.node_of_face(f, 0));
            const double* n1 = m.nc(m.node_of_face(f, 1));
            for (int i = 0; i < 2; i++) { x0[i] = n0[i] - w0[i]; x1[i] = n1[i] - w0[i]; }
            mv2(Ji, x0, x0);
            mv2(Ji, x1, x1);
            for (int q = 0; q < nq; q++) {
                double& out = face[(((size_t)f * nq + q) * 2 + side) * NC + v];
                out = U[(size_t)c * NC + v];
                double xq[2];
                for (int i = 0; i < 2; i++) xq[i] = (cs.qface.pts[q] + 1.0) * 0.5 * (x1[i] - x0[i]) + x0[i];
                for (int sl = 0; sl < gs; sl++) {
                    if (sw[(size_t)sl * NC + v] == 0.0) continue;
                    uint32_t so = t.off_stencils[g0 + sl];
                    for (int k = 0; k < K; k++) {
                        double phi = basis2(t.basis, t.pidx[2 * k], t.pidx[2 * k + 1], xq[0], xq[1]);
                        double shape = cs.teno_variant >= 1 ? phi - t.ipt[k] : phi + (t.ipt[k] / t.areas[so]);
                        out += sw[(size_t)sl * NC + v] * dw[(size_t)sl * K * NC + (size_t)k * NC + v] * shape;
                    }
                }
            }
        }
    }
    if (cs.teno_variant == 2) {
        double keep[NC];
        robust_cell(cs, c, U, face, dlo, dhi, keep);
        if (!cs.cgrad.empty())
            for (int v = 0; v < NC; ++v) {
                double* g = &cs.cgrad[((size_t)c * NC + v) * 2];
                if (keep[v] == 0.0) {
                    g[0] = 0.0;
                    g[1] = 0.0;
                } else if (keep[v] < 1.0) {
                    g[0] = keep[v] * g[0];
                    g[1] = keep[v] * g[1];
                }
            }
    }
}

void recon(Case& cs, const double* U, double* face) {
    if (cs.recon == RECON_FO) {
        recon_fo(cs, U, face);
        return;
    }
    const OMesh& m = *cs.mesh;
    if (cs.viscous && cs.visc_grad == 0) cs.cgrad.assign((size_t)m.n_cells * NC * 2, 0.0);
    else cs.cgrad.clear();
#pragma omp parallel for schedule(dynamic, 64) if (g_threads > 1) num_threads(g_threads)
    for (int64_t c = 0; c < (int64_t)m.n_cells; ++c) recon_teno_cell(cs, (uint32_t)c, U, face);
}

inline void scatter_add(double* dst, double val) {
    if (g_threads > 1) {
#pragma omp atomic
        *dst += val;
    } else {
        *dst += val;
    }
}

// Left/right states of one face quadrature point: InteriorFluxFunctor and the
// boundary functors' calc_lr_states_impl (flux_functor.h:164-178,
// boundary_symmetry.cpp:38-69, boundary_extrapolation.cpp:38-55,
// boundary_upt.cpp:83-100, boundary_p_out.cpp:57-100).
void lr_states(const Case& cs, int bc, const Bc* b, const double* face_q, const double* n_unit, double* cl, double* cr,
               double* pl, double* pr) {
    const Gas& g = cs.gas;
    for (int i = 0; i < NC; i++) cl[i] = face_q[i];
    if (bc < 0) {
        for (int i = 0; i < NC; i++) cr[i] = face_q[NC + i];
        g.prims(cl, pl);
        g.prims(cr, pr);
        return;
    }
    g.prims(cl, pl);
    switch (bc) {
        case BC_SYMMETRY: {
            for (int i = 0; i < NC; i++) cr[i] = cl[i];
            for (int i = 0; i < NP; i++) pr[i] = pl[i];
            double un = pl[0] * n_unit[0] + pl[1] * n_unit[1];
            pr[0] = pl[0] - 2.0 * un * n_unit[0];
            pr[1] = pl[1] - 2.0 * un * n_unit[1];
            break;
        }
        case BC_EXTRAPOLATION:
            for (int i = 0; i < NC; i++) cr[i] = cl[i];
            for (int i = 0; i < NP; i++) pr[i] = pl[i];
            break;
        case BC_UPT:
            cr[0] = b->data[0];
            for (int i = 0; i < NP; i++) pr[i] = b->data[i + 1];
            break;
        case BC_P_OUT: {
            double rho_l = cl[0];
            double um = std::sqrt(pl[0] * pl[0] + pl[1] * pl[1]);
            double a = g.sos(pl[2], rho_l);
            double po = (um < a) ? b->data[0] : pl[2];
            double T = pl[3];
            double rho = po / (g.R * T);
            double e = g.cv * T;
            double h = e + po / rho;
            cr[0] = rho;
            pr[0] = pl[0];
            pr[1] = pl[1];
            pr[2] = po;
            pr[3] = T;
            pr[4] = h;
            break;
        }
        default: break;
    }
}

// BaseFluxFunctor::call_impl (flux_functor.h:124-162) and
// WallAdiabaticFluxFunctor::call_impl (boundary_wall_adiabatic.cpp:38-70).
// Positivity fallback of the corrected TENO variant: a face state whose
// density or pressure is not positive reverts to the cell average.
bool admissible(const Gas& g, const double* W) {
    double rho = W[0];
    if (!(rho > 0.0)) return false;
    double u0 = W[1] / rho, u1 = W[2] / rho;
    double e = W[3] / rho - 0.5 * (u0 * u0 + u1 * u1);
    return (g.gamma - 1.0) * rho * e > 0.0;
}

// ---------------------------------------------------------------------------
// Viscous face flux (no counterpart in the reference)
// ---------------------------------------------------------------------------

inline void uvT(const Gas& g, const double* U, double* q) {
    double rho = U[0];
    double u = U[1] / rho, v = U[2] / rho;
    double E = U[3] / rho;
    double e = E - 0.5 * (u * u + v * v);
    q[0] = u;
    q[1] = v;
    q[2] = e / g.cv;
}

// Green-Gauss gradients of (u, v, T) per cell: (1/V) sum_f phi_f n_out A,
// phi_f the mean of the two cells, u = v = 0 and T = T_c on a wall, phi_c on
// other boundaries.
void viscous_gradients(Case& cs, const double* U) {
    const OMesh& m = *cs.mesh;
    cs.grad.assign((size_t)m.n_cells * 6, 0.0);
    if (cs.recon == RECON_TENO && cs.visc_grad == 0) {
        // from the polynomials' gradients of the conserved variables and the
        // cell averages: u = m0 / rho, v = m1 / rho, e = E - (u^2 + v^2) / 2,
        // T = e / cv, by the quotient rule
        for (uint32_t c = 0; c < m.n_cells; ++c) {
            const double* r = U + (size_t)c * NC;
            const double* g = &cs.cgrad[(size_t)c * NC * 2];
            const double rho = r[0];
            const double u = r[1] / rho, w = r[2] / rho, E = r[3] / rho;
            const double ux = (g[2] - u * g[0]) / rho, uy = (g[3] - u * g[1]) / rho;
            const double vx = (g[4] - w * g[0]) / rho, vy = (g[5] - w * g[1]) / rho;
            const double ex = (g[6] - E * g[0]) / rho - (u * ux + w * vx);
            const double ey = (g[7] - E * g[1]) / rho - (u * uy + w * vy);
            double* o = &cs.grad[(size_t)c * 6];
            o[0] = ux;
            o[1] = uy;
            o[2] = vx;
            o[3] = vy;
            o[4] = ex / cs.gas.cv;
            o[5] = ey / cs.gas.cv;
        }
        return;
    }
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        double qc[3], gx[3] = {0, 0, 0}, gy[3] = {0, 0, 0};
        uvT(cs.gas, U + (size_t)c * NC, qc);
        for (uint32_t k = m.off_foc[c]; k < m.off_foc[c + 1]; ++k) {
            uint32_t f = m.foc[k];
            int32_t L = m.cof[2 * (size_t)f], R = m.cof[2 * (size_t)f + 1];
            double n[2];
            unit2(&m.face_normals[2 * (size_t)f], n);
            double A = m.face_area[f];
            double sg = L == (int32_t)c ? 1.0 : -1.0;
            double nx = sg * n[0], ny = sg * n[1];
            double qf[3];
            if (R >= 0) {
                double qo[3];
                uvT(cs.gas, U + (size_t)(L == (int32_t)c ? R : L) * NC, qo);
                for (int i = 0; i < 3; ++i) qf[i] = 0.5 * (qc[i] + qo[i]);
            } else {
                bool w = cs.wall[f] != 0;
                qf[0] = w ? 0.0 : qc[0];
                qf[1] = w ? 0.0 : qc[1];
                qf[2] = qc[2];
            }
            for (int i = 0; i < 3; ++i) {
                gx[i] = gx[i] + qf[i] * nx * A;
                gy[i] = gy[i] + qf[i] * ny * A;
            }
        }
        for (int i = 0; i < 3; ++i) {
            cs.grad[(size_t)c * 6 + 2 * i] = gx[i] / m.cell_volume[c];
            cs.grad[(size_t)c * 6 + 2 * i + 1] = gy[i] / m.cell_volume[c];
        }
    }
}

// Navier-Stokes flux through face f (unit normal n out of its first cell):
// mean gradient corrected by the jump along the centre-to-centre line;
// on a no-slip adiabatic wall the cell's gradient corrected to velocity 0,
// with no heat flux and no work.
void viscous_flux(const Case& cs, uint32_t f, bool wall, const double* U, const double* n, double* Fv) {
    const OMesh& m = *cs.mesh;
    int32_t L = m.cof[2 * (size_t)f], R = m.cof[2 * (size_t)f + 1];
    double qL[3], qR[3], gf[6], dx, dy;
    uvT(cs.gas, U + (size_t)L * NC, qL);
    const double* gL = &cs.grad[(size_t)L * 6];
    const double* xL = m.cc(L);
    if (R >= 0) {
        uvT(cs.gas, U + (size_t)R * NC, qR);
        const double* gR = &cs.grad[(size_t)R * 6];
        for (int i = 0; i < 6; ++i) gf[i] = 0.5 * (gL[i] + gR[i]);
        const double* xR = m.cc(R);
        dx = xR[0] - xL[0];
        dy = xR[1] - xL[1];
    } else {
        qR[0] = 0.0;
        qR[1] = 0.0;
        qR[2] = qL[2];
        for (int i = 0; i < 6; ++i) gf[i] = gL[i];
        const double* p0 = m.nc(m.node_of_face(f, 0));
        const double* p1 = m.nc(m.node_of_face(f, 1));
        dx = 0.5 * (p0[0] + p1[0]) - xL[0];
        dy = 0.5 * (p0[1] + p1[1]) - xL[1];
    }
    double dl = std::sqrt(dx * dx + dy * dy);
    double tx = dx / dl, ty = dy / dl;
    for (int k = 0; k < 3; ++k) {
        double corr = (qR[k] - qL[k]) / dl - (gf[2 * k] * tx + gf[2 * k + 1] * ty);
        gf[2 * k] = gf[2 * k] + corr * tx;
        gf[2 * k + 1] = gf[2 * k + 1] + corr * ty;
    }
    double u = 0.5 * (qL[0] + qR[0]), v = 0.5 * (qL[1] + qR[1]), T = 0.5 * (qL[2] + qR[2]);
    double mu = cs.mu_ref;
    if (cs.sutherland_S > 0.0) {
        double r = T / cs.T_mu_ref;
        mu = cs.mu_ref * (r * std::sqrt(r)) * ((cs.T_mu_ref + cs.sutherland_S) / (T + cs.sutherland_S));
    }
    double k = mu * cs.cp_over_pr;
    double ux = gf[0], uy = gf[1], vx = gf[2], vy = gf[3], Tx = gf[4], Ty = gf[5];
    double div = ux + vy;
    double txx = mu * (2.0 * ux - 2.0 / 3.0 * div);
    double tyy = mu * (2.0 * vy - 2.0 / 3.0 * div);
    double txy = mu * (uy + vx);
    Fv[0] = 0.0;
    Fv[1] = txx * n[0] + txy * n[1];
    Fv[2] = txy * n[0] + tyy * n[1];
    Fv[3] = wall ? 0.0 : (u * txx + v * txy + k * Tx) * n[0] + (u * txy + v * tyy + k * Ty) * n[1];
}

void face_flux(Case& cs, uint32_t f, int bc, const Bc* b, const double* U, const double* face, double* rhs) {
    const OMesh& m = *cs.mesh;
    double F[4] = {0, 0, 0, 0}, Ft[4], cl[4], cr[4], pl[5], pr[5], n[2];
    unit2(&m.face_normals[2 * (size_t)f], n);
    for (int q = 0; q < cs.nq; q++) {
        const double* fq = &face[((size_t)f * cs.nq + q) * 2 * NC];
        double fix[2 * NC];
        if (cs.recon == RECON_TENO && cs.teno_variant >= 1) {
            for (int i = 0; i < 2 * NC; i++) fix[i] = fq[i];
            for (int sd = 0; sd < 2; sd++) {
                int32_t c = m.cof[2 * (size_t)f + sd];
                if (c < 0 || (sd == 1 && bc >= 0)) continue;
                if (!admissible(cs.gas, fix + sd * NC))
                    for (int i = 0; i < NC; i++) fix[sd * NC + i] = U[(size_t)c * NC + i];
            }
            fq = fix;
        }
        if (bc == BC_WALL_ADIABATIC) {
            for (int i = 0; i < NC; i++) cl[i] = fq[i];
            cs.gas.prims(cl, pl);
            Ft[0] = 0.0;
            Ft[1] = pl[2] * n[0];
            Ft[2] = pl[2] * n[1];
            Ft[3] = 0.0;
        } else {
            lr_states(cs, bc, b, fq, n, cl, cr, pl, pr);
            riemann(cs.rsolver, Ft, n, cl[0], pl, pl[2], cs.gas.gamma, pl[4], cr[0], pr, pr[2], cs.gas.gamma, pr[4],
                    cs.teno_variant == 2);
        }
        for (int i = 0; i < NC; i++) F[i] += cs.qface.wts[q] * Ft[i];
    }
    for (int i = 0; i < NC; i++) F[i] *= 0.5;
    int32_t L = m.cof[2 * (size_t)f], R = m.cof[2 * (size_t)f + 1];
    double Fv[4] = {0.0, 0.0, 0.0, 0.0};
    const bool visc = cs.viscous && (bc < 0 || bc == BC_WALL_ADIABATIC);
    if (visc) viscous_flux(cs, f, bc == BC_WALL_ADIABATIC, U, n, Fv);
    for (int i = 0; i < NC; i++) {
        double g = m.face_area[f] * F[i];
        if (visc && i > 0) g = g - m.face_area[f] * Fv[i];
        scatter_add(&rhs[(size_t)L * NC + i], -g);
        if (bc < 0 && R >= 0) scatter_add(&rhs[(size_t)R * NC + i], g);
    }
}

// Faces of the no-slip adiabatic walls, for the viscous flux.
void mark_walls(Case& cs) {
    const OMesh& m = *cs.mesh;
    cs.wall.assign(m.n_faces, 0);
    for (const Bc& b : cs.bcs)
        if (b.type == BC_WALL_ADIABATIC)
            for (uint32_t k = m.zone_off[b.zone]; k < m.zone_off[b.zone + 1]; ++k) cs.wall[m.zone_faces[k]] = 1;
}

// Solver::calc_rhs (solver_rhs.cpp:44-115)
void calc_rhs(Case& cs, const double* U, double* face, double* rhs) {
    const OMesh& m = *cs.mesh;
    for (size_t i = 0; i < (size_t)m.n_cells * NC; i++) rhs[i] = 0.0;
    recon(cs, U, face);
    if (cs.viscous) {
        mark_walls(cs);
        viscous_gradients(cs, U);
    }
    uint32_t z0 = m.zone_off[0], z1 = m.zone_off[1];
#pragma omp parallel for if (g_threads > 1) num_threads(g_threads)
    for (int64_t k = z0; k < (int64_t)z1; ++k) face_flux(cs, m.zone_faces[k], -1, nullptr, U, face, rhs);
    for (const Bc& b : cs.bcs) {
        uint32_t a = m.zone_off[b.zone], e = m.zone_off[b.zone + 1];
#pragma omp parallel for if (g_threads > 1) num_threads(g_threads)
        for (int64_t k = a; k < (int64_t)e; ++k) face_flux(cs, m.zone_faces[k], b.type, &b, U, face, rhs);
    }
#pragma omp parallel for if (g_threads > 1) num_threads(g_threads)
    for (int64_t c = 0; c < (int64_t)m.n_cells; ++c)
        for (int i = 0; i < NC; i++) rhs[(size_t)c * NC + i] /= m.cell_volume[c];
}

// SpectralRadiusFunctor + Solver::calc_dt (solver.cpp:580-742)
double calc_dt(Case& cs, double cfl) {
    const OMesh& m = *cs.mesh;
    const Gas& g = cs.gas;
    double rmax = -1.0;
#pragma omp parallel for reduction(max : rmax) if (g_threads > 1) num_threads(g_threads)
    for (int64_t ci = 0; ci < (int64_t)m.n_cells; ++ci) {
        uint32_t c = (uint32_t)ci;
        double conv = 0.0, acou = 0.0;
        uint32_t nf = m.n_faces_of_cell(c);
        for (uint32_t k = 0; k < nf; k++) {
            uint32_t f = m.face_of_cell(c, k);
            int32_t L = m.cof[2 * (size_t)f], R = m.cof[2 * (size_t)f + 1];
            double n[2], s[2];
            unit2(&m.face_normals[2 * (size_t)f], n);
            if (R == -1) {
                s[0] = 2.0 * std::pow(m.cell_volume[L], 1.0 / 2);
                s[1] = 2.0 * std::pow(m.cell_volume[L], 1.0 / 2);
                R = L;
            } else {
                s[0] = m.cc(R)[0] - m.cc(L)[0];
                s[1] = m.cc(R)[1] - m.cc(L)[1];
            }
            double dxn = std::fabs(s[0] * n[0] + s[1] * n[1]);
            double rl = cs.U[(size_t)L * NC], rr = cs.U[(size_t)R * NC];
            const double* wl = &cs.prim[(size_t)L * NP];
            const double* wr = &cs.prim[(size_t)R * NP];
            double al = g.sos(wl[2], rl), ar = g.sos(wr[2], rr);
            double af = 0.5 * (al + ar);
            double uf[2] = {0.5 * (wl[0] + wr[0]), 0.5 * (wl[1] + wr[1])};
            double un = std::fabs(uf[0] * n[0] + uf[1] * n[1]);
            conv += un / dxn;
            double t = af / dxn;
            acou += t * t;
        }
        double geom = 3.0 / nf;
        conv *= 1.37 * geom;
        acou = 1.37 * std::sqrt(geom * acou);
        double tot = conv + acou;
        rmax = std::max(rmax, tot);
        cs.cfl_local[c] = tot;
    }
    double dt = cfl / rmax;
    for (size_t c = 0; c < cs.cfl_local.size(); c++) cs.cfl_local[c] = dt * cs.cfl_local[c];
    if (dt < 0.0) throw std::runtime_error("dt negative: " + std::to_string(dt) + ".");
    return dt;
}

// Solver::update_primitives (solver.cpp:533-578)
void update_prims(Case& cs) {
    const OMesh& m = *cs.mesh;
#pragma omp parallel for if (g_threads > 1) num_threads(g_threads)
    for (int64_t c = 0; c < (int64_t)m.n_cells; ++c) cs.gas.prims(&cs.U[(size_t)c * NC], &cs.prim[(size_t)c * NP]);
}

// KokkosBlas::axpy(a, x, y): y <- y + a x ; axpby(a, x, b, y): y <- a x + b y
void axpy(double a, const std::vector<double>& x, std::vector<double>& y) {
    const int64_t n = (int64_t)y.size();
#pragma omp parallel for if (g_threads > 1) num_threads(g_threads)
    for (int64_t i = 0; i < n; i++) y[i] += a * x[i];
}
void axpby(double a, const std::vector<double>& x, double b, std::vector<double>& y) {
    const int64_t n = (int64_t)y.size();
#pragma omp parallel for if (g_threads > 1) num_threads(g_threads)
    for (int64_t i = 0; i < n; i++) y[i] = a * x[i] + b * y[i];
}

// FE::take_step (time_integrator.cpp:57-69)
void take_step_fe(Case& cs, double dt) {
    calc_rhs(cs, cs.U.data(), cs.face.data(), cs.r1.data());
    axpy(dt, cs.r1, cs.U);
    update_prims(cs);
}

// RK4::take_step (time_integrator.cpp:85-120), coefficients 1/6, 1/3, 1/3, 1/6 (:71-79)
void take_step_rk4(Case& cs, double dt) {
    const double c[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    if (cs.r4.size() != cs.r1.size()) cs.r4.assign(cs.r1.size(), 0.0);
    calc_rhs(cs, cs.U.data(), cs.face.data(), cs.r1.data());
    cs.Utmp = cs.U;
    axpy(dt / 2.0, cs.r1, cs.Utmp);
    calc_rhs(cs, cs.Utmp.data(), cs.face.data(), cs.r2.data());
    cs.Utmp = cs.U;
    axpy(dt / 2.0, cs.r2, cs.Utmp);
    calc_rhs(cs, cs.Utmp.data(), cs.face.data(), cs.r3.data());
    cs.Utmp = cs.U;
    axpy(dt, cs.r3, cs.Utmp);
    calc_rhs(cs, cs.Utmp.data(), cs.face.data(), cs.r4.data());
    axpy(dt * c[0], cs.r1, cs.U);
    axpy(dt * c[1], cs.r2, cs.U);
    axpy(dt * c[2], cs.r3, cs.U);
    axpy(dt * c[3], cs.r4, cs.U);
    update_prims(cs);
}

// SSPRK3::take_step (time_integrator.cpp:135-163) + Solver::take_step (solver.cpp:521-531)
void take_step(Case& cs, double dt) {
    if (cs.integrator == 1) return take_step_fe(cs, dt);
    if (cs.integrator == 2) return take_step_rk4(cs, dt);
    calc_rhs(cs, cs.U.data(), cs.face.data(), cs.r1.data());
    cs.Utmp = cs.U;
    axpy(dt, cs.r1, cs.Utmp);
    calc_rhs(cs, cs.Utmp.data(), cs.face.data(), cs.r2.data());
    axpby(3.0 / 4.0, cs.U, 1.0 / 4.0, cs.Utmp);
    axpy(dt / 4.0, cs.r2, cs.Utmp);
    calc_rhs(cs, cs.Utmp.data(), cs.face.data(), cs.r3.data());
    axpy(dt * (1.0 / 6.0), cs.r1, cs.U);
    axpy(dt * (1.0 / 6.0), cs.r2, cs.U);
    axpy(dt * (2.0 / 3.0), cs.r3, cs.U);
    update_prims(cs);
}

template <class F>
int guarded(F&& fn) {
    try {
        fn();
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return -1;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C API for the Python test harness (ctypes)
// ---------------------------------------------------------------------------

extern "C" {

const char* orc_last_error() { return g_last_error.c_str(); }

void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// mesh_type: 0 cartesian, 1 cartesian_tri, 2 wedge
void* orc_mesh_generate(int mesh_type, uint32_t nx, uint32_t ny, double Lx, double Ly) {
    OMesh* m = nullptr;
    int rc = guarded([&] {
        if (mesh_type == 0) m = new OMesh(gen_cart(nx, ny, Lx, Ly));
        else if (mesh_type == 1) m = new OMesh(gen_cart_tri(nx, ny, Lx, Ly));
        else if (mesh_type == 2) m = new OMesh(gen_wedge(nx, ny, Lx, Ly));
        else throw std::runtime_error("Unknown mesh type.");
    });
    return rc == 0 ? m : nullptr;
}

// Mesh from connectivity arrays (the reference's unimplemented FILE type);
// geometry is derived with the reference's formulas.  Zone 0 is interior.
void* orc_mesh_from_arrays(uint32_t n_nodes, const double* node_coords, uint32_t n_cells, const uint32_t* off_noc,
                           const uint32_t* noc, const uint32_t* off_foc, const uint32_t* foc, uint32_t n_faces,
                           const uint32_t* off_nof, const uint32_t* nof, const int32_t* cof, uint32_t n_zones,
                           const uint32_t* zone_off, const uint32_t* zone_faces) {
    OMesh* m = new OMesh();
    m->n_nodes = n_nodes;
    m->n_cells = n_cells;
    m->n_faces = n_faces;
    m->node_coords.assign(node_coords, node_coords + 2 * (size_t)n_nodes);
    m->off_noc.assign(off_noc, off_noc + n_cells + 1);
    m->noc.assign(noc, noc + off_noc[n_cells]);
    m->off_foc.assign(off_foc, off_foc + n_cells + 1);
    m->foc.assign(foc, foc + off_foc[n_cells]);
    m->off_nof.assign(off_nof, off_nof + n_faces + 1);
    m->nof.assign(nof, nof + off_nof[n_faces]);
    m->cof.assign(cof, cof + 2 * (size_t)n_faces);
    m->zone_off.assign(zone_off, zone_off + n_zones + 1);
    m->zone_faces.assign(zone_faces, zone_faces + zone_off[n_zones]);
    for (uint32_t z = 0; z < n_zones; z++) m->zone_names.push_back(z == 0 ? "interior" : "zone" + std::to_string(z));
    if (guarded([&] { geom_all(*m); }) != 0) {
        delete m;
        return nullptr;
    }
    return m;
}

void orc_mesh_free(void* h) { delete static_cast<OMesh*>(h); }

// Seeded relabelling of the cells (the benchmark meshes' random cell order),
// the same permutation the GPU library's mesh helper applies: a Fisher-Yates
// shuffle of new_of_old driven by std::mt19937_64(seed), position i - 1
// swapped with rng() % i for i = n .. 2.  Cell lists, centroids and volumes
// move with their cells; faces keep their numbers and only the cell ids on
// the faces of the zones change.  new_of_old (optional) receives the map.
int orc_mesh_permute_cells(void* h, uint64_t seed, uint32_t* new_of_old) {
    return guarded([&] {
        OMesh& m = *static_cast<OMesh*>(h);
        const uint32_t n = m.n_cells;
        std::vector<uint32_t> to_new(n), to_old(n);
        for (uint32_t i = 0; i < n; ++i) to_new[i] = i;
        std::mt19937_64 rng(seed);
        for (uint32_t i = n; i > 1; --i) std::swap(to_new[i - 1], to_new[(uint32_t)(rng() % i)]);
        for (uint32_t i = 0; i < n; ++i) to_old[to_new[i]] = i;
        auto move_lists = [&](std::vector<uint32_t>& off, std::vector<uint32_t>& flat) {
            std::vector<uint32_t> o2(1, 0), f2;
            f2.reserve(flat.size());
            for (uint32_t c = 0; c < n; ++c) {
                const uint32_t old = to_old[c];
                for (uint32_t k = off[old]; k < off[old + 1]; ++k) f2.push_back(flat[k]);
                o2.push_back((uint32_t)f2.size());
            }
            off.swap(o2);
            flat.swap(f2);
        };
        move_lists(m.off_noc, m.noc);
        move_lists(m.off_foc, m.foc);
        std::vector<double> cc(m.cell_coords.size()), vol(m.cell_volume.size());
        for (uint32_t c = 0; c < n; ++c) {
            cc[2 * (size_t)c] = m.cell_coords[2 * (size_t)to_old[c]];
            cc[2 * (size_t)c + 1] = m.cell_coords[2 * (size_t)to_old[c] + 1];
            vol[c] = m.cell_volume[to_old[c]];
        }
        m.cell_coords.swap(cc);
        m.cell_volume.swap(vol);
        for (uint32_t f : m.zone_faces)
            for (int sd = 0; sd < 2; ++sd) {
                int32_t& c = m.cof[2 * (size_t)f + sd];
                if (c >= 0) c = (int32_t)to_new[(uint32_t)c];
            }
        if (new_of_old) std::copy(to_new.begin(), to_new.end(), new_of_old);
    });
}

// field ids: 0 node_coords 1 cell_coords 2 cell_volume 3 face_area 4 face_normals
// 5 off_noc 6 noc 7 off_foc 8 foc 9 off_nof 10 nof 11 cells_of_face 12 zone_off 13 zone_faces
uint64_t orc_mesh_len(void* h, int field) {
    const OMesh& m = *static_cast<OMesh*>(h);
    switch (field) {
        case 0: return m.node_coords.size();
        case 1: return m.cell_coords.size();
        case 2: return m.cell_volume.size();
        case 3: return m.face_area.size();
        case 4: return m.face_normals.size();
        case 5: return m.off_noc.size();
        case 6: return m.noc.size();
        case 7: return m.off_foc.size();
        case 8: return m.foc.size();
        case 9: return m.off_nof.size();
        case 10: return m.nof.size();
        case 11: return m.cof.size();
        case 12: return m.zone_off.size();
        case 13: return m.zone_faces.size();
    }
    return 0;
}

void orc_mesh_copy(void* h, int field, void* dst) {
    const OMesh& m = *static_cast<OMesh*>(h);
    auto cp = [&](const auto& v) { std::memcpy(dst, v.data(), v.size() * sizeof(v[0])); };
    switch (field) {
        case 0: cp(m.node_coords); break;
        case 1: cp(m.cell_coords); break;
        case 2: cp(m.cell_volume); break;
        case 3: cp(m.face_area); break;
        case 4: cp(m.face_normals); break;
        case 5: cp(m.off_noc); break;
        case 6: cp(m.noc); break;
        case 7: cp(m.off_foc); break;
        case 8: cp(m.foc); break;
        case 9: cp(m.off_nof); break;
        case 10: cp(m.nof); break;
        case 11: cp(m.cof); break;
        case 12: cp(m.zone_off); break;
        case 13: cp(m.zone_faces); break;
    }
}

uint32_t orc_mesh_counts(void* h, uint32_t* n_nodes, uint32_t* n_cells, uint32_t* n_faces) {
    const OMesh& m = *static_cast<OMesh*>(h);
    *n_nodes = m.n_nodes;
    *n_cells = m.n_cells;
    *n_faces = m.n_faces;
    return (uint32_t)m.zone_names.size();
}

// Build a case.  recon: 0 FO, 1 TENO; basis: 0 monomial, 1 legendre;
// rsolver: 0 Rusanov, 1 HLL, 2 HLLC.  Quadrature orders follow TENO::init
// defaults (cell p+1 Dunavant, face (p+1)/2 Gauss-Legendre) when passed 0.
void* orc_case_create(void* mesh, int recon, int basis, int poly_order, double stencil_factor, int q_cell_order,
                      int q_face_order, int rsolver, double gamma, double p_ref, double T_ref, double rho_ref,
                      double p_min, double p_max) {
    Case* cs = new Case();
    int rc = guarded([&] {
        cs->mesh = static_cast<OMesh*>(mesh);
        cs->recon = recon;
        cs->rsolver = rsolver;
        cs->gas.gamma = gamma;
        cs->gas.p_ref = p_ref;
        cs->gas.T_ref = T_ref;
        cs->gas.rho_ref = rho_ref;
        cs->gas.p_min = p_min;
        cs->gas.p_max = p_max;
        cs->gas.derive();
        if (recon == RECON_FO) {
            cs->qface = gauss_legendre(1);
        } else {
            Teno& t = cs->teno;
            t.basis = basis;
            t.p = poly_order;
            t.qcell = dunavant(q_cell_order > 0 ? q_cell_order : poly_order + 1);
            cs->qface = gauss_legendre(q_face_order > 0 ? q_face_order : (poly_order + 1) / 2);
            teno_sizes(t, stencil_factor);
            teno_stencils(t, *cs->mesh);
            teno_matrices(t, *cs->mesh);
            teno_oscillation(t);
        }
        cs->nq = cs->qface.n();
        const OMesh& m = *cs->mesh;
        size_t nc = (size_t)m.n_cells * NC;
        cs->U.assign(nc, 0.0);
        cs->Utmp.assign(nc, 0.0);
        cs->r1.assign(nc, 0.0);
        cs->r2.assign(nc, 0.0);
        cs->r3.assign(nc, 0.0);
        cs->prim.assign((size_t)m.n_cells * NP, 0.0);
        cs->cfl_local.assign(m.n_cells, 0.0);
        cs->face.assign((size_t)m.n_faces * cs->nq * 2 * NC, 0.0);
    });
    if (rc != 0) {
        delete cs;
        return nullptr;
    }
    return cs;
}

void orc_case_free(void* h) { delete static_cast<Case*>(h); }

int orc_case_add_boundary(void* h, uint32_t zone, int type, const double* data, int n_data) {
    Case& cs = *static_cast<Case*>(h);
    return guarded([&] {
        if (zone == 0 || zone + 1 >= cs.mesh->zone_off.size()) throw std::runtime_error("Boundary zone not found in mesh.");
        Bc b;
        b.zone = zone;
        b.type = type;
        if (type == BC_UPT) {
            // BoundaryUPT::init (boundary_upt.cpp:38-73): data = (u0, u1, p, T)
            if (n_data < 4) throw std::runtime_error("Missing u, p or T for boundary.");
            double u0 = data[0], u1 = data[1], p = data[2], T = data[3];
            double rho = p / (cs.gas.R * T);
            double e = cs.gas.cv * T;
            double hh = e + p / rho;
            double d[6] = {rho, u0, u1, p, T, hh};
            std::memcpy(b.data, d, sizeof(d));
        } else if (type == BC_P_OUT) {
            if (n_data < 1) throw std::runtime_error("Missing p for boundary.");
            b.data[0] = data[0];
        }
        cs.bcs.push_back(b);
    });
}

void orc_case_set_state(void* h, const double* U, const double* prim) {
    Case& cs = *static_cast<Case*>(h);
    std::memcpy(cs.U.data(), U, cs.U.size() * sizeof(double));
    if (prim) std::memcpy(cs.prim.data(), prim, cs.prim.size() * sizeof(double));
    else update_prims(cs);
}

void orc_case_get_state(void* h, double* U, double* prim) {
    Case& cs = *static_cast<Case*>(h);
    if (U) std::memcpy(U, cs.U.data(), cs.U.size() * sizeof(double));
    if (prim) std::memcpy(prim, cs.prim.data(), cs.prim.size() * sizeof(double));
}

int orc_case_nq(void* h) { return static_cast<Case*>(h)->nq; }

void orc_case_set_teno_variant(void* h, int variant) { static_cast<Case*>(h)->teno_variant = variant; }

// Cell gradients of the viscous flux: 0 from the reconstructed polynomials
// (with TENO), 1 Green-Gauss.
void orc_case_set_viscous_gradients(void* h, int kind) { static_cast<Case*>(h)->visc_grad = kind; }

// Viscous face flux on (mu_ref > 0 or Sutherland) / off (viscous = 0).
void orc_case_set_viscous(void* h, int viscous, double mu_ref, double T_mu_ref, double sutherland_S, double prandtl) {
    Case* cs = static_cast<Case*>(h);
    cs->viscous = viscous != 0;
    cs->mu_ref = mu_ref;
    cs->T_mu_ref = T_mu_ref;
    cs->sutherland_S = sutherland_S;
    const double cp = cs->gas.R * cs->gas.gamma / (cs->gas.gamma - 1.0);
    cs->cp_over_pr = cp / prandtl;
}

// FaceReconstruction::calc_face_values; face must hold n_faces*nq*2*4 doubles.
// masks (optional, [n_cells][4]) receives the TENO decision bits.
int orc_case_face_values(void* h, const double* U, double* face, uint8_t* masks) {
    Case& cs = *static_cast<Case*>(h);
    return guarded([&] {
        if (masks) cs.masks.assign((size_t)cs.mesh->n_cells * NC, 0);
        recon(cs, U, face);
        if (masks) {
            std::memcpy(masks, cs.masks.data(), cs.masks.size());
            cs.masks.clear();
        }
    });
}

// The viscous flux's cell gradients of state U, [n_cells][6]: du/dx, du/dy,
// dv/dx, dv/dy, dT/dx, dT/dy (reconstructing first when they come from the
// polynomials).
int orc_case_viscous_gradients(void* h, const double* U, double* grad) {
    Case& cs = *static_cast<Case*>(h);
    return guarded([&] {
        const OMesh& m = *cs.mesh;
        const bool was = cs.viscous;
        cs.viscous = true;
        if (cs.recon == RECON_TENO && cs.visc_grad == 0) {
            std::vector<double> face((size_t)m.n_faces * cs.nq * 2 * NC);
            recon(cs, U, face.data());
        }
        mark_walls(cs);
        viscous_gradients(cs, U);
        cs.viscous = was;
        std::copy(cs.grad.begin(), cs.grad.end(), grad);
    });
}

int orc_case_calc_rhs(void* h, const double* U, double* rhs) {
    Case& cs = *static_cast<Case*>(h);
    return guarded([&] { calc_rhs(cs, U, cs.face.data(), rhs); });
}

int orc_case_calc_dt(void* h, double cfl, double* dt, double* cfl_local) {
    Case& cs = *static_cast<Case*>(h);
    return guarded([&] {
        *dt = calc_dt(cs, cfl);
        if (cfl_local) std::memcpy(cfl_local, cs.cfl_local.data(), cs.cfl_local.size() * sizeof(double));
    });
}

int orc_case_take_step(void* h, double dt) {
    Case& cs = *static_cast<Case*>(h);
    return guarded([&] { take_step(cs, dt); });
}

// The run loop (Solver::run, solver.cpp:352-373) without output or checks:
// n_steps x (calc_dt ; take_step).  Returns the simulated time reached.
int orc_case_run(void* h, double cfl, uint32_t n_steps, double* t_out) {
    Case& cs = *static_cast<Case*>(h);
    return guarded([&] {
        double t = 0.0;
        for (uint32_t s = 0; s < n_steps; s++) {
            double dt = calc_dt(cs, cfl);
            take_step(cs, dt);
            t += dt;
        }
        if (t_out) *t_out = t;
    });
}

// TENO tables in the reference's layout.  field: 0 off_groups 1 off_stencils
// 2 stencils 3 off_mats 4 mats 5 areas 6 ipt 7 oi 8 poly_indices (int32 pairs)
uint64_t orc_teno_len(void* h, int field) {
    const Teno& t = static_cast<Case*>(h)->teno;
    switch (field) {
        case 0: return t.off_groups.size();
        case 1: return t.off_stencils.size();
        case 2: return t.stencils.size();
        case 3: return t.off_mats.size();
        case 4: return t.mats.size();
        case 5: return t.areas.size();
        case 6: return t.ipt.size();
        case 7: return t.oi.size();
        case 8: return t.pidx.size();
    }
    return 0;
}

void orc_teno_copy(void* h, int field, void* dst) {
    const Teno& t = static_cast<Case*>(h)->teno;
    auto cp = [&](const auto& v) { std::memcpy(dst, v.data(), v.size() * sizeof(v[0])); };
    switch (field) {
        case 0: cp(t.off_groups); break;
        case 1: cp(t.off_stencils); break;
        case 2: cp(t.stencils); break;
        case 3: cp(t.off_mats); break;
        case 4: cp(t.mats); break;
        case 5: cp(t.areas); break;
        case 6: cp(t.ipt); break;
        case 7: cp(t.oi); break;
        case 8: {
            std::vector<int32_t> p(t.pidx.begin(), t.pidx.end());
            cp(p);
            break;
        }
    }
}

// Unit-level entry points used by the known-answer tests.
void orc_riemann_flux(int kind, const double* n_unit, double rl, const double* ul, double pl, double gl, double hl,
                      double rr, const double* ur, double pr, double gr, double hr, double* flux) {
    // kind | 16: the robust variant's guarded star pressure
    riemann(kind & 15, flux, n_unit, rl, ul, pl, gl, hl, rr, ur, pr, gr, hr, (kind & 16) != 0);
}

void orc_gas_constants(double gamma, double p_ref, double T_ref, double rho_ref, double* R_cp_cv) {
    Gas g;
    g.gamma = gamma;
    g.p_ref = p_ref;
    g.T_ref = T_ref;
    g.rho_ref = rho_ref;
    g.derive();
    R_cp_cv[0] = g.R;
    R_cp_cv[1] = g.cp;
    R_cp_cv[2] = g.cv;
}

void orc_primitives(double gamma, double p_ref, double T_ref, double rho_ref, double p_min, double p_max,
                    const double* U, double* W, uint32_t n) {
    Gas g;
    g.gamma = gamma;
    g.p_ref = p_ref;
    g.T_ref = T_ref;
    g.rho_ref = rho_ref;
    g.p_min = p_min;
    g.p_max = p_max;
    g.derive();
    for (uint32_t i = 0; i < n; i++) g.prims(U + (size_t)i * NC, W + (size_t)i * NP);
}

int orc_qr_householder(const double* A, double* R, int m, int n) { return guarded([&] { householder_r(A, R, m, n); }); }
void orc_forward_substitution(const double* L, const double* B, double* X, int m, int n, int p, int tL, int tB) {
    fwd_subst(L, B, X, m, n, p, tL != 0, tB != 0);
}
void orc_back_substitution(const double* U, const double* B, double* X, int m, int n, int p, int tU, int tB) {
    back_subst(U, B, X, m, n, p, tU != 0, tB != 0);
}
void orc_triangle_jac(const double* a, const double* b, const double* c, double* J, double* Jinv) {
    tri_jac(a, b, c, J);
    inv2(J, Jinv);
}
double orc_triangle_area(const double* a, const double* b, const double* c) { return tri_area(a, b, c); }

// FE and RK4 with a U-independent right-hand side (the same stub).
void orc_fe_const_rhs(double* U, const double* rhs, uint32_t n, double dt) {
    std::vector<double> u(U, U + (size_t)n * NC), r(rhs, rhs + (size_t)n * NC);
    axpy(dt, r, u);
    std::memcpy(U, u.data(), u.size() * sizeof(double));
}
void orc_rk4_const_rhs(double* U, const double* rhs, uint32_t n, double dt) {
    const double c[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    std::vector<double> u(U, U + (size_t)n * NC), r(rhs, rhs + (size_t)n * NC);
    for (int k = 0; k < 4; ++k) axpy(dt * c[k], r, u);
    std::memcpy(U, u.data(), u.size() * sizeof(double));
}

void orc_case_set_integrator(void* h, int integrator) { static_cast<Case*>(h)->integrator = integrator; }

// SSPRK3 with a caller-supplied right-hand side that does not depend on U
// (time_integrator_test.cpp:22-28 stub): rhs is [n][4], applied to U [n][4].
void orc_ssprk3_const_rhs(double* U, const double* rhs, uint32_t n, double dt) {
    std::vector<double> u(U, U + (size_t)n * NC), ut, r(rhs, rhs + (size_t)n * NC);
    ut = u;
    axpy(dt, r, ut);
    axpby(3.0 / 4.0, u, 1.0 / 4.0, ut);
    axpy(dt / 4.0, r, ut);
    axpy(dt * (1.0 / 6.0), r, u);
    axpy(dt * (1.0 / 6.0), r, u);
    axpy(dt * (2.0 / 3.0), r, u);
    std::memcpy(U, u.data(), u.size() * sizeof(double));
}

}  // extern "C"
