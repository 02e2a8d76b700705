// host_teno.cpp -- TENO stencil and least-squares table build for the GPU path.
//
// Computes what the reference's TENO::init computes
// (MatthewBonanni/Mallard src/numerics/face_reconstruction.cpp:109-788):
// per cell one central and one directional stencil per face, the
// pseudo-inverse of each stencil's least-squares matrix, the transformed
// cell areas, the basis means and the oscillation-indicator matrix.  The
// tables must be bit-identical to the reference's, because the GPU kernels'
// parity target is the reference's arithmetic; so every floating-point
// expression below keeps the reference's operation order.  What differs is
// the organisation:
//  * cells are processed in parallel (OpenMP), cell 0 first because the
//    basis means come from its central stencil;
//  * ring membership uses an epoch-stamped marker array instead of linear
//    searches over all previous rings (same membership, same order);
//  * the Householder QR applies each reflector only to the rows and columns
//    it changes: the reference multiplies by the full m x m reflector, whose
//    other entries contribute exact zeros, so the results are identical
//    while the work drops from O(m^3 n) to O(m^2 n) per stencil.
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>
#include <cstring>
#include <memory>
#include <utility>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "host.h"

namespace mgpu {

// ---------------------------------------------------------------------------
// Quadrature tables (quadrature.cpp:23-273)
// ---------------------------------------------------------------------------

bool gauss_legendre_rule(int order, QuadRule& r) {
    r.dim = 1;
    switch (order) {
        case 1: r.pts = {0.0}; r.wts = {2.0}; return true;
        case 2:
            r.pts = {-0.577350269189625764509149, 0.577350269189625764509149};
            r.wts = {1.0, 1.0};
            return true;
        case 3:
            r.pts = {-0.774596669241483377035853, 0.0, 0.774596669241483377035853};
            r.wts = {0.55555555555555555555556, 0.88888888888888888888889, 0.55555555555555555555556};
            return true;
        case 4:
            r.pts = {-0.861136311594052575223946, -0.339981043584856264802666, 0.339981043584856264802666,
                     0.861136311594052575223946};
            r.wts = {0.34785484513745385737306, 0.65214515486254614262694, 0.65214515486254614262694,
                     0.34785484513745385737306};
            return true;
    }
    return false;
}

bool dunavant_rule(int order, QuadRule& r) {
    r.dim = 2;
    switch (order) {
        case 1: r.pts = {1.0 / 3.0, 1.0 / 3.0}; r.wts = {1.0}; return true;
        case 2:
            r.pts = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
            r.wts = {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0};
            return true;
        case 3:
            r.pts = {1.0 / 3.0, 1.0 / 3.0, 0.6, 0.2, 0.2, 0.6, 0.2, 0.2};
            r.wts = {-0.5625, 0.52083333333333333333333333333333, 0.52083333333333333333333333333333,
                     0.52083333333333333333333333333333};
            return true;
        case 4:
            r.pts = {0.108103018168070, 0.445948490915965, 0.445948490915965, 0.108103018168070,
                     0.445948490915965, 0.445948490915965, 0.816847572980459, 0.091576213509771,
                     0.091576213509771, 0.816847572980459, 0.091576213509771, 0.091576213509771};
            r.wts = {0.223381589678011, 0.223381589678011, 0.223381589678011,
                     0.109951743655322, 0.109951743655322, 0.109951743655322};
            return true;
        case 5:
            r.pts = {0.333333333333333, 0.333333333333333, 0.059715871789770, 0.470142064105115,
                     0.470142064105115, 0.059715871789770, 0.470142064105115, 0.470142064105115,
                     0.797426985353087, 0.101286507323456, 0.101286507323456, 0.797426985353087,
                     0.101286507323456, 0.101286507323456};
            r.wts = {0.225000000000000, 0.132394152788506, 0.132394152788506, 0.132394152788506,
                     0.125939180544827, 0.125939180544827, 0.125939180544827};
            return true;
    }
    return false;
}

// ---------------------------------------------------------------------------
// Basis functions (basis.h:65-221), p <= 4
// ---------------------------------------------------------------------------

double basis_1d(int type, int p, double x) {
    if (type == MGPU_BASIS_MONOMIAL) return std::pow(x, (double)p);
    switch (p) {
        case 0: return 1.0 * (1.0);
        case 1: return 1.0 * (1.0 * x);
        case 2: return 0.5 * (3.0 * x * x - 1.0);
        case 3: return 0.5 * (5.0 * x * x * x - 3.0 * x);
        case 4: return 0.125 * (35.0 * x * x * x * x - 30.0 * x * x + 3.0);
    }
    throw std::runtime_error("basis order above 4 is not supported");
}

double basis_1d_deriv(int type, int n, int p, double x) {
    if (type == MGPU_BASIS_MONOMIAL) {
        // MonomialTraits::derivative_1D keeps the reference's (p - k + 1) factor.
        double r = std::pow(x, (double)(p - n));
        for (int k = 0; k < n; ++k) r *= (double)(p - k + 1);
        return r;
    }
    if (n > p) return 0.0;
    if (n == 0) return basis_1d(type, p, x);
    const int key = 10 * n + p;
    switch (key) {
        case 11: return 1.0 * (1.0 * 1.0);
        case 12: return 0.5 * (3.0 * 2.0 * x);
        case 13: return 0.5 * (5.0 * 3.0 * x * x - 3.0 * 1.0);
        case 14: return 0.125 * (35.0 * 4.0 * x * x * x - 30.0 * 2.0 * x);
        case 22: return 0.5 * (3.0 * 2.0 * 1.0);
        case 23: return 0.5 * (5.0 * 3.0 * 2.0 * x);
        case 24: return 0.125 * (35.0 * 4.0 * 3.0 * x * x - 30.0 * 2.0 * 1.0);
        case 33: return 0.5 * (5.0 * 3.0 * 2.0 * 1.0);
        case 34: return 0.125 * (35.0 * 4.0 * 3.0 * 2.0 * x);
        case 44: return 0.125 * (35.0 * 4.0 * 3.0 * 2.0 * 1.0);
    }
    throw std::runtime_error("basis derivative above order 4 is not supported");
}

namespace {

// ---------------------------------------------------------------------------
// Stencil search (face_reconstruction.cpp:217-475)
// ---------------------------------------------------------------------------

struct Graph {
    // first-order neighbourhood of each cell: the cell and its face
    // neighbours, sorted and unique (Mesh::h_neighbors_of_cell, n_order 1)
    std::vector<uint32_t> off, nb;
};

Graph neighbourhoods(const mgpu_mesh& m) {
    Graph g;
    const uint32_t N = m.n_cells;
    g.off.assign((size_t)N + 1, 0);
    // per cell at most 1 + its faces entries: fill fixed slots in parallel,
    // then compact
    std::vector<uint32_t> cnt(N), slot(N + (size_t)m.offsets_faces_of_cell[N]);
#pragma omp parallel
    {
        std::vector<uint32_t> tmp;
#pragma omp for schedule(static)
        for (int64_t ci = 0; ci < (int64_t)N; ++ci) {
            const uint32_t c = (uint32_t)ci;
            tmp.clear();
            tmp.push_back(c);
            for (uint32_t k = m.offsets_faces_of_cell[c]; k < m.offsets_faces_of_cell[c + 1]; ++k) {
                const uint32_t f = m.faces_of_cell[k];
                const int32_t a = m.cells_of_face[2 * (size_t)f], b = m.cells_of_face[2 * (size_t)f + 1];
                if (b == -1) continue;
                tmp.push_back(a == (int32_t)c ? (uint32_t)b : (uint32_t)a);
            }
            std::sort(tmp.begin(), tmp.end());
            tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
            cnt[c] = (uint32_t)tmp.size();
            std::copy(tmp.begin(), tmp.end(), &slot[c + (size_t)m.offsets_faces_of_cell[c]]);
        }
    }
    for (uint32_t c = 0; c < N; ++c) g.off[c + 1] = g.off[c] + cnt[c];
    g.nb.resize(g.off[N]);
#pragma omp parallel for schedule(static)
    for (int64_t ci = 0; ci < (int64_t)N; ++ci) {
        const uint32_t c = (uint32_t)ci;
        std::copy(&slot[c + (size_t)m.offsets_faces_of_cell[c]], &slot[c + (size_t)m.offsets_faces_of_cell[c]] + cnt[c],
                  &g.nb[g.off[c]]);
    }
    return g;
}

// Ring expansion with per-thread scratch.  A cell is "seen" when its stamp
// equals the current epoch; the reference's membership test over all rings
// plus the ring under construction is exactly this set.
struct RingBuilder {
    const mgpu_mesh* m = nullptr;
    const Graph* g = nullptr;
    std::vector<uint32_t> stamp;
    uint32_t epoch = 0;
    std::vector<std::pair<uint32_t, double>> dist;

    void init(const mgpu_mesh& mesh, const Graph& graph) {
        m = &mesh;
        g = &graph;
        stamp.assign(mesh.n_cells, 0);
    }
    void begin() {
        if (++epoch == 0) {
            std::fill(stamp.begin(), stamp.end(), 0);
            epoch = 1;
        }
    }
    void mark(uint32_t c) { stamp[c] = epoch; }

    // TENO::get_next_ring: candidates in the order met from the previous
    // ring, then std::sort by squared distance to the target.
    void next(const std::vector<uint32_t>& prev, uint32_t target, std::vector<uint32_t>& out) {
        out.clear();
        for (uint32_t c : prev)
            for (uint32_t k = g->off[c]; k < g->off[c + 1]; ++k) {
                const uint32_t n = g->nb[k];
                if (stamp[n] == epoch) continue;
                stamp[n] = epoch;
                out.push_back(n);
            }
        dist.clear();
        const double* X = m->cell_coords;
        for (uint32_t n : out) {
            double d = 0.0;
            for (int i = 0; i < 2; i++) {
                const double t = X[2 * (size_t)n + i] - X[2 * (size_t)target + i];
                d += t * t;
            }
            dist.push_back(std::make_pair(n, d));
        }
        std::sort(dist.begin(), dist.end(), [](auto& a, auto& b) { return a.second < b.second; });
        for (size_t i = 0; i < out.size(); ++i) out[i] = dist[i].first;
    }
};

// All stencils of one cell: central first, then one per face
// (compute_stencils_of_cell, face_reconstruction.cpp:406-433).
void cell_stencils(RingBuilder& rb, uint32_t c, int M, std::vector<std::vector<uint32_t>>& st) {
    const mgpu_mesh& m = *rb.m;
    const uint32_t f0 = m.offsets_faces_of_cell[c];
    const int nf = (int)(m.offsets_faces_of_cell[c + 1] - f0);
    st.assign(1 + nf, {});

    // Rings around c, shared by the central stencil and the first phase of
    // the directional search (both start from {c}).
    std::vector<std::vector<uint32_t>> rings;
    rb.begin();
    rb.mark(c);
    rings.push_back({c});
    auto grow = [&]() {
        std::vector<uint32_t> nr;
        rb.next(rings.back(), c, nr);
        rings.push_back(std::move(nr));
    };

    // central (Naive Cell Based, face_reconstruction.cpp:267-286)
    std::vector<uint32_t>& cen = st[0];
    cen.push_back(c);
    for (size_t r = 1; (int)cen.size() < M; ++r) {
        if (r >= rings.size()) grow();
        for (uint32_t n : rings[r]) {
            if ((int)cen.size() == M) break;
            cen.push_back(n);
        }
        if (rings[r].empty() && r + 1 >= rings.size() && (int)cen.size() < M) {
            // the whole connected mesh is exhausted: the reference would loop forever
            throw std::runtime_error("Mesh too small for the TENO stencil size.");
        }
    }

    // directional (Type 4, face_reconstruction.cpp:288-404)
    const double* X = m.cell_coords;
    std::vector<double> Jinv(4 * (size_t)nf);
    for (int s = 0; s < nf; ++s) {
        const uint32_t f = m.faces_of_cell[f0 + s];
        const uint32_t n0 = m.nodes_of_face[m.offsets_nodes_of_face[f]];
        const uint32_t n1 = m.nodes_of_face[m.offsets_nodes_of_face[f] + 1];
        double J[4];
        tri_jacobian(X + 2 * (size_t)c, m.node_coords + 2 * (size_t)n0, m.node_coords + 2 * (size_t)n1, J);
        mat2_inverse(J, &Jinv[4 * (size_t)s]);
        st[1 + s].push_back(c);
    }
    auto is_bnd = [&](int s) { return m.cells_of_face[2 * (size_t)m.faces_of_cell[f0 + s] + 1] == -1; };
    std::vector<char> grew(nf);
    bool done = false;
    for (size_t r = 1; !done; ++r) {
        if (r >= rings.size()) grow();
        std::fill(grew.begin(), grew.end(), 0);
        for (int s = 0; s < nf; ++s) {
            std::vector<uint32_t>& d = st[1 + s];
            for (uint32_t n : rings[r]) {
                if ((int)d.size() == M) break;
                const double dx[2] = {X[2 * (size_t)n] - X[2 * (size_t)c], X[2 * (size_t)n + 1] - X[2 * (size_t)c + 1]};
                double t[2];
                mat2_vec(&Jinv[4 * (size_t)s], dx, t);
                if (!(t[0] < 0.0) && !(t[1] < 0.0)) {
                    d.push_back(n);
                    grew[s] = 1;
                }
            }
        }
        done = true;
        for (int s = 0; s < nf; ++s)
            if (!is_bnd(s) && (int)st[1 + s].size() < M && grew[s]) {
                done = false;
                break;
            }
    }
    // fill-up phase: grow outwards from the whole stencil
    std::vector<uint32_t> cur, nr;
    for (int s = 0; s < nf; ++s) {
        std::vector<uint32_t>& d = st[1 + s];
        if (is_bnd(s)) {
            d.clear();
            continue;
        }
        if ((int)d.size() >= M) continue;
        rb.begin();
        for (uint32_t n : d) rb.mark(n);
        cur = d;
        while ((int)d.size() < M) {
            rb.next(cur, c, nr);
            if (nr.empty()) throw std::runtime_error("Mesh too small for the TENO stencil size.");
            for (uint32_t n : nr) {
                if ((int)d.size() == M) break;
                d.push_back(n);
            }
            cur.swap(nr);
        }
    }
    for (auto& s : st)
        if ((int)s.size() < M && !s.empty()) throw std::runtime_error("Stencil is not full.");
}

// ---------------------------------------------------------------------------
// Least squares (face_reconstruction.cpp:477-741, common_math.h:355-493)
// ---------------------------------------------------------------------------

// QR_householder_noQ restricted to the rows/columns each reflector touches.
void householder_upper(const double* A, double* R, int m, int n, std::vector<double>& v, std::vector<double>& col) {
    for (int i = 0; i < m * n; i++) R[i] = A[i];
    v.resize(m);
    col.resize(m);
    for (int j = 0; j < n; j++) {
        double nx = 0.0;
        for (int i = j; i < m; i++) nx += R[i * n + j] * R[i * n + j];
        nx = std::sqrt(nx);
        if (nx < 1.0e-15) continue;
        const double sgn = (R[j * n + j] >= 0.0) ? 1.0 : -1.0;
        const double alpha = -sgn * nx;
        double nu = 0.0;
        for (int k = 0; k < m - j; k++) {
            v[k] = R[(j + k) * n + j];
            if (k == 0) v[k] -= alpha;
            nu += v[k] * v[k];
        }
        nu = std::sqrt(nu);
        for (int k = 0; k < m - j; k++) v[k] /= nu;
        // rows < j are unchanged by I - 2 v v^T (exact); columns < j are never read again
        for (int c = j; c < n; c++) {
            for (int i = j; i < m; i++) {
                double s = 0.0;
                for (int k = j; k < m; k++) {
                    const double q = ((i == k) ? 1.0 : 0.0) - 2.0 * v[i - j] * v[k - j];
                    s += q * R[k * n + c];
                }
                col[i] = s;
            }
            for (int i = j; i < m; i++) R[i * n + c] = col[i];
        }
    }
}

// forward_substitution with tL = tB = true: solves R^T Y = B^T
void solve_rt(const double* R, const double* B, double* Y, int m, int n, int p) {
    for (int i = 0; i < m; i++)
        for (int j = 0; j < p; j++) {
            double s = 0.0;
            for (int k = 0; k < i; k++) s += R[k * m + i] * Y[k * p + j];
            Y[i * p + j] = (B[j * n + i] - s) / R[i * m + i];
        }
}

// back_substitution with tU = tB = false: solves R X = Y
void solve_r(const double* R, const double* Y, double* X, int m, int n, int p) {
    for (int i = m - 1; i >= 0; i--)
        for (int j = 0; j < p; j++) {
            double s = 0.0;
            for (int k = i + 1; k < m; k++) s += R[i * n + k] * X[k * p + j];
            X[i * p + j] = (Y[i * p + j] - s) / R[i * n + i];
        }
}

struct LsqScratch {
    std::vector<double> at, A, B, R, Y, qp, v, col;
};

// Moments of the basis over every stencil cell in the target's reference
// frame; returns the transformed areas in `at` and the moment matrix in `A`
// ([M][K] row-major), before the mean subtraction.
void stencil_moments(const mgpu_mesh& m, const TenoTables& t, uint32_t c, const uint32_t* cells, int M, LsqScratch& s) {
    const int K = t.K, nq = t.qcell.n();
    const double* N = m.node_coords;
    const uint32_t* nc = m.nodes_of_cell + m.offsets_nodes_of_cell[c];
    const double* w0 = N + 2 * (size_t)nc[0];
    double J[4], Ji[4];
    tri_jacobian(w0, N + 2 * (size_t)nc[1], N + 2 * (size_t)nc[2], J);
    mat2_inverse(J, Ji);
    s.at.resize(M);
    s.A.resize((size_t)M * K);
    s.qp.resize(2 * (size_t)nq);
    for (int j = 0; j < M; ++j) {
        const uint32_t* nn = m.nodes_of_cell + m.offsets_nodes_of_cell[cells[j]];
        double v[3][2], vt[3][2];
        for (int k = 0; k < 3; ++k) {
            v[k][0] = N[2 * (size_t)nn[k]];
            v[k][1] = N[2 * (size_t)nn[k] + 1];
        }
        double Jn[4];
        tri_jacobian(v[0], v[1], v[2], Jn);
        for (int k = 0; k < 3; ++k) {
            vt[k][0] = v[k][0] - w0[0];
            vt[k][1] = v[k][1] - w0[1];
            mat2_vec(Ji, vt[k], vt[k]);
        }
        s.at[j] = tri_area(vt[0], vt[1], vt[2]);
        for (int q = 0; q < nq; ++q) {
            double x[2] = {t.qcell.pts[2 * q], t.qcell.pts[2 * q + 1]};
            mat2_vec(Jn, x, x);
            x[0] += v[0][0];
            x[1] += v[0][1];
            x[0] -= w0[0];
            x[1] -= w0[1];
            mat2_vec(Ji, x, x);
            s.qp[2 * q] = x[0];
            s.qp[2 * q + 1] = x[1];
        }
        for (int k = 0; k < K; ++k) {
            double a = 0.0;
            for (int q = 0; q < nq; ++q)
                a += t.qcell.wts[q] * basis_2d(t.basis, t.pidx[2 * k], t.pidx[2 * k + 1], s.qp[2 * q], s.qp[2 * q + 1]);
            a *= s.at[j];
            s.A[(size_t)j * K + k] = a;
        }
    }
}

// Pseudo-inverse of the mean-subtracted moment matrix, written K x M
// row-major into out (compute_reconstruction_matrices, :604-693).
void stencil_pinv(const TenoTables& t, int M, LsqScratch& s, double* out) {
    const int K = t.K;
    for (int j = 0; j < M; ++j)
        for (int k = 0; k < K; ++k) s.A[(size_t)j * K + k] -= s.at[j] * t.ipt[k];
    bool col0_zero = true;
    for (int j = 0; j < M; ++j)
        if (s.A[(size_t)j * K] > 1.0e-12) {
            col0_zero = false;
            break;
        }
    if (col0_zero) {
        const int m = M - 1, n = K - 1;
        s.B.resize((size_t)m * n);
        s.R.resize((size_t)m * n);
        s.Y.resize((size_t)n * m);
        for (int j = 1; j < M; ++j)
            for (int k = 1; k < K; ++k) s.B[(size_t)(j - 1) * n + (k - 1)] = s.A[(size_t)j * K + k];
        householder_upper(s.B.data(), s.R.data(), m, n, s.v, s.col);
        solve_rt(s.R.data(), s.B.data(), s.Y.data(), n, n, m);
        solve_r(s.R.data(), s.Y.data(), s.B.data(), n, n, m);
        for (int k = 0; k < K; ++k)
            for (int j = 0; j < M; ++j)
                out[(size_t)k * M + j] = (k == 0 || j == 0) ? 0.0 : s.B[(size_t)(k - 1) * m + (j - 1)];
    } else {
        s.R.resize((size_t)M * K);
        s.Y.resize((size_t)K * M);
        householder_upper(s.A.data(), s.R.data(), M, K, s.v, s.col);
        solve_rt(s.R.data(), s.A.data(), s.Y.data(), K, K, M);
        solve_r(s.R.data(), s.Y.data(), out, K, K, M);
    }
}

}  // namespace

struct LsqWork {
    LsqScratch s;
};

LsqWork* lsq_work_new() { return new LsqWork(); }
void lsq_work_free(LsqWork* w) { delete w; }

void teno_stencil_lsq(const mgpu_mesh& m, const TenoTables& t, size_t stencil, LsqWork& w, double* pinv, double* areas) {
    const uint32_t c = (uint32_t)(stencil / 4);
    const uint32_t so = t.off_stencils[stencil];
    const int Ms = (int)(t.off_stencils[stencil + 1] - so);
    if (Ms == 0) return;
    stencil_moments(m, t, c, &t.stencils[so], Ms, w.s);
    std::copy(w.s.at.begin(), w.s.at.end(), areas);
    stencil_pinv(t, Ms, w.s, pinv);
}

double teno_target_area(const mgpu_mesh& m, const TenoTables& t, uint32_t c, LsqWork& w) {
    stencil_moments(m, t, c, &c, 1, w.s);
    return w.s.at[0];
}

void build_teno_stencils(const mgpu_mesh& m, int basis, int p, double factor, int q_cell, int q_face, TenoTables& t,
                         bool gpu_search) {
    if (p < 1 || p > 4) throw std::runtime_error("TENO basis order must be 1..4");
    t.basis = basis;
    t.p = p;
    if (!dunavant_rule(q_cell > 0 ? q_cell : p + 1, t.qcell))
        throw std::runtime_error("Triangle Dunavant quadrature rule of order " + std::to_string(q_cell > 0 ? q_cell : p + 1) +
                                 " not implemented.");
    if (!gauss_legendre_rule(q_face > 0 ? q_face : (p + 1) / 2, t.qface))
        throw std::runtime_error("Gauss-Legendre quadrature rule of order " +
                                 std::to_string(q_face > 0 ? q_face : (p + 1) / 2) + " not implemented.");
    // calc_max_stencil_size / calc_polynomial_indices (:170-215)
    t.K = (p + 1) * (p + 2) / 2;
    t.M = (int)(uint16_t)(factor * t.K);
    t.pidx.clear();
    for (int ip = 0; ip <= p; ++ip)
        for (int b = 0; b <= ip; ++b) {
            t.pidx.push_back(ip - b);
            t.pidx.push_back(b);
        }
    for (uint32_t c = 0; c < m.n_cells; ++c)
        if (m.offsets_nodes_of_cell[c + 1] - m.offsets_nodes_of_cell[c] != 3)
            throw std::runtime_error("TENO has only been implemented for triangular cells.");

    const uint32_t N = m.n_cells;
    const int M = t.M, K = t.K;
    const int S = 4;  // 1 central + 3 directional for triangles
    const Graph g = neighbourhoods(m);

    // --- stencils, stored [cell][S][M] with their sizes (each written up
    // to its size); on the GPU, then on the host for the cells it marks
    // (all of them without it)
    std::unique_ptr<uint32_t[]> flat(new uint32_t[(size_t)N * S * M]);
    std::vector<uint8_t> sizes((size_t)N * S, 0);
    std::vector<uint8_t> redo(N, 1);
    std::string err;
    if (gpu_search && M <= 255 && !gpu_stencil_search(m, g.off.data(), g.nb.data(), M, flat.get(), sizes.data(),
                                                      redo.data(), err))
        throw std::runtime_error(err);
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nthreads)
    {
        RingBuilder rb;
        std::vector<std::vector<uint32_t>> st;
        bool ready = false;
#pragma omp for schedule(dynamic, 256)
        for (int64_t ci = 0; ci < (int64_t)N; ++ci) {
            if (!redo[ci]) continue;
            if (!ready) {
                rb.init(m, g);
                ready = true;
            }
            try {
                cell_stencils(rb, (uint32_t)ci, M, st);
                for (int s = 0; s < S; ++s) {
                    sizes[(size_t)ci * S + s] = (uint8_t)st[s].size();
                    std::copy(st[s].begin(), st[s].end(), &flat[((size_t)ci * S + s) * M]);
                }
            } catch (const std::exception& e) {
#pragma omp critical
                err = e.what();
            }
        }
    }
    if (!err.empty()) throw std::runtime_error(err);

    // --- offsets in the reference's layout
    t.off_groups.assign((size_t)N + 1, 0);
    t.off_stencils.assign((size_t)N * S + 1, 0);
    t.off_mats.assign((size_t)N * S + 1, 0);
    for (uint32_t c = 0; c < N; ++c) {
        t.off_groups[c + 1] = (c + 1) * S;
        for (int s = 0; s < S; ++s) {
            const size_t i = (size_t)c * S + s;
            t.off_stencils[i + 1] = t.off_stencils[i] + sizes[i];
            t.off_mats[i + 1] = t.off_mats[i] + (uint32_t)(sizes[i] * K);
            if (s == 0 && sizes[i] == 0) throw std::runtime_error("Central stencil is empty for cell " + std::to_string(c) + ".");
        }
    }
    t.stencils.resize(t.off_stencils.back());
#pragma omp parallel for schedule(static)
    for (int64_t ci = 0; ci < (int64_t)N; ++ci)
        for (int s = 0; s < S; ++s) {
            const size_t i = (size_t)ci * S + s;
            std::copy(&flat[i * M], &flat[i * M] + sizes[i], &t.stencils[t.off_stencils[i]]);
        }
    flat.reset();
    // --- basis means from cell 0's central stencil (:598-602)
    t.ipt.assign(K, 0.0);
    {
        LsqScratch s;
        stencil_moments(m, t, 0, &t.stencils[t.off_stencils[0]], M, s);
        for (int k = 0; k < K; ++k) t.ipt[k] = s.A[k] / s.at[0];
    }

    // --- oscillation indicator (:743-788)
    const int nq = t.qcell.n();
    t.oi.assign((size_t)K * K, 0.0);
    for (int i = 0; i < K; i++)
        for (int j = 0; j < K; j++) {
            double acc = 0.0;
            for (int k = 1; k < K; k++)
                for (int q = 0; q < nq; ++q) {
                    double di = 1.0, dj = 1.0;
                    for (int d = 0; d < 2; d++) di *= basis_1d_deriv(basis, t.pidx[2 * k + d], t.pidx[2 * i + d], t.qcell.pts[2 * q + d]);
                    for (int d = 0; d < 2; d++) dj *= basis_1d_deriv(basis, t.pidx[2 * k + d], t.pidx[2 * j + d], t.qcell.pts[2 * q + d]);
                    acc += t.qcell.wts[q] * di * dj;
                }
            t.oi[(size_t)i * K + j] = acc;
        }
}


void build_teno_tables(const mgpu_mesh& m, int basis, int p, double factor, int q_cell, int q_face, TenoTables& t) {
    build_teno_stencils(m, basis, p, factor, q_cell, q_face, t);
    t.mats.assign(t.off_mats.back(), 0.0);
    t.areas.assign(t.off_stencils.back(), 0.0);
    const int64_t ns = (int64_t)t.off_stencils.size() - 1;
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nthreads)
    {
        LsqWork w;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < ns; ++i)
            teno_stencil_lsq(m, t, (size_t)i, w, &t.mats[t.off_mats[i]], &t.areas[t.off_stencils[i]]);
    }
}

}  // namespace mgpu

// ---------------------------------------------------------------------------
// C ABI: host-side TENO tables in the reference layout (for inspection and
// for checking the table build against the reference's arithmetic).
// ---------------------------------------------------------------------------

struct mgpu_teno_tables {
    mgpu::TenoTables t;
};

extern "C" {

int mgpu_teno_tables_build(const mgpu_mesh* mesh, int basis, int poly_order, double stencil_factor, int q_cell,
                           int q_face, mgpu_teno_tables** out) {
    if (!mesh || !out) {
        mgpu::set_error("mgpu_teno_tables_build: null argument");
        return MGPU_ERR_ARG;
    }
    try {
        auto* h = new mgpu_teno_tables();
        try {
            mgpu::build_teno_tables(*mesh, basis, poly_order, stencil_factor, q_cell, q_face, h->t);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
        return MGPU_OK;
    } catch (const std::exception& e) {
        mgpu::set_error(e.what());
        return MGPU_ERR_ARG;
    }
}

uint64_t mgpu_teno_tables_len(const mgpu_teno_tables* h, int field) {
    if (!h) return 0;
    const mgpu::TenoTables& t = h->t;
    switch (field) {
        case MGPU_TENO_OFFSETS_STENCIL_GROUPS: return t.off_groups.size();
        case MGPU_TENO_OFFSETS_STENCILS: return t.off_stencils.size();
        case MGPU_TENO_STENCILS: return t.stencils.size();
        case MGPU_TENO_OFFSETS_MATRICES: return t.off_mats.size();
        case MGPU_TENO_MATRICES: return t.mats.size();
        case MGPU_TENO_TRANSFORMED_AREAS: return t.areas.size();
        case MGPU_TENO_INTEGRAL_PSI_TARGET: return t.ipt.size();
        case MGPU_TENO_OSCILLATION_INDICATOR: return t.oi.size();
        case MGPU_TENO_POLY_INDICES: return t.pidx.size();
    }
    return 0;
}

int mgpu_teno_tables_copy(const mgpu_teno_tables* h, int field, void* dst) {
    if (!h || !dst) {
        mgpu::set_error("mgpu_teno_tables_copy: null argument");
        return MGPU_ERR_ARG;
    }
    const mgpu::TenoTables& t = h->t;
    auto cp = [&](const auto& v) { std::memcpy(dst, v.data(), v.size() * sizeof(v[0])); };
    switch (field) {
        case MGPU_TENO_OFFSETS_STENCIL_GROUPS: cp(t.off_groups); break;
        case MGPU_TENO_OFFSETS_STENCILS: cp(t.off_stencils); break;
        case MGPU_TENO_STENCILS: cp(t.stencils); break;
        case MGPU_TENO_OFFSETS_MATRICES: cp(t.off_mats); break;
        case MGPU_TENO_MATRICES: cp(t.mats); break;
        case MGPU_TENO_TRANSFORMED_AREAS: cp(t.areas); break;
        case MGPU_TENO_INTEGRAL_PSI_TARGET: cp(t.ipt); break;
        case MGPU_TENO_OSCILLATION_INDICATOR: cp(t.oi); break;
        case MGPU_TENO_POLY_INDICES: {
            std::vector<int32_t> p(t.pidx.begin(), t.pidx.end());
            cp(p);
            break;
        }
        default:
            mgpu::set_error("mgpu_teno_tables_copy: unknown field");
            return MGPU_ERR_ARG;
    }
    return MGPU_OK;
}

void mgpu_teno_tables_free(mgpu_teno_tables* h) { delete h; }

}  // extern "C"
