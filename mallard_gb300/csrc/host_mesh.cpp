// host_mesh.cpp -- meshes for the GPU path: the reference's generators and
// geometry (MatthewBonanni/Mallard src/mesh/mesh.cpp), written straight into
// CSR arrays, plus a seeded cell relabelling used to store structured meshes
// as unstructured ones.
//
// Numbering, zone order and floating-point expressions follow the reference
// so that a mesh generated here is bit-identical to the reference's: the
// TENO stencil search breaks distance ties by cell index, so the numbering is
// part of the algorithm's input.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <stdexcept>

#include "host.h"

namespace mgpu {

mgpu_mesh HostMesh::view() const {
    mgpu_mesh v{};
    v.n_nodes = n_nodes;
    v.n_cells = n_cells;
    v.n_faces = n_faces;
    v.node_coords = node_coords.data();
    v.cell_coords = cell_coords.data();
    v.cell_volume = cell_volume.data();
    v.face_area = face_area.data();
    v.face_normals = face_normals.data();
    v.offsets_nodes_of_cell = off_noc.data();
    v.nodes_of_cell = noc.data();
    v.offsets_faces_of_cell = off_foc.data();
    v.faces_of_cell = foc.data();
    v.offsets_nodes_of_face = off_nof.data();
    v.nodes_of_face = nof.data();
    v.cells_of_face = cof.data();
    v.n_zones = zone_off.empty() ? 0 : (uint32_t)zone_off.size() - 1;
    v.zone_offsets = zone_off.data();
    v.zone_faces = zone_faces.data();
    return v;
}

double tri_area(const double* a, const double* b, const double* c) {
    // triangle_area<2> (common_math.h:509-516)
    return 0.5 * std::fabs(a[0] * (b[1] - c[1]) + b[0] * (c[1] - a[1]) + c[0] * (a[1] - b[1]));
}

void mat2_inverse(const double* A, double* Ai) {
    // invert_matrix<2> (common_math.h:145-159)
    const double det = A[0] * A[3] - A[1] * A[2];
    if (det == 0.0) throw std::runtime_error("Matrix is singular.");
    const double r = 1.0 / det;
    Ai[0] = A[3] * r;
    Ai[1] = -A[1] * r;
    Ai[2] = -A[2] * r;
    Ai[3] = A[0] * r;
}

void derive_geometry(HostMesh& m) {
    const double* X = m.node_coords.data();
    m.face_area.assign(m.n_faces, 0.0);
    m.cell_volume.assign(m.n_cells, 0.0);
    m.cell_coords.assign(2 * (size_t)m.n_cells, 0.0);
    m.face_normals.assign(2 * (size_t)m.n_faces, 0.0);
    // face lengths (mesh.cpp:218-227)
    for (uint32_t f = 0; f < m.n_faces; ++f) {
        const double* a = X + 2 * (size_t)m.nof[m.off_nof[f]];
        const double* b = X + 2 * (size_t)m.nof[m.off_nof[f] + 1];
        const double dx = b[0] - a[0], dy = b[1] - a[1];
        m.face_area[f] = std::sqrt(dx * dx + dy * dy);
    }
    // cell areas (mesh.cpp:181-216): triangles directly, quads as 0-1-2 + 0-2-3
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        const uint32_t* nd = &m.noc[m.off_noc[c]];
        const uint32_t nn = m.off_noc[c + 1] - m.off_noc[c];
        if (nn == 3) {
            m.cell_volume[c] = tri_area(X + 2 * nd[0], X + 2 * nd[1], X + 2 * nd[2]);
        } else if (nn == 4) {
            const double a1 = tri_area(X + 2 * nd[0], X + 2 * nd[1], X + 2 * nd[2]);
            const double a2 = tri_area(X + 2 * nd[0], X + 2 * nd[2], X + 2 * nd[3]);
            m.cell_volume[c] = a1 + a2;
        } else {
            throw std::runtime_error("Unknown cell type.");
        }
    }
    // vertex centroids (mesh.cpp:167-179)
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        const uint32_t nn = m.off_noc[c + 1] - m.off_noc[c];
        double sx = 0.0, sy = 0.0;
        for (uint32_t i = 0; i < nn; ++i) {
            const uint32_t n = m.noc[m.off_noc[c] + i];
            sx += X[2 * n];
            sy += X[2 * n + 1];
        }
        m.cell_coords[2 * (size_t)c] = sx / nn;
        m.cell_coords[2 * (size_t)c + 1] = sy / nn;
    }
    // area-weighted normals pointing out of cells_of_face(f,0) (mesh.cpp:229-261)
    for (uint32_t f = 0; f < m.n_faces; ++f) {
        const double* a = X + 2 * (size_t)m.nof[m.off_nof[f]];
        const double* b = X + 2 * (size_t)m.nof[m.off_nof[f] + 1];
        const double dx = b[0] - a[0], dy = b[1] - a[1];
        const double len = std::sqrt(dx * dx + dy * dy);
        double nx = dy / len * m.face_area[f];
        double ny = -dx / len * m.face_area[f];
        const int32_t c0 = m.cof[2 * (size_t)f];
        const double ox = 0.5 * (a[0] + b[0]) - m.cell_coords[2 * (size_t)c0];
        const double oy = 0.5 * (a[1] + b[1]) - m.cell_coords[2 * (size_t)c0 + 1];
        if (ox * nx + oy * ny < 0) {
            nx *= -1;
            ny *= -1;
        }
        m.face_normals[2 * (size_t)f] = nx;
        m.face_normals[2 * (size_t)f + 1] = ny;
    }
}

namespace {

void lattice_nodes(HostMesh& m, uint32_t nx, uint32_t ny, double Lx, double Ly) {
    m.n_nodes = (nx + 1) * (ny + 1);
    m.node_coords.assign(2 * (size_t)m.n_nodes, 0.0);
    const double dx = Lx / nx, dy = Ly / ny;
    for (uint32_t i = 0; i <= nx; ++i)
        for (uint32_t j = 0; j <= ny; ++j) {
            const size_t n = (size_t)i * (ny + 1) + j;
            m.node_coords[2 * n] = i * dx;
            m.node_coords[2 * n + 1] = j * dy;
        }
}

// Zones in the reference's order: interior (sorted, deduplicated), right,
// top, left, bottom.
void pack_zones(HostMesh& m, std::vector<uint32_t>& zi, const std::vector<uint32_t>* b4) {
    std::sort(zi.begin(), zi.end());
    zi.erase(std::unique(zi.begin(), zi.end()), zi.end());
    m.zone_off = {0, (uint32_t)zi.size()};
    m.zone_faces = zi;
    for (int z = 0; z < 4; ++z) {
        m.zone_faces.insert(m.zone_faces.end(), b4[z].begin(), b4[z].end());
        m.zone_off.push_back((uint32_t)m.zone_faces.size());
    }
}

void uniform_offsets(std::vector<uint32_t>& off, uint32_t n, uint32_t width) {
    off.resize((size_t)n + 1);
    for (uint32_t i = 0; i <= n; ++i) off[i] = i * width;
}

}  // namespace

HostMesh make_cartesian(uint32_t nx, uint32_t ny, double Lx, double Ly) {
    // Mesh::init_cart (mesh.cpp:305-557)
    HostMesh m;
    m.n_cells = nx * ny;
    m.n_faces = 2 * m.n_cells + nx + ny;
    lattice_nodes(m, nx, ny, Lx, Ly);
    uniform_offsets(m.off_noc, m.n_cells, 4);
    uniform_offsets(m.off_foc, m.n_cells, 4);
    uniform_offsets(m.off_nof, m.n_faces, 2);
    m.noc.assign(4 * (size_t)m.n_cells, 0);
    m.foc.assign(4 * (size_t)m.n_cells, 0);
    m.nof.assign(2 * (size_t)m.n_faces, 0);
    m.cof.assign(2 * (size_t)m.n_faces, 0);
    const uint32_t col = 2 * ny + 1;
    auto face = [&](uint32_t f, int32_t c0, int32_t c1, uint32_t n0, uint32_t n1) {
        m.cof[2 * (size_t)f] = c0;
        m.cof[2 * (size_t)f + 1] = c1;
        m.nof[2 * (size_t)f] = n0;
        m.nof[2 * (size_t)f + 1] = n1;
    };
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        const uint32_t ic = c / ny, jc = c % ny;
        const uint32_t n_tr = (ic + 1) * (ny + 1) + jc + 1, n_tl = ic * (ny + 1) + jc + 1;
        const uint32_t n_bl = ic * (ny + 1) + jc, n_br = (ic + 1) * (ny + 1) + jc;
        const uint32_t f_r = col * (ic + 1) + jc, f_t = col * ic + jc + ny + 1;
        const uint32_t f_l = col * ic + jc, f_b = col * ic + jc + ny;
        const uint32_t nodes[4] = {n_tr, n_tl, n_bl, n_br}, faces[4] = {f_r, f_t, f_l, f_b};
        std::copy(nodes, nodes + 4, &m.noc[4 * (size_t)c]);
        std::copy(faces, faces + 4, &m.foc[4 * (size_t)c]);
        face(f_r, c, ic == nx - 1 ? -1 : (int32_t)(c + ny), n_br, n_tr);
        face(f_t, c, jc == ny - 1 ? -1 : (int32_t)(c + 1), n_tr, n_tl);
        face(f_l, c, ic == 0 ? -1 : (int32_t)(c - ny), n_tl, n_bl);
        face(f_b, c, jc == 0 ? -1 : (int32_t)(c - 1), n_bl, n_br);
    }
    std::vector<uint32_t> zi, zb[4];
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        const uint32_t ic = c / ny, jc = c % ny;
        const uint32_t* fc = &m.foc[4 * (size_t)c];
        (ic == nx - 1 ? zb[0] : zi).push_back(fc[0]);
        (jc == ny - 1 ? zb[1] : zi).push_back(fc[1]);
        (ic == 0 ? zb[2] : zi).push_back(fc[2]);
        (jc == 0 ? zb[3] : zi).push_back(fc[3]);
    }
    pack_zones(m, zi, zb);
    derive_geometry(m);
    return m;
}

HostMesh make_cartesian_tri(uint32_t nx, uint32_t ny, double Lx, double Ly) {
    // Mesh::init_cart_tri (mesh.cpp:559-826).  The reference allocates
    // 3*n_cells+nx+ny faces but numbers only 1.5*n_cells+nx+ny of them; the
    // unused ones keep zero nodes/cells and get NaN normals, and belong to no
    // zone.  They are kept so that face numbers match the reference.
    HostMesh m;
    m.n_cells = 2 * nx * ny;
    m.n_faces = 3 * m.n_cells + nx + ny;
    lattice_nodes(m, nx, ny, Lx, Ly);
    uniform_offsets(m.off_noc, m.n_cells, 3);
    uniform_offsets(m.off_foc, m.n_cells, 3);
    uniform_offsets(m.off_nof, m.n_faces, 2);
    m.noc.assign(3 * (size_t)m.n_cells, 0);
    m.foc.assign(3 * (size_t)m.n_cells, 0);
    m.nof.assign(2 * (size_t)m.n_faces, 0);
    m.cof.assign(2 * (size_t)m.n_faces, 0);
    const uint32_t col = 3 * ny + 1;
    auto face = [&](uint32_t f, int32_t c0, int32_t c1, uint32_t n0, uint32_t n1) {
        m.cof[2 * (size_t)f] = c0;
        m.cof[2 * (size_t)f + 1] = c1;
        m.nof[2 * (size_t)f] = n0;
        m.nof[2 * (size_t)f + 1] = n1;
    };
    for (uint32_t q = 0; q < nx * ny; ++q) {
        const uint32_t ic = q / ny, jc = q % ny;
        const uint32_t cr = 2 * q, cl = cr + 1;  // lower-right and upper-left triangles
        const uint32_t n_tr = (ic + 1) * (ny + 1) + jc + 1, n_tl = ic * (ny + 1) + jc + 1;
        const uint32_t n_bl = ic * (ny + 1) + jc, n_br = (ic + 1) * (ny + 1) + jc;
        const uint32_t f_r = col * (ic + 1) + jc, f_t = col * ic + 2 * jc + ny + 2;
        const uint32_t f_l = col * ic + jc, f_b = col * ic + 2 * jc + ny, f_d = col * ic + 2 * jc + ny + 1;
        uint32_t* ncr = &m.noc[3 * (size_t)cr];
        uint32_t* ncl = &m.noc[3 * (size_t)cl];
        ncr[0] = n_br; ncr[1] = n_tr; ncr[2] = n_bl;
        ncl[0] = n_tl; ncl[1] = n_bl; ncl[2] = n_tr;
        uint32_t* fcr = &m.foc[3 * (size_t)cr];
        uint32_t* fcl = &m.foc[3 * (size_t)cl];
        fcr[0] = f_b; fcr[1] = f_r; fcr[2] = f_d;
        fcl[0] = f_t; fcl[1] = f_l; fcl[2] = f_d;
        face(f_r, cr, ic == nx - 1 ? -1 : (int32_t)(cl + 2 * ny), n_br, n_tr);
        face(f_t, cl, jc == ny - 1 ? -1 : (int32_t)(cl + 1), n_tr, n_tl);
        face(f_l, cl, ic == 0 ? -1 : (int32_t)(cr - 2 * ny), n_tl, n_bl);
        face(f_b, cr, jc == 0 ? -1 : (int32_t)(cr - 1), n_bl, n_br);
        face(f_d, cr, cl, n_bl, n_tr);
    }
    std::vector<uint32_t> zi, zb[4];
    for (uint32_t q = 0; q < nx * ny; ++q) {
        const uint32_t ic = q / ny, jc = q % ny;
        const uint32_t* fcr = &m.foc[3 * (size_t)(2 * q)];
        const uint32_t* fcl = &m.foc[3 * (size_t)(2 * q + 1)];
        (ic == nx - 1 ? zb[0] : zi).push_back(fcr[1]);
        (jc == ny - 1 ? zb[1] : zi).push_back(fcl[0]);
        (ic == 0 ? zb[2] : zi).push_back(fcl[1]);
        (jc == 0 ? zb[3] : zi).push_back(fcr[0]);
        zi.push_back(fcr[2]);
    }
    pack_zones(m, zi, zb);
    derive_geometry(m);
    return m;
}

HostMesh make_wedge(uint32_t nx, uint32_t ny, double Lx, double Ly) {
    // Mesh::init_wedge (mesh.cpp:828-848): nodes right of x = 0.5 are sheared
    // onto an 8 degree ramp.
    HostMesh m = make_cartesian(nx, ny, Lx, Ly);
    const double theta = 8 * 3.14159265358979323846 / 180.0, x_ramp = 0.5;
    for (uint32_t n = 0; n < m.n_nodes; ++n) {
        const double x = m.node_coords[2 * (size_t)n], y = m.node_coords[2 * (size_t)n + 1];
        if (x > x_ramp) {
            const double yb = (x - x_ramp) * std::tan(theta);
            m.node_coords[2 * (size_t)n + 1] = (y / Ly) * (Ly - yb) + yb;
        }
    }
    derive_geometry(m);
    return m;
}

// Triangulated channel [0, Lx] x [yb(x), Ly] whose lower wall rises as a
// ramp of angle ramp_deg from x = x0 (no reference counterpart).  Nodes form
// an (nx+1) x (ny+1) lattice mapped onto the channel; interior nodes move by
// a seeded uniform jitter of up to +-jitter of the local spacing in x and y.
// Each lattice quad is split along its Delaunay diagonal, then edges are
// flipped until the triangulation is Delaunay.
// Zones: 0 interior, 1 inflow (x = 0), 2 outflow (x = Lx), 3 lower wall,
// 4 upper wall.
HostMesh make_ramp_channel(uint32_t nx, uint32_t ny, double Lx, double Ly, double x0, double ramp_deg, double jitter,
                           uint64_t seed) {
    if (jitter < 0 || jitter >= 0.5) throw std::runtime_error("ramp channel: jitter must be in [0, 0.5)");
    const double tn = std::tan(ramp_deg * 3.14159265358979323846 / 180.0);
    if (!(Ly > (Lx - x0) * tn)) throw std::runtime_error("ramp channel: the ramp reaches the upper wall");
    HostMesh m;
    const uint32_t W = nx + 1;
    m.n_nodes = W * (ny + 1);
    m.node_coords.resize(2 * (size_t)m.n_nodes);
    std::mt19937_64 rng(seed);
    auto unit = [&]() { return (double)(rng() >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0; };  // [-1, 1)
    const double hx = Lx / nx;
    for (uint32_t j = 0; j <= ny; ++j)
        for (uint32_t i = 0; i <= nx; ++i) {
            double x = i * hx;
            const bool inner = i > 0 && i < nx && j > 0 && j < ny;
            const double jx = inner ? unit() * jitter : 0.0, jy = inner ? unit() * jitter : 0.0;
            x += jx * hx;
            const double yb = x > x0 ? (x - x0) * tn : 0.0;
            const double hy = (Ly - yb) / ny;
            const double y = yb + (j + jy) * hy;
            m.node_coords[2 * ((size_t)j * W + i)] = x;
            m.node_coords[2 * ((size_t)j * W + i) + 1] = y;
        }
    const double* X = m.node_coords.data();
    // in-circle determinant of d against the counter-clockwise triangle (a, b, c)
    auto incircle = [&](uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
        const double adx = X[2 * a] - X[2 * d], ady = X[2 * a + 1] - X[2 * d + 1];
        const double bdx = X[2 * b] - X[2 * d], bdy = X[2 * b + 1] - X[2 * d + 1];
        const double cdx = X[2 * c] - X[2 * d], cdy = X[2 * c + 1] - X[2 * d + 1];
        return (adx * adx + ady * ady) * (bdx * cdy - cdx * bdy) - (bdx * bdx + bdy * bdy) * (adx * cdy - cdx * ady) +
               (cdx * cdx + cdy * cdy) * (adx * bdy - bdx * ady);
    };
    m.n_cells = 2 * nx * ny;
    m.off_noc.resize(m.n_cells + 1);
    m.noc.resize(3 * (size_t)m.n_cells);
    for (uint32_t j = 0; j < ny; ++j)
        for (uint32_t i = 0; i < nx; ++i) {
            const uint32_t a = j * W + i, b = a + 1, c = a + W + 1, d = a + W;
            const size_t t = 2 * ((size_t)j * nx + i);
            uint32_t* q = &m.noc[3 * t];
            if (incircle(a, b, c, d) > 0) {  // d inside: split along b-d
                q[0] = a; q[1] = b; q[2] = d;
                q[3] = b; q[4] = c; q[5] = d;
            } else {
                q[0] = a; q[1] = b; q[2] = c;
                q[3] = a; q[4] = c; q[5] = d;
            }
        }
    for (uint32_t c = 0; c <= m.n_cells; ++c) m.off_noc[c] = 3 * c;
    // Lawson flips: where the lattice is sheared or compressed (over the
    // ramp) a quad's diagonal is not enough; flip every interior edge whose
    // opposite vertex lies inside the neighbour's circumcircle until none
    // does.  The channel is convex, so the result is the Delaunay
    // triangulation of the nodes (up to co-circular ties).
    {
        const uint32_t T = m.n_cells;
        std::vector<int64_t> nbr(3 * (size_t)T, -1);  // neighbour triangle*3 + edge across edge k (v_k, v_k+1)
        {
            std::vector<std::pair<uint64_t, uint32_t>> es(3 * (size_t)T);
            for (uint32_t t = 0; t < T; ++t)
                for (int k = 0; k < 3; ++k) {
                    const uint32_t p = m.noc[3 * (size_t)t + k], r = m.noc[3 * (size_t)t + (k + 1) % 3];
                    es[3 * (size_t)t + k] = {((uint64_t)std::min(p, r) << 32) | std::max(p, r), 3 * t + (uint32_t)k};
                }
            std::sort(es.begin(), es.end());
            for (size_t e = 0; e + 1 < es.size(); ++e)
                if (es[e].first == es[e + 1].first) {
                    nbr[es[e].second] = es[e + 1].second;
                    nbr[es[e + 1].second] = es[e].second;
                }
        }
        std::vector<uint32_t> stack(3 * (size_t)T);
        std::iota(stack.begin(), stack.end(), 0u);
        size_t flips = 0;
        const size_t max_flips = 100 * (size_t)T;
        while (!stack.empty()) {
            const uint32_t te = stack.back();
            stack.pop_back();
            const int64_t ue = nbr[te];
            if (ue < 0) continue;
            const uint32_t t = te / 3, k = te % 3, u = (uint32_t)ue / 3, l = (uint32_t)ue % 3;
            uint32_t* A = &m.noc[3 * (size_t)t];
            uint32_t* B = &m.noc[3 * (size_t)u];
            const uint32_t a = A[k], b = A[(k + 1) % 3], c = A[(k + 2) % 3];  // edge a-b, t = (a, b, c) ccw
            const uint32_t d = B[(l + 2) % 3];                              // u = (b, a, d) ccw
            if (!(incircle(a, b, c, d) > 0)) continue;
            if (++flips > max_flips) throw std::runtime_error("ramp channel: edge flips did not converge");
            // neighbours of the outer edges before the flip
            const int64_t n_bc = nbr[3 * (size_t)t + (k + 1) % 3], n_ca = nbr[3 * (size_t)t + (k + 2) % 3];
            const int64_t n_ad = nbr[3 * (size_t)u + (l + 1) % 3], n_db = nbr[3 * (size_t)u + (l + 2) % 3];
            // new t = (c, a, d), new u = (d, b, c); edges: t0 c-a, t1 a-d, t2 d-c; u0 d-b, u1 b-c, u2 c-d
            A[0] = c; A[1] = a; A[2] = d;
            B[0] = d; B[1] = b; B[2] = c;
            auto link = [&](uint32_t x, int64_t y) {
                nbr[x] = y;
                if (y >= 0) nbr[(size_t)y] = x;
            };
            link(3 * t + 0, n_ca);
            link(3 * t + 1, n_ad);
            link(3 * t + 2, 3 * (int64_t)u + 2);
            link(3 * u + 0, n_db);
            link(3 * u + 1, n_bc);
            for (uint32_t x : {3 * t + 0, 3 * t + 1, 3 * u + 0, 3 * u + 1}) stack.push_back(x);
        }
    }
    // faces: unique edges, numbered in order of first appearance
    std::vector<std::pair<uint64_t, uint32_t>> edges(3 * (size_t)m.n_cells);  // (key, cell*3 + k)
    for (uint32_t c = 0; c < m.n_cells; ++c)
        for (int k = 0; k < 3; ++k) {
            const uint32_t p = m.noc[3 * (size_t)c + k], r = m.noc[3 * (size_t)c + (k + 1) % 3];
            const uint64_t key = ((uint64_t)std::min(p, r) << 32) | std::max(p, r);
            edges[3 * (size_t)c + k] = {key, 3 * c + (uint32_t)k};
        }
    std::sort(edges.begin(), edges.end());
    m.foc.assign(3 * (size_t)m.n_cells, 0);
    std::vector<uint32_t> first;  // face -> first (cell*3+k) slot
    std::vector<int32_t> second;
    for (size_t e = 0; e < edges.size();) {
        size_t g = e + 1;
        while (g < edges.size() && edges[g].first == edges[e].first) ++g;
        if (g - e > 2) throw std::runtime_error("ramp channel: an edge is shared by more than two triangles");
        first.push_back(std::min(edges[e].second, g - e == 2 ? edges[e + 1].second : edges[e].second));
        second.push_back(g - e == 2 ? (int32_t)std::max(edges[e].second, edges[e + 1].second) : -1);
        e = g;
    }
    // renumber faces by first appearance
    std::vector<uint32_t> order(first.size());
    std::iota(order.begin(), order.end(), 0u);
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return first[a] < first[b]; });
    m.n_faces = (uint32_t)order.size();
    m.cof.assign(2 * (size_t)m.n_faces, -1);
    m.off_nof.resize(m.n_faces + 1);
    m.nof.resize(2 * (size_t)m.n_faces);
    for (uint32_t f = 0; f < m.n_faces; ++f) {
        const uint32_t o = order[f];
        const uint32_t s0 = first[o];
        const uint32_t c0 = s0 / 3, k0 = s0 % 3;
        m.cof[2 * (size_t)f] = (int32_t)c0;
        m.foc[s0] = f;
        m.nof[2 * (size_t)f] = m.noc[3 * (size_t)c0 + k0];
        m.nof[2 * (size_t)f + 1] = m.noc[3 * (size_t)c0 + (k0 + 1) % 3];
        if (second[o] >= 0) {
            m.cof[2 * (size_t)f + 1] = second[o] / 3;
            m.foc[(size_t)second[o]] = f;
        }
        m.off_nof[f] = 2 * f;
    }
    m.off_nof[m.n_faces] = 2 * m.n_faces;
    m.off_foc.resize(m.n_cells + 1);
    for (uint32_t c = 0; c <= m.n_cells; ++c) m.off_foc[c] = 3 * c;
    // zones
    std::vector<std::vector<uint32_t>> zones(5);
    for (uint32_t f = 0; f < m.n_faces; ++f) {
        if (m.cof[2 * (size_t)f + 1] >= 0) {
            zones[0].push_back(f);
            continue;
        }
        const uint32_t p = m.nof[2 * (size_t)f], r = m.nof[2 * (size_t)f + 1];
        const uint32_t ip = p % W, jp = p / W, ir = r % W, jr = r / W;
        if (ip == 0 && ir == 0) zones[1].push_back(f);
        else if (ip == nx && ir == nx) zones[2].push_back(f);
        else if (jp == 0 && jr == 0) zones[3].push_back(f);
        else if (jp == ny && jr == ny) zones[4].push_back(f);
        else throw std::runtime_error("ramp channel: boundary face off the boundary");
    }
    m.zone_off.assign(1, 0);
    for (auto& z : zones) {
        m.zone_faces.insert(m.zone_faces.end(), z.begin(), z.end());
        m.zone_off.push_back((uint32_t)m.zone_faces.size());
    }
    derive_geometry(m);
    for (uint32_t c = 0; c < m.n_cells; ++c)
        if (!(m.cell_volume[c] > 0)) throw std::runtime_error("ramp channel: degenerate triangle");
    return m;
}

}  // namespace mgpu

using mgpu::HostMesh;

extern "C" {

int mgpu_mesh_generate_ramp(uint32_t nx, uint32_t ny, double Lx, double Ly, double x0, double ramp_deg, double jitter,
                            uint64_t seed, mgpu_mesh_buf** out) {
    if (!out || nx == 0 || ny == 0 || !(Lx > 0) || !(Ly > 0) || !(x0 >= 0) || !(x0 < Lx)) {
        mgpu::set_error("mgpu_mesh_generate_ramp: invalid arguments");
        return MGPU_ERR_ARG;
    }
    try {
        auto* b = new mgpu_mesh_buf();
        try {
            b->m = mgpu::make_ramp_channel(nx, ny, Lx, Ly, x0, ramp_deg, jitter, seed);
        } catch (...) {
            delete b;
            throw;
        }
        b->zone_names = {"interior", "inflow", "outflow", "wall", "top"};
        *out = b;
        return MGPU_OK;
    } catch (const std::exception& e) {
        mgpu::set_error(e.what());
        return MGPU_ERR_ARG;
    }
}

int mgpu_mesh_generate(int mesh_type, uint32_t nx, uint32_t ny, double Lx, double Ly, mgpu_mesh_buf** out) {
    if (!out || nx == 0 || ny == 0 || !(Lx > 0) || !(Ly > 0)) {
        mgpu::set_error("mgpu_mesh_generate: invalid arguments");
        return MGPU_ERR_ARG;
    }
    try {
        auto* b = new mgpu_mesh_buf();
        if (mesh_type == MGPU_MESH_CARTESIAN) b->m = mgpu::make_cartesian(nx, ny, Lx, Ly);
        else if (mesh_type == MGPU_MESH_CARTESIAN_TRI) b->m = mgpu::make_cartesian_tri(nx, ny, Lx, Ly);
        else if (mesh_type == MGPU_MESH_WEDGE) b->m = mgpu::make_wedge(nx, ny, Lx, Ly);
        else {
            delete b;
            mgpu::set_error("Unknown mesh type.");
            return MGPU_ERR_ARG;
        }
        mgpu::default_zone_names(*b);
        *out = b;
        return MGPU_OK;
    } catch (const std::exception& e) {
        mgpu::set_error(e.what());
        return MGPU_ERR_HOST;
    }
}

int mgpu_mesh_from_connectivity(uint32_t n_nodes, const double* node_coords, uint32_t n_cells,
                                const uint32_t* offsets_nodes_of_cell, const uint32_t* nodes_of_cell,
                                const uint32_t* offsets_faces_of_cell, const uint32_t* faces_of_cell,
                                uint32_t n_faces, const uint32_t* offsets_nodes_of_face,
                                const uint32_t* nodes_of_face, const int32_t* cells_of_face, uint32_t n_zones,
                                const uint32_t* zone_offsets, const uint32_t* zone_faces, mgpu_mesh_buf** out) {
    if (!out || !node_coords || !offsets_nodes_of_cell || !nodes_of_cell || !offsets_faces_of_cell ||
        !faces_of_cell || !offsets_nodes_of_face || !nodes_of_face || !cells_of_face || !zone_offsets ||
        n_zones == 0) {
        mgpu::set_error("mgpu_mesh_from_connectivity: null array");
        return MGPU_ERR_ARG;
    }
    try {
        auto* b = new mgpu_mesh_buf();
        HostMesh& m = b->m;
        m.n_nodes = n_nodes;
        m.n_cells = n_cells;
        m.n_faces = n_faces;
        m.node_coords.assign(node_coords, node_coords + 2 * (size_t)n_nodes);
        m.off_noc.assign(offsets_nodes_of_cell, offsets_nodes_of_cell + n_cells + 1);
        m.noc.assign(nodes_of_cell, nodes_of_cell + m.off_noc.back());
        m.off_foc.assign(offsets_faces_of_cell, offsets_faces_of_cell + n_cells + 1);
        m.foc.assign(faces_of_cell, faces_of_cell + m.off_foc.back());
        m.off_nof.assign(offsets_nodes_of_face, offsets_nodes_of_face + n_faces + 1);
        m.nof.assign(nodes_of_face, nodes_of_face + m.off_nof.back());
        m.cof.assign(cells_of_face, cells_of_face + 2 * (size_t)n_faces);
        m.zone_off.assign(zone_offsets, zone_offsets + n_zones + 1);
        m.zone_faces.assign(zone_faces, zone_faces + m.zone_off.back());
        for (uint32_t n : m.noc)
            if (n >= n_nodes) throw std::runtime_error("mesh: node index out of range");
        for (uint32_t f : m.foc)
            if (f >= n_faces) throw std::runtime_error("mesh: face index out of range");
        for (uint32_t f : m.zone_faces)
            if (f >= n_faces) throw std::runtime_error("mesh: zone face out of range");
        for (size_t i = 0; i < m.cof.size(); ++i)
            if (m.cof[i] >= (int32_t)n_cells || (m.cof[i] < 0 && (i % 2 == 0 || m.cof[i] != -1)))
                throw std::runtime_error("mesh: cells_of_face out of range");
        mgpu::derive_geometry(m);
        mgpu::default_zone_names(*b);
        *out = b;
        return MGPU_OK;
    } catch (const std::exception& e) {
        mgpu::set_error(e.what());
        return MGPU_ERR_ARG;
    }
}

int mgpu_mesh_permute_cells(mgpu_mesh_buf* b, uint64_t seed, uint32_t* new_of_old) {
    if (!b) {
        mgpu::set_error("mgpu_mesh_permute_cells: null mesh");
        return MGPU_ERR_ARG;
    }
    HostMesh& m = b->m;
    const uint32_t n = m.n_cells;
    std::vector<uint32_t> perm(n);  // perm[old] = new
    for (uint32_t i = 0; i < n; ++i) perm[i] = i;
    std::mt19937_64 rng(seed);
    for (uint32_t i = n; i > 1; --i) {
        const uint32_t j = (uint32_t)(rng() % i);
        std::swap(perm[i - 1], perm[j]);
    }
    std::vector<uint32_t> old_of_new(n);
    for (uint32_t i = 0; i < n; ++i) old_of_new[perm[i]] = i;
    auto relabel_csr = [&](std::vector<uint32_t>& off, std::vector<uint32_t>& flat) {
        std::vector<uint32_t> o2(n + 1, 0), f2;
        f2.reserve(flat.size());
        for (uint32_t c = 0; c < n; ++c) {
            const uint32_t old = old_of_new[c];
            f2.insert(f2.end(), flat.begin() + off[old], flat.begin() + off[old + 1]);
            o2[c + 1] = (uint32_t)f2.size();
        }
        off.swap(o2);
        flat.swap(f2);
    };
    relabel_csr(m.off_noc, m.noc);
    relabel_csr(m.off_foc, m.foc);
    std::vector<double> cc(m.cell_coords.size()), cv(m.cell_volume.size());
    for (uint32_t c = 0; c < n; ++c) {
        const uint32_t old = old_of_new[c];
        cc[2 * (size_t)c] = m.cell_coords[2 * (size_t)old];
        cc[2 * (size_t)c + 1] = m.cell_coords[2 * (size_t)old + 1];
        cv[c] = m.cell_volume[old];
    }
    m.cell_coords.swap(cc);
    m.cell_volume.swap(cv);
    // Faces keep their numbers; only the cell labels on them change.  Faces
    // outside every zone (the reference's unused slots) keep their zero cells.
    std::vector<char> used(m.n_faces, 0);
    for (uint32_t f : m.zone_faces) used[f] = 1;
    for (uint32_t f = 0; f < m.n_faces; ++f) {
        if (!used[f]) continue;
        for (int s = 0; s < 2; ++s) {
            int32_t& c = m.cof[2 * (size_t)f + s];
            if (c >= 0) c = (int32_t)perm[c];
        }
    }
    if (new_of_old) std::copy(perm.begin(), perm.end(), new_of_old);
    return MGPU_OK;
}

int mgpu_mesh_view(const mgpu_mesh_buf* b, mgpu_mesh* view) {
    if (!b || !view) {
        mgpu::set_error("mgpu_mesh_view: null argument");
        return MGPU_ERR_ARG;
    }
    *view = b->m.view();
    return MGPU_OK;
}

void mgpu_mesh_free(mgpu_mesh_buf* b) { delete b; }

}  // extern "C"
