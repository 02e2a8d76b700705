// host_mesh_io.cpp -- mesh ingest: the Gmsh reader the reference's "file"
// mesh type names (src/mesh/mesh.cpp:41-43 reads [mesh] filename, default
// "mesh.msh", then throws "MeshType::FILE not implemented."), a binary mesh
// format of the library's own, and zone names.
//
// Gmsh: ASCII MSH 2.2 and 4.1, two-dimensional meshes.  Triangles (element
// type 2) and quadrilaterals (type 3) become cells in file order; line
// elements (type 1) name the boundary zones, by their physical group
// ($PhysicalNames), else by their geometric entity.  Faces are built from
// the cells' edges (build_faces); geometry is derived with the reference's
// formulas (derive_geometry).
//
// Binary: "MGPUMSH1", a byte-order word, the counts, the reference Mesh's
// connectivity arrays (mesh.h:228-253) as stored, the zone names; geometry is
// derived again on reading, so a round trip returns the same bits.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "host.h"

namespace mgpu {

void default_zone_names(mgpu_mesh_buf& b) {
    const uint32_t nz = (uint32_t)b.m.zone_off.size() - 1;
    if (b.zone_names.size() == nz) return;
    b.zone_names.clear();
    if (nz == 5) {
        b.zone_names = {"interior", "right", "top", "left", "bottom"};
        return;
    }
    for (uint32_t i = 0; i < nz; ++i) b.zone_names.push_back(i == 0 ? "interior" : "zone" + std::to_string(i));
}

static uint64_t edge_key(uint32_t a, uint32_t b) {
    return a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
}

void build_faces(mgpu_mesh_buf& buf, const std::vector<std::pair<uint64_t, uint32_t>>& edge_zone,
                 const std::vector<std::string>& names) {
    HostMesh& m = buf.m;
    std::unordered_map<uint64_t, uint32_t> face_of;
    face_of.reserve((size_t)m.n_cells * 2);
    m.off_foc.assign((size_t)m.n_cells + 1, 0);
    m.foc.clear();
    m.nof.clear();
    m.cof.clear();
    for (uint32_t c = 0; c < m.n_cells; ++c) {
        const uint32_t n0 = m.off_noc[c], nn = m.off_noc[c + 1] - n0;
        for (uint32_t k = 0; k < nn; ++k) {
            const uint32_t a = m.noc[n0 + k], b = m.noc[n0 + (k + 1) % nn];
            const uint64_t key = edge_key(a, b);
            auto it = face_of.find(key);
            uint32_t f;
            if (it == face_of.end()) {
                f = (uint32_t)(m.nof.size() / 2);
                face_of.emplace(key, f);
                m.nof.push_back(a);
                m.nof.push_back(b);
                m.cof.push_back((int32_t)c);
                m.cof.push_back(-1);
            } else {
                f = it->second;
                if (m.cof[2 * (size_t)f + 1] != -1) throw std::runtime_error("mesh: an edge is shared by more than two cells");
                m.cof[2 * (size_t)f + 1] = (int32_t)c;
            }
            m.foc.push_back(f);
        }
        m.off_foc[c + 1] = (uint32_t)m.foc.size();
    }
    m.n_faces = (uint32_t)(m.nof.size() / 2);
    m.off_nof.resize((size_t)m.n_faces + 1);
    for (uint32_t f = 0; f <= m.n_faces; ++f) m.off_nof[f] = 2 * f;
    // zones: interior, the named boundary zones in order, then "boundary"
    std::unordered_map<uint64_t, uint32_t> zone_of_edge(edge_zone.begin(), edge_zone.end());
    std::vector<std::vector<uint32_t>> zf(names.size() + 2);
    for (uint32_t f = 0; f < m.n_faces; ++f) {
        if (m.cof[2 * (size_t)f + 1] >= 0) {
            zf[0].push_back(f);
            continue;
        }
        auto it = zone_of_edge.find(edge_key(m.nof[2 * (size_t)f], m.nof[2 * (size_t)f + 1]));
        zf[it == zone_of_edge.end() ? names.size() + 1 : it->second].push_back(f);
    }
    buf.zone_names.assign(1, "interior");
    m.zone_off.assign(1, 0);
    m.zone_faces.clear();
    for (size_t z = 0; z < zf.size(); ++z) {
        if (z > 0 && zf[z].empty()) continue;  // boundary groups with no face of this mesh
        if (z > 0) buf.zone_names.push_back(z <= names.size() ? names[z - 1] : "boundary");
        m.zone_faces.insert(m.zone_faces.end(), zf[z].begin(), zf[z].end());
        m.zone_off.push_back((uint32_t)m.zone_faces.size());
    }
    derive_geometry(m);
}

namespace {

struct GmshData {
    std::vector<double> xy;                       // node coordinates
    std::unordered_map<uint64_t, uint32_t> node;  // file tag -> index
    std::vector<uint32_t> off{0}, cells;          // cells (file node tags)
    std::vector<std::pair<uint64_t, uint64_t>> lines;  // boundary line (tags)
    std::vector<int> line_group;                  // its zone key
    std::map<int, std::string> phys_names;        // dim-1 physical tag -> name
};

void expect(std::istream& in, const char* word) {
    std::string s;
    if (!(in >> s) || s != word) throw std::runtime_error(std::string("gmsh: expected ") + word);
}

void skip_section(std::istream& in, const std::string& head) {
    const std::string end = "$End" + head.substr(1);
    std::string s;
    while (in >> s)
        if (s == end) return;
    throw std::runtime_error("gmsh: unterminated section " + head);
}

void add_element(GmshData& g, int type, const std::vector<uint64_t>& nodes, int group) {
    if (type == 2 || type == 3) {
        for (uint64_t t : nodes) {
            auto it = g.node.find(t);
            if (it == g.node.end()) throw std::runtime_error("gmsh: element refers to an unknown node");
            g.cells.push_back(it->second);
        }
        g.off.push_back((uint32_t)g.cells.size());
    } else if (type == 1) {
        g.lines.emplace_back(nodes[0], nodes[1]);
        g.line_group.push_back(group);
    } else if (type == 15) {
        // points: ignored
    } else {
        throw std::runtime_error("gmsh: element type " + std::to_string(type) +
                                 " not supported (2-D meshes of triangles, quadrilaterals and boundary lines)");
    }
}

int nodes_per(int type) {
    switch (type) {
        case 1: return 2;
        case 2: return 3;
        case 3: return 4;
        case 15: return 1;
    }
    return -1;
}

void read_v2(std::istream& in, GmshData& g) {
    std::string s;
    while (in >> s) {
        if (s == "$PhysicalNames") {
            size_t n;
            in >> n;
            for (size_t i = 0; i < n; ++i) {
                int dim, tag;
                std::string name;
                in >> dim >> tag;
                std::getline(in, name);
                const size_t a = name.find('"'), b = name.rfind('"');
                if (dim == 1) g.phys_names[tag] = (a != std::string::npos && b > a) ? name.substr(a + 1, b - a - 1) : name;
            }
            expect(in, "$EndPhysicalNames");
        } else if (s == "$Nodes") {
            size_t n;
            in >> n;
            for (size_t i = 0; i < n; ++i) {
                uint64_t tag;
                double x, y, z;
                if (!(in >> tag >> x >> y >> z)) throw std::runtime_error("gmsh: truncated $Nodes");
                g.node[tag] = (uint32_t)(g.xy.size() / 2);
                g.xy.push_back(x);
                g.xy.push_back(y);
            }
            expect(in, "$EndNodes");
        } else if (s == "$Elements") {
            size_t n;
            in >> n;
            for (size_t i = 0; i < n; ++i) {
                uint64_t tag;
                int type, ntags;
                if (!(in >> tag >> type >> ntags)) throw std::runtime_error("gmsh: truncated $Elements");
                std::vector<int> tags(ntags);
                for (int& t : tags) in >> t;
                const int nn = nodes_per(type);
                if (nn < 0) throw std::runtime_error("gmsh: element type " + std::to_string(type) + " not supported");
                std::vector<uint64_t> nodes(nn);
                for (auto& v : nodes) in >> v;
                // group: physical tag when there is one, else -(elementary tag) - 1
                const int group = ntags >= 1 && tags[0] != 0 ? tags[0] : -(ntags >= 2 ? tags[1] : 0) - 1;
                add_element(g, type, nodes, group);
            }
            expect(in, "$EndElements");
        } else if (!s.empty() && s[0] == '$' && s.compare(0, 4, "$End") != 0) {
            skip_section(in, s);
        }
    }
}

void read_v4(std::istream& in, GmshData& g) {
    std::map<int, int> curve_phys;  // curve entity -> first physical tag (0: none)
    std::string s;
    while (in >> s) {
        if (s == "$PhysicalNames") {
            size_t n;
            in >> n;
            for (size_t i = 0; i < n; ++i) {
                int dim, tag;
                std::string name;
                in >> dim >> tag;
                std::getline(in, name);
                const size_t a = name.find('"'), b = name.rfind('"');
                if (dim == 1) g.phys_names[tag] = (a != std::string::npos && b > a) ? name.substr(a + 1, b - a - 1) : name;
            }
            expect(in, "$EndPhysicalNames");
        } else if (s == "$Entities") {
            size_t np, nc, ns, nv;
            in >> np >> nc >> ns >> nv;
            for (size_t i = 0; i < np; ++i) {
                int tag, nph;
                double x, y, z;
                in >> tag >> x >> y >> z >> nph;
                for (int k = 0; k < nph; ++k) in >> tag;
            }
            for (size_t i = 0; i < nc; ++i) {
                int tag, nph, nb;
                double bb[6];
                in >> tag;
                for (double& v : bb) in >> v;
                in >> nph;
                int first = 0;
                for (int k = 0; k < nph; ++k) {
                    int p;
                    in >> p;
                    if (k == 0) first = p;
                }
                in >> nb;
                for (int k = 0; k < nb; ++k) {
                    int t;
                    in >> t;
                }
                curve_phys[tag] = first;
            }
            skip_section(in, "$Entities");
        } else if (s == "$Nodes") {
            size_t blocks, n, lo, hi;
            in >> blocks >> n >> lo >> hi;
            for (size_t b = 0; b < blocks; ++b) {
                int edim, etag, param;
                size_t nb;
                in >> edim >> etag >> param >> nb;
                if (param) throw std::runtime_error("gmsh: parametric nodes not supported");
                std::vector<uint64_t> tags(nb);
                for (auto& t : tags) in >> t;
                for (size_t i = 0; i < nb; ++i) {
                    double x, y, z;
                    if (!(in >> x >> y >> z)) throw std::runtime_error("gmsh: truncated $Nodes");
                    g.node[tags[i]] = (uint32_t)(g.xy.size() / 2);
                    g.xy.push_back(x);
                    g.xy.push_back(y);
                }
            }
            expect(in, "$EndNodes");
        } else if (s == "$Elements") {
            size_t blocks, n, lo, hi;
            in >> blocks >> n >> lo >> hi;
            for (size_t b = 0; b < blocks; ++b) {
                int edim, etag, type;
                size_t nb;
                in >> edim >> etag >> type >> nb;
                const int nn = nodes_per(type);
                if (nn < 0) throw std::runtime_error("gmsh: element type " + std::to_string(type) + " not supported");
                int group = 0;
                if (type == 1) {
                    auto it = curve_phys.find(etag);
                    group = it != curve_phys.end() && it->second != 0 ? it->second : -etag - 1;
                }
                for (size_t i = 0; i < nb; ++i) {
                    uint64_t tag;
                    in >> tag;
                    std::vector<uint64_t> nodes(nn);
                    for (auto& v : nodes) in >> v;
                    add_element(g, type, nodes, group);
                }
            }
            expect(in, "$EndElements");
        } else if (!s.empty() && s[0] == '$' && s.compare(0, 4, "$End") != 0) {
            skip_section(in, s);
        }
    }
}

mgpu_mesh_buf* mesh_from_gmsh(GmshData& g) {
    if (g.off.size() < 2) throw std::runtime_error("gmsh: no triangles or quadrilaterals");
    auto* b = new mgpu_mesh_buf();
    try {
        HostMesh& m = b->m;
        m.n_nodes = (uint32_t)(g.xy.size() / 2);
        m.node_coords = g.xy;
        m.n_cells = (uint32_t)(g.off.size() - 1);
        m.off_noc = g.off;
        m.noc = g.cells;
        // boundary zones: groups in order of first appearance
        std::vector<std::string> names;
        std::map<int, uint32_t> zone_of_group;
        std::vector<std::pair<uint64_t, uint32_t>> edge_zone;
        for (size_t i = 0; i < g.lines.size(); ++i) {
            const int grp = g.line_group[i];
            auto it = zone_of_group.find(grp);
            if (it == zone_of_group.end()) {
                std::string name;
                if (grp > 0) {
                    auto pn = g.phys_names.find(grp);
                    name = pn != g.phys_names.end() ? pn->second : "physical" + std::to_string(grp);
                } else {
                    name = "curve" + std::to_string(-grp - 1);
                }
                it = zone_of_group.emplace(grp, (uint32_t)names.size() + 1).first;
                names.push_back(name);
            }
            auto na = g.node.find(g.lines[i].first), nb = g.node.find(g.lines[i].second);
            if (na == g.node.end() || nb == g.node.end()) throw std::runtime_error("gmsh: line refers to an unknown node");
            edge_zone.emplace_back(edge_key(na->second, nb->second), it->second);
        }
        build_faces(*b, edge_zone, names);
        return b;
    } catch (...) {
        delete b;
        throw;
    }
}

// ---- binary format -----------------------------------------------------------
constexpr char MAGIC[8] = {'M', 'G', 'P', 'U', 'M', 'S', 'H', '1'};
constexpr uint32_t BOM = 0x01020304u;

template <class T>
void put(std::ofstream& f, const std::vector<T>& v) {
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}
template <class T>
void get(std::ifstream& f, std::vector<T>& v, size_t n) {
    v.resize(n);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
    if (!f) throw std::runtime_error("mesh file: truncated");
}

}  // namespace

}  // namespace mgpu

using mgpu::HostMesh;

extern "C" {

int mgpu_mesh_read_gmsh(const char* path, mgpu_mesh_buf** out) {
    if (!path || !out) {
        mgpu::set_error("mgpu_mesh_read_gmsh: null argument");
        return MGPU_ERR_ARG;
    }
    try {
        std::ifstream in(path);
        if (!in) throw std::runtime_error(std::string("cannot open ") + path);
        std::string s, version;
        int ftype = 0, dsize = 0;
        in >> s;
        if (s != "$MeshFormat") throw std::runtime_error("gmsh: no $MeshFormat");
        in >> version >> ftype >> dsize;
        if (ftype != 0) throw std::runtime_error("gmsh: binary MSH files are not supported (save as ASCII)");
        mgpu::expect(in, "$EndMeshFormat");
        mgpu::GmshData g;
        if (version.compare(0, 2, "2.") == 0) mgpu::read_v2(in, g);
        else if (version.compare(0, 2, "4.") == 0) mgpu::read_v4(in, g);
        else throw std::runtime_error("gmsh: MSH version " + version + " not supported (2.2 or 4.1)");
        *out = mgpu::mesh_from_gmsh(g);
        return MGPU_OK;
    } catch (const std::exception& e) {
        mgpu::set_error(e.what());
        return MGPU_ERR_ARG;
    }
}

int mgpu_mesh_write(const mgpu_mesh_buf* b, const char* path) {
    if (!b || !path) {
        mgpu::set_error("mgpu_mesh_write: null argument");
        return MGPU_ERR_ARG;
    }
    try {
        std::ofstream f(path, std::ios::binary);
        if (!f) throw std::runtime_error(std::string("cannot open ") + path);
        const HostMesh& m = b->m;
        const uint32_t nz = (uint32_t)m.zone_off.size() - 1;
        f.write(mgpu::MAGIC, 8);
        const uint32_t head[5] = {mgpu::BOM, m.n_nodes, m.n_cells, m.n_faces, nz};
        f.write(reinterpret_cast<const char*>(head), sizeof(head));
        mgpu::put(f, m.node_coords);
        mgpu::put(f, m.off_noc);
        mgpu::put(f, m.noc);
        mgpu::put(f, m.off_foc);
        mgpu::put(f, m.foc);
        mgpu::put(f, m.off_nof);
        mgpu::put(f, m.nof);
        mgpu::put(f, m.cof);
        mgpu::put(f, m.zone_off);
        mgpu::put(f, m.zone_faces);
        for (uint32_t z = 0; z < nz; ++z) {
            const std::string& nm = z < b->zone_names.size() ? b->zone_names[z] : std::string();
            const uint32_t len = (uint32_t)nm.size();
            f.write(reinterpret_cast<const char*>(&len), 4);
            f.write(nm.data(), len);
        }
        if (!f) throw std::runtime_error(std::string("write failed: ") + path);
        return MGPU_OK;
    } catch (const std::exception& e) {
        mgpu::set_error(e.what());
        return MGPU_ERR_HOST;
    }
}

int mgpu_mesh_read(const char* path, mgpu_mesh_buf** out) {
    if (!path || !out) {
        mgpu::set_error("mgpu_mesh_read: null argument");
        return MGPU_ERR_ARG;
    }
    mgpu_mesh_buf* b = nullptr;
    try {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw std::runtime_error(std::string("cannot open ") + path);
        char magic[8];
        uint32_t head[5];
        f.read(magic, 8);
        f.read(reinterpret_cast<char*>(head), sizeof(head));
        if (!f || std::memcmp(magic, mgpu::MAGIC, 8) != 0) throw std::runtime_error("not a MGPUMSH1 mesh file");
        if (head[0] != mgpu::BOM) throw std::runtime_error("mesh file: other byte order");
        b = new mgpu_mesh_buf();
        HostMesh& m = b->m;
        m.n_nodes = head[1];
        m.n_cells = head[2];
        m.n_faces = head[3];
        const uint32_t nz = head[4];
        mgpu::get(f, m.node_coords, 2 * (size_t)m.n_nodes);
        mgpu::get(f, m.off_noc, (size_t)m.n_cells + 1);
        mgpu::get(f, m.noc, m.off_noc.back());
        mgpu::get(f, m.off_foc, (size_t)m.n_cells + 1);
        mgpu::get(f, m.foc, m.off_foc.back());
        mgpu::get(f, m.off_nof, (size_t)m.n_faces + 1);
        mgpu::get(f, m.nof, m.off_nof.back());
        mgpu::get(f, m.cof, 2 * (size_t)m.n_faces);
        mgpu::get(f, m.zone_off, (size_t)nz + 1);
        mgpu::get(f, m.zone_faces, m.zone_off.back());
        for (uint32_t z = 0; z < nz; ++z) {
            uint32_t len = 0;
            f.read(reinterpret_cast<char*>(&len), 4);
            if (!f || len > 4096) throw std::runtime_error("mesh file: bad zone name");
            std::string nm(len, '\0');
            f.read(&nm[0], len);
            b->zone_names.push_back(nm);
        }
        if (!f) throw std::runtime_error("mesh file: truncated");
        for (uint32_t n : m.noc)
            if (n >= m.n_nodes) throw std::runtime_error("mesh file: node index out of range");
        for (uint32_t x : m.foc)
            if (x >= m.n_faces) throw std::runtime_error("mesh file: face index out of range");
        for (uint32_t x : m.nof)
            if (x >= m.n_nodes) throw std::runtime_error("mesh file: node index out of range");
        for (uint32_t x : m.zone_faces)
            if (x >= m.n_faces) throw std::runtime_error("mesh file: zone face out of range");
        for (int32_t c : m.cof)
            if (c >= (int32_t)m.n_cells || c < -1) throw std::runtime_error("mesh file: cells_of_face out of range");
        mgpu::derive_geometry(m);
        *out = b;
        return MGPU_OK;
    } catch (const std::exception& e) {
        delete b;
        mgpu::set_error(e.what());
        return MGPU_ERR_ARG;
    }
}

int mgpu_mesh_zone_name(const mgpu_mesh_buf* b, uint32_t zone, char* name, uint32_t len) {
    if (!b || !name || len == 0 || zone >= b->zone_names.size()) {
        mgpu::set_error("mgpu_mesh_zone_name: bad argument");
        return MGPU_ERR_ARG;
    }
    std::snprintf(name, len, "%s", b->zone_names[zone].c_str());
    return MGPU_OK;
}

int mgpu_mesh_set_zone_name(mgpu_mesh_buf* b, uint32_t zone, const char* name) {
    if (!b || !name || zone >= b->zone_names.size()) {
        mgpu::set_error("mgpu_mesh_set_zone_name: bad argument");
        return MGPU_ERR_ARG;
    }
    b->zone_names[zone] = name;
    return MGPU_OK;
}

}  // extern "C"
