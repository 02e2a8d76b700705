// The GPU stencil search's per-cell routine (search_cell, stencil_search.cu)
// compiled for the host, for a CPU test against the host search
// (host_teno.cpp): search_host runs it over every cell of a mesh.
#include "../mallard_gb300/csrc/stencil_search.cu"

extern "C" int search_host(const mgpu_mesh* m, const uint32_t* goff, const uint32_t* gnb, int M, uint32_t* flat,
                           uint8_t* sizes, uint8_t* status) {
    mgpu::SearchArgs a{};
    a.goff = goff;
    a.gnb = gnb;
    a.X = m->cell_coords;
    a.nodes = m->node_coords;
    a.ofc = m->offsets_faces_of_cell;
    a.foc = m->faces_of_cell;
    a.cof = m->cells_of_face;
    a.onf = m->offsets_nodes_of_face;
    a.nof = m->nodes_of_face;
    a.n_cells = m->n_cells;
    a.M = M;
    a.flat = flat;
    a.sizes = sizes;
    a.status = status;
    static mgpu::Scratch w;
    int redo = 0;
    for (uint32_t c = 0; c < m->n_cells; ++c) {
        int sz[4] = {0, 0, 0, 0};
        const bool ok = mgpu::search_cell(a, c, w, sz);
        for (int s = 0; s < 4; ++s) sizes[(size_t)c * 4 + s] = ok ? (uint8_t)sz[s] : 0;
        status[c] = ok ? 0 : 1;
        redo += !ok;
    }
    return redo;
}
