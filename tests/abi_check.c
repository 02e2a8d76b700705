/* A plain-C client of the C ABI (include/mallard_gb300.h): the header must
 * compile as C99 and the host-only entry points must work without a GPU.
 * Generates the reference's 16 x 16 cartesian_tri mesh, builds its TENO
 * tables on the host, writes and reads the binary mesh format, writes a VTU
 * file, and prints a summary line the test checks. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "mallard_gb300.h"

static int fail(const char* what) {
    fprintf(stderr, "%s: %s\n", what, mgpu_last_error());
    return 1;
}

int main(int argc, char** argv) {
    const char* dir = argc > 1 ? argv[1] : ".";
    char path[4096];
    mgpu_config cfg;
    mgpu_config_defaults(&cfg);
    if (cfg.recon != MGPU_RECON_TENO || cfg.poly_order != 3 || cfg.time_integrator != MGPU_INTEGRATOR_SSPRK3)
        return fail("defaults");
    mgpu_mesh_buf* buf = NULL;
    if (mgpu_mesh_generate(MGPU_MESH_CARTESIAN_TRI, 16, 16, 1.0, 1.0, &buf) != MGPU_OK) return fail("generate");
    mgpu_mesh v;
    if (mgpu_mesh_view(buf, &v) != MGPU_OK) return fail("view");
    char zone[64];
    if (mgpu_mesh_zone_name(buf, 1, zone, sizeof zone) != MGPU_OK) return fail("zone name");
    mgpu_teno_tables* t = NULL;
    if (mgpu_teno_tables_build(&v, MGPU_BASIS_LEGENDRE, 3, 2.0, 0, 0, &t) != MGPU_OK) return fail("tables");
    const uint64_t n_mat = mgpu_teno_tables_len(t, MGPU_TENO_MATRICES);
    double* oi = (double*)malloc(sizeof(double) * mgpu_teno_tables_len(t, MGPU_TENO_OSCILLATION_INDICATOR));
    if (mgpu_teno_tables_copy(t, MGPU_TENO_OSCILLATION_INDICATOR, oi) != MGPU_OK) return fail("copy");
    snprintf(path, sizeof path, "%s/mesh.mgm", dir);
    if (mgpu_mesh_write(buf, path) != MGPU_OK) return fail("write");
    mgpu_mesh_buf* back = NULL;
    if (mgpu_mesh_read(path, &back) != MGPU_OK) return fail("read");
    mgpu_mesh w;
    mgpu_mesh_view(back, &w);
    double* rho = (double*)malloc(sizeof(double) * v.n_cells);
    for (uint32_t c = 0; c < v.n_cells; ++c) rho[c] = 1.0 + v.cell_coords[2 * c];
    const char* names[1] = {"RHO"};
    snprintf(path, sizeof path, "%s/rho_000000.vtu", dir);
    if (mgpu_vtu_write(buf, path, 1, names, rho) != MGPU_OK) return fail("vtu");
    /* a bad argument comes back as a status code with a message */
    mgpu_mesh_buf* none = NULL;
    const int bad = mgpu_mesh_generate(99, 4, 4, 1.0, 1.0, &none) == MGPU_ERR_ARG && none == NULL;
    printf("cells=%u faces=%u zones=%u zone1=%s matrices=%llu oi11=%.17g read_cells=%u bad_arg=%d version=%d\n",
           v.n_cells, v.n_faces, v.n_zones, zone, (unsigned long long)n_mat, oi[11], w.n_cells, bad, mgpu_version());
    free(oi);
    free(rho);
    mgpu_teno_tables_free(t);
    mgpu_mesh_free(back);
    mgpu_mesh_free(buf);
    return 0;
}
