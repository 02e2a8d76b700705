/*
 * mallard_gb300.h -- C ABI of the GB300 residual-and-update path for the
 * Mallard finite-volume solver (TENO reconstruction -> face flux ->
 * residual assembly -> SSPRK3 stage update, with primitive recovery and the
 * CFL reduction), for one GPU.
 *
 * Plain C: pointers, sizes and status codes; no C++ or framework types.
 * Every call returns MGPU_OK (0) or an error code; mgpu_last_error() gives
 * the message of the last failure on the calling thread.  Host arrays are
 * borrowed for the duration of a call; device memory is owned by the context.
 *
 * Array conventions follow the reference's host views (row-major):
 *   U (conservatives)  [n_cells][4]            rho, rho*u, rho*v, rho*E
 *   primitives         [n_cells][5]            u, v, p, T, h
 *   face values        [n_faces][n_q][2][4]    side 0 = cells_of_face(f,0)
 *   rhs                [n_cells][4]
 * Cell and face numbering at this boundary is always the caller's (the
 * reference Mesh's); the library reorders internally.
 *
 * Reference interfaces each entry point replaces (paths inside the
 * MatthewBonanni/Mallard tree):
 *   mgpu_create/mgpu_add_boundary/mgpu_finalize
 *        -> Solver::init_numerics + init_boundaries (src/solver/solver.cpp:110-237),
 *           TENO::init (src/numerics/face_reconstruction.cpp:109-152)
 *   mgpu_calc_face_values
 *        -> FaceReconstruction::calc_face_values (src/numerics/face_reconstruction.h:82-83)
 *   mgpu_calc_rhs
 *        -> Solver::calc_rhs (src/solver/solver_rhs.cpp:44-55), which runs
 *           InteriorFluxFunctor (src/numerics/flux_functor.h:124-178) and
 *           Boundary::apply (src/boundary/boundary.h:115-116)
 *   mgpu_take_step
 *        -> SSPRK3::take_step (src/numerics/time_integrator.cpp:135-163)
 *           + Solver::update_primitives (src/solver/solver.cpp:568-578)
 *   mgpu_calc_dt
 *        -> Solver::calc_dt / calc_spectral_radius (src/solver/solver.cpp:580-742)
 *   mgpu_run
 *        -> the time-step loop of Solver::run (src/solver/solver.cpp:352-373)
 *   mgpu_riemann_flux_batch
 *        -> RiemannSolver::calc_flux (src/numerics/riemann_solver.h:85-90)
 *   mgpu_primitives_batch
 *        -> Physics::compute_primitives_from_conservatives (src/physics/physics.h:274-278)
 *   mgpu_mesh_*
 *        -> Mesh::init_cart / init_cart_tri / init_wedge and the derived
 *           geometry (src/mesh/mesh.cpp:167-261, 305-848)
 */
#ifndef MALLARD_GB300_H
#define MALLARD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MGPU_OK 0
#define MGPU_ERR_ARG 1         /* invalid argument or configuration          */
#define MGPU_ERR_CUDA 2        /* a CUDA runtime call failed                 */
#define MGPU_ERR_NAN 3         /* a non-finite state or time step was seen   */
#define MGPU_ERR_TIMEOUT 4     /* a bounded device wait gave up              */
#define MGPU_ERR_STATE 5       /* call out of order (e.g. before finalize)   */
#define MGPU_ERR_UNSUPPORTED 6 /* configuration not built for the GPU path   */
#define MGPU_ERR_HOST 7        /* host-side failure (allocation, table build) */

/* ---- enumerations (values match the reference's string keys) ----------- */
enum { MGPU_MESH_CARTESIAN = 0, MGPU_MESH_CARTESIAN_TRI = 1, MGPU_MESH_WEDGE = 2 };
enum { MGPU_RECON_FO = 0, MGPU_RECON_TENO = 1 };
enum { MGPU_BASIS_MONOMIAL = 0, MGPU_BASIS_LEGENDRE = 1 };
enum { MGPU_RIEMANN_RUSANOV = 0, MGPU_RIEMANN_HLL = 1, MGPU_RIEMANN_HLLC = 2 };
enum { MGPU_INTEGRATOR_SSPRK3 = 0, MGPU_INTEGRATOR_FE = 1, MGPU_INTEGRATOR_RK4 = 2 };
enum { MGPU_TABLES_GPU = 0, MGPU_TABLES_HOST = 1 };
enum { MGPU_VISC_GRAD_RECON = 0, MGPU_VISC_GRAD_GREEN_GAUSS = 1 };
enum {
    MGPU_BC_SYMMETRY = 0,
    MGPU_BC_EXTRAPOLATION = 1,
    MGPU_BC_WALL_ADIABATIC = 2,
    MGPU_BC_UPT = 3,
    MGPU_BC_P_OUT = 4
};
/* TENO weighting: 0 = the reference's arithmetic, quirks included;
 * 1 = corrected cut-off weights, zero-mean evaluation basis and a
 * positivity fallback in the face flux (same work per cell);
 * 2 = robust: the corrected weighting, then per cell: a cell with a
 * boundary face takes its average at all its face points; otherwise each
 * variable's face values are scaled toward the cell average into the range
 * of the cell's central stencil, and a cell whose face states are then not
 * all admissible (density and pressure positive) takes its average at all
 * its face points.  HLL and HLLC count a star pressure that is not a
 * number (the reference's two-rarefaction estimate under a strong
 * expansion next to near-vacuum pressure) as zero.  No reference
 * counterpart; it runs the four-quadrant and random-ensemble workloads to
 * their end times. */
enum { MGPU_TENO_REFERENCE = 0, MGPU_TENO_CORRECTED = 1, MGPU_TENO_ROBUST = 2 };
/* Arithmetic of the GPU path.
 * FP64      : FP64 with the reference's rounding (no FMA contraction, the
 *             reference's operation order); bit-identical to the reference's
 *             serial CPU build wherever the math libraries agree.
 * FP64_FAST : FP64 with FMA contraction and reduced-instruction forms of the
 *             smoothness indicator and x^6; agrees to ~1e-15 relative.
 * FP32      : reconstruction and face flux in FP32 (TENO with the corrected
 *             or robust weighting only); tables, geometry, the conserved state and its
 *             RK accumulation stay FP64, and face states near vacuum are
 *             recovered in FP64. */
enum { MGPU_PREC_FP64 = 0, MGPU_PREC_FP64_FAST = 1, MGPU_PREC_FP32 = 2 };

/* ---- mesh view: exactly the reference Mesh's public arrays (mesh.h:228-253)
 * plus its face zones (zone 0 is "interior", mesh.h:98-104). ------------- */
typedef struct mgpu_mesh {
    uint32_t n_nodes, n_cells, n_faces;
    const double* node_coords;             /* [n_nodes][2]                   */
    const double* cell_coords;             /* [n_cells][2] vertex centroid   */
    const double* cell_volume;             /* [n_cells]                      */
    const double* face_area;               /* [n_faces]                      */
    const double* face_normals;            /* [n_faces][2] area-weighted      */
    const uint32_t* offsets_nodes_of_cell; /* [n_cells+1]                    */
    const uint32_t* nodes_of_cell;
    const uint32_t* offsets_faces_of_cell; /* [n_cells+1]                    */
    const uint32_t* faces_of_cell;
    const uint32_t* offsets_nodes_of_face; /* [n_faces+1]                    */
    const uint32_t* nodes_of_face;
    const int32_t* cells_of_face;          /* [n_faces][2], -1 = boundary    */
    uint32_t n_zones;                      /* face zones, zone 0 = interior  */
    const uint32_t* zone_offsets;          /* [n_zones+1]                    */
    const uint32_t* zone_faces;
} mgpu_mesh;

typedef struct mgpu_mesh_buf mgpu_mesh_buf; /* an owning host mesh */

/* Generate one of the reference's meshes (same numbering and geometry). */
int mgpu_mesh_generate(int mesh_type, uint32_t nx, uint32_t ny, double Lx, double Ly, mgpu_mesh_buf** out);
/* A channel [0, Lx] x [yb(x), Ly] whose lower wall rises as a ramp of
 * ramp_deg degrees from x = x0 (no reference counterpart): an
 * (nx+1) x (ny+1) node lattice mapped onto the channel, interior nodes
 * jittered by up to +-jitter (< 0.5) of the local spacing (seeded),
 * triangulated by Delaunay (quad diagonals, then Lawson edge flips):
 * 2 nx ny triangles.  Zones:
 * 0 interior, 1 inflow (x = 0), 2 outflow (x = Lx), 3 lower wall, 4 upper
 * wall. */
int mgpu_mesh_generate_ramp(uint32_t nx, uint32_t ny, double Lx, double Ly, double x0, double ramp_deg, double jitter,
                            uint64_t seed, mgpu_mesh_buf** out);
/* Build a mesh from connectivity (the reference's unimplemented FILE type):
 * geometry is derived with the reference's formulas. */
int mgpu_mesh_from_connectivity(uint32_t n_nodes, const double* node_coords, uint32_t n_cells,
                                const uint32_t* offsets_nodes_of_cell, const uint32_t* nodes_of_cell,
                                const uint32_t* offsets_faces_of_cell, const uint32_t* faces_of_cell,
                                uint32_t n_faces, const uint32_t* offsets_nodes_of_face,
                                const uint32_t* nodes_of_face, const int32_t* cells_of_face, uint32_t n_zones,
                                const uint32_t* zone_offsets, const uint32_t* zone_faces, mgpu_mesh_buf** out);
/* Relabel cells with a seeded random permutation (mt19937_64, Fisher-Yates).
 * new_of_old (optional, [n_cells]) receives the permutation. */
int mgpu_mesh_permute_cells(mgpu_mesh_buf* m, uint64_t seed, uint32_t* new_of_old);
int mgpu_mesh_view(const mgpu_mesh_buf* m, mgpu_mesh* view);
void mgpu_mesh_free(mgpu_mesh_buf* m);
/* Mesh ingest (the reference's "file" mesh type, src/mesh/mesh.cpp:41-43,
 * whose default filename is mesh.msh and which the reference leaves
 * unimplemented).  Gmsh ASCII MSH 2.2 or 4.1, 2-D: triangles and
 * quadrilaterals are the cells (file order), line elements name the boundary
 * zones by physical group (else by curve).  Faces: one per distinct cell edge,
 * numbered in order of first appearance; zone 0 "interior", then the
 * boundary zones in order of first appearance, then "boundary" for boundary
 * faces no line element names. */
int mgpu_mesh_read_gmsh(const char* path, mgpu_mesh_buf** out);
/* The library's binary mesh format (connectivity, zones and zone names;
 * geometry is derived again on reading, so a round trip gives equal bits). */
int mgpu_mesh_write(const mgpu_mesh_buf* m, const char* path);
int mgpu_mesh_read(const char* path, mgpu_mesh_buf** out);
/* Zone names: generated meshes name theirs (interior, right, top, left,
 * bottom; the ramp channel interior, inflow, outflow, wall, top), read meshes
 * take the file's, others zone<i>. */
int mgpu_mesh_zone_name(const mgpu_mesh_buf* m, uint32_t zone, char* name, uint32_t len);
int mgpu_mesh_set_zone_name(mgpu_mesh_buf* m, uint32_t zone, const char* name);

/* ---- TENO tables (host) ----------------------------------------------- */
/* The tables TENO::init builds (face_reconstruction.cpp:109-788), in the
 * reference's layout (face_reconstruction.h:195-260), built on the host
 * without a GPU.  mgpu_finalize builds the same tables itself (in its tiled
 * device layout); this entry point exposes them for inspection. */
typedef struct mgpu_teno_tables mgpu_teno_tables;
enum {
    MGPU_TENO_OFFSETS_STENCIL_GROUPS = 0, /* uint32 [n_cells+1]             */
    MGPU_TENO_OFFSETS_STENCILS = 1,       /* uint32 [n_stencils+1]          */
    MGPU_TENO_STENCILS = 2,               /* uint32                         */
    MGPU_TENO_OFFSETS_MATRICES = 3,       /* uint32 [n_stencils+1]          */
    MGPU_TENO_MATRICES = 4,               /* double, K x M_s row-major each */
    MGPU_TENO_TRANSFORMED_AREAS = 5,      /* double                         */
    MGPU_TENO_INTEGRAL_PSI_TARGET = 6,    /* double [K]                     */
    MGPU_TENO_OSCILLATION_INDICATOR = 7,  /* double [K][K]                  */
    MGPU_TENO_POLY_INDICES = 8            /* int32 [K][2]                   */
};
int mgpu_teno_tables_build(const mgpu_mesh* mesh, int basis, int poly_order, double stencil_factor, int q_cell,
                           int q_face, mgpu_teno_tables** out);
uint64_t mgpu_teno_tables_len(const mgpu_teno_tables* t, int field);
int mgpu_teno_tables_copy(const mgpu_teno_tables* t, int field, void* dst);
void mgpu_teno_tables_free(mgpu_teno_tables* t);

/* ---- solver context ---------------------------------------------------- */
typedef struct mgpu_config {
    int recon;                      /* MGPU_RECON_*                          */
    int basis;                      /* MGPU_BASIS_*                          */
    int poly_order;                 /* TENO basis order (1..3 on the GPU)    */
    double max_stencil_size_factor; /* reference default 2.0                 */
    int quadrature_order_cell;      /* 0 = reference default p+1             */
    int quadrature_order_face;      /* 0 = reference default (p+1)/2         */
    int riemann_solver;             /* MGPU_RIEMANN_*                        */
    int time_integrator;            /* MGPU_INTEGRATOR_*                     */
    double gamma, p_ref, T_ref, rho_ref, p_min, p_max; /* physics (physics.cpp:27-53) */
    int teno_variant;               /* MGPU_TENO_*                           */
    int precision;                  /* MGPU_PREC_*                           */
    int reorder;                    /* 1 = reverse Cuthill-McKee cell order  */
    int device;                     /* CUDA device ordinal                   */
    /* Viscous (Navier-Stokes) face flux; no counterpart in the reference.
     * mu(T) = mu_ref (T/T_mu_ref)^1.5 (T_mu_ref + S) / (T + S) (Sutherland)
     * for sutherland_S > 0, else the constant mu_ref; conductivity
     * mu cp / prandtl; temperatures in the units of the solver's T = e / cv.
     * Cell gradients of (u, v, T) as viscous_gradients selects; at a face
     * the average of its two cells' plus the jump correction along the line
     * joining their centres.  With viscous != 0 wall_adiabatic walls are
     * no-slip and adiabatic; other boundaries carry no viscous flux. */
    int viscous;
    double mu_ref, T_mu_ref, sutherland_S, prandtl;
    /* Where mgpu_finalize builds the TENO tables: MGPU_TABLES_GPU (default:
     * the stencil search, face_reconstruction.cpp:217-475, on the GPU, and
     * the least squares, :477-741, on the GPU for the Legendre basis, on the
     * host for the monomial one) or MGPU_TABLES_HOST (both on the host).
     * Both give the same bits. */
    int table_build;
    /* Cell gradients of the viscous flux: MGPU_VISC_GRAD_RECON (default)
     * differentiates each cell's reconstructed TENO polynomials at its
     * centroid -- the conserved variables' gradients, after the variant's
     * per-cell step (the robust variant's scaling, or zero where a cell falls
     * back to its average), turned into (u, v, T) gradients with the cell
     * averages; the reconstruction kernel writes them, so no gradient
     * kernel runs.  With first-order reconstruction, or
     * MGPU_VISC_GRAD_GREEN_GAUSS, the Green-Gauss gradients of the cell
     * averages: (1/V) sum_f phi_f n A, phi_f the mean of the two cells (a
     * wall: u = v = 0, T of the cell; another boundary: the cell's value). */
    int viscous_gradients;
} mgpu_config;

typedef struct mgpu_ctx mgpu_ctx;

/* Fill cfg with the reference's defaults (TENO p=3 legendre, HLLC, SSPRK3,
 * gamma 1.4, reference state of physics_test.cpp, p clip +-1e20). */
void mgpu_config_defaults(mgpu_config* cfg);
int mgpu_create(const mgpu_mesh* mesh, const mgpu_config* cfg, mgpu_ctx** out);
/* Boundaries are applied in the order added, like the TOML [[boundaries]]
 * list.  data: upt = (u, v, p, T); p_out = (p); others none. */
int mgpu_add_boundary(mgpu_ctx* ctx, uint32_t zone, int bc_type, const double* data, int n_data);
/* Build the TENO tables (host), reorder, upload; required before compute. */
int mgpu_finalize(mgpu_ctx* ctx);
int mgpu_destroy(mgpu_ctx* ctx);
/* Launch on a caller stream (cudaStream_t passed as void*); NULL = own stream. */
int mgpu_set_stream(mgpu_ctx* ctx, void* stream);
int mgpu_synchronize(mgpu_ctx* ctx);

/* State in the caller's cell order, [n_cells][4] and [n_cells][5].
 * set_state: primitives NULL recovers them on the device from U with the
 * reference's arithmetic (physics.h:842-867).  get_state: either output may
 * be NULL.  Host buffers (pinned or pageable) are borrowed for the call;
 * pinned ones (cudaHostAlloc / cudaHostRegister) must hold the whole array,
 * as for a copy: a kernel reads or writes them in place, permuting the rows
 * (and writing the FP32 form's copy) in the same pass, where pageable ones
 * go through a device staging array.
 * The FP32 form's steps carry no FP64 primitives (its flux and time step
 * read the FP32 state copy): after a step, get_state recovers them from U
 * as set_state does; before any step it returns the ones set_state had. */
int mgpu_set_state(mgpu_ctx* ctx, const double* U, const double* primitives);
int mgpu_get_state(mgpu_ctx* ctx, double* U, double* primitives);

/* Parity hooks (host buffers in, host buffers out). */
int mgpu_calc_face_values(mgpu_ctx* ctx, const double* U, double* face_values, uint8_t* teno_masks);
int mgpu_calc_rhs(mgpu_ctx* ctx, const double* U, double* rhs);

/* Time stepping on the resident state.  The FP32 form computes the
 * spectral radius in FP32 from its FP32 state copy. */
int mgpu_calc_dt(mgpu_ctx* ctx, double cfl, double* dt, double* cfl_local);
int mgpu_take_step(mgpu_ctx* ctx, double dt);
/* n_steps x (spectral radius -> dt = cfl / max -> SSPRK3 step) without host
 * round trips; t_out (optional) receives the simulated time advanced. */
int mgpu_run(mgpu_ctx* ctx, double cfl, uint32_t n_steps, double* t_out);
/* Device error flags: bit 0 non-finite state, bit 1 non-positive dt, bit 2
 * a bounded device wait ran out (MGPU_ERR_TIMEOUT). */
int mgpu_status(mgpu_ctx* ctx, uint32_t* flags);

/* The CFL time step of the resident state, as mgpu_calc_dt computes it, for
 * callers that must not allocate device memory once they are stepping: a
 * host application whose device memory all comes from its own pool or
 * arena, or a real-time loop that cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree.  This entry point has no
 * counterpart in the reference.
 *   dt_device               device pointer to one double (caller-owned): dt
 *   spectral_radius_device  optional device array [n_cells] in the caller's
 *                           cell order: per-cell spectral radius (the
 *                           reference's cfl_local before its scaling by dt)
 * Enqueued on the context's stream; it does not synchronise.  It calls no
 * cudaMalloc/cudaFree: its reduction scratch is a static device array of
 * 512 KiB (one partial per 256 cells), so empty meshes and meshes above
 * 16,777,216 cells are rejected with MGPU_ERR_ARG.  The first call on each
 * device looks up that array's device address (with the context's device
 * current), so make that first call before any stream capture.  The
 * caller's current device is restored on return.  Calls share the array:
 * calls that overlap on the GPU race.  A dt that is not finite and
 * non-negative sets bit 1 of mgpu_status.  The plain FP64 and the FP32 forms
 * give mgpu_calc_dt's values bit for bit; on the FP64-fast form (which
 * mgpu_calc_dt evaluates with reciprocals and FMA) they agree to 1e-12
 * relative. */
int mgpu_calc_dt_noalloc(mgpu_ctx* ctx, double cfl, double* dt_device, double* spectral_radius_device);

/* ---- learned TENO stencil selector ------------------------------------
 * No counterpart in the reference.  A 96-64-64-32 MLP (GELU) predicts, per
 * cell and conserved variable, the stencil decision of the corrected TENO
 * form (face_reconstruction.cpp:939-981): class 0 = central stencil only,
 * class m = 1..7 = the directional stencils whose bit is set in m.  Inputs
 * per variable: the 19 central-stencil differences divided by their range,
 * the scaled log10 of that range, the three directional ranges relative to
 * it, and a zero (24 x 4 = 96).  Parameters are packed FP32: W1 [96][64],
 * b1 [64], W2 [64][64], b2 [64], W3 [64][32], b3 [32] (MGPU_SEL_PARAMS).
 * Training runs on the GPU (FP32 kernels, softmax cross-entropy per head,
 * Adam); inference runs on the tcgen05 tensor cores in BF16 with FP32
 * accumulation.  Attached to an FP32-form context (p = 3) it replaces the
 * smoothness indicators of every variable whose predicted class reaches
 * the probability threshold in the cell and in all its face neighbours, and
 * the cell evaluates only the stencils its variables need; any other
 * variable runs full TENO. */
#define MGPU_SEL_INPUTS 96
#define MGPU_SEL_OUTPUTS 32
#define MGPU_SEL_CLASSES 8
#define MGPU_SEL_PARAMS 12448
typedef struct mgpu_selector mgpu_selector;
/* Seeded uniform(+-1/sqrt(fan_in)) weights, zero biases. */
int mgpu_selector_create(int device, uint64_t seed, mgpu_selector** out);
void mgpu_selector_destroy(mgpu_selector* sel);
int mgpu_selector_get_params(mgpu_selector* sel, float* params);
/* Also resets the Adam moments. */
int mgpu_selector_set_params(mgpu_selector* sel, const float* params);
/* The training set lives on the device: rows X [n][96] FP32 and labels
 * Y [n][4] (class per variable). */
int mgpu_selector_dataset_size(const mgpu_selector* sel, uint64_t* n);
int mgpu_selector_clear(mgpu_selector* sel);
int mgpu_selector_add_samples(mgpu_selector* sel, const float* X, const uint8_t* Y, uint64_t n);
int mgpu_selector_get_samples(mgpu_selector* sel, uint64_t first, uint64_t n, float* X, uint8_t* Y);
/* Appends the current state of an FP64 or FP64-fast context (corrected TENO,
 * p = 3): every cell where some variable leaves the central stencil, and
 * each all-central cell with probability keep_central (seeded). */
int mgpu_selector_harvest(mgpu_selector* sel, mgpu_ctx* ctx, double keep_central, uint64_t seed, uint64_t* added);
/* One forward + backward pass over host rows: gradient of the mean
 * cross-entropy (over rows and heads) in the packed parameter layout. */
int mgpu_selector_gradient(mgpu_selector* sel, const float* X, const uint8_t* Y, uint32_t n, float* grad,
                           float* loss);
/* Minibatch Adam (beta 0.9/0.999, eps 1e-8) over the dataset, shuffled per
 * epoch with seed + epoch; epoch_loss[epochs] receives each epoch's mean
 * loss (may be NULL). */
int mgpu_selector_train(mgpu_selector* sel, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                        float* epoch_loss);
/* Tensor-core inference over host rows: logits [n][32] and predictions
 * [n][4] (predicted TENO mask, bit 7 set when the predicted class has at
 * least probability thr_central if it is the central class, thr_directional
 * otherwise; a threshold outside (0, 1] is never reached); either output
 * may be NULL.  MGPU_ERR_TIMEOUT when a bounded wait in the kernel ran out. */
int mgpu_selector_infer(mgpu_selector* sel, const float* X, uint32_t n, float thr_central, float thr_directional,
                        float* logits, uint8_t* pred);
/* Attaches a copy of the selector's current weights to an FP32-form context
 * (thr_central in (0, 1]; thr_directional above 1 trusts no directional
 * prediction); sel NULL or thr_central <= 0 detaches. */
int mgpu_set_selector(mgpu_ctx* ctx, mgpu_selector* sel, float thr_central, float thr_directional);
/* By default the selector predicts once per time step, from the step's
 * initial state, and the three SSPRK3 stages use those predictions;
 * every_stage != 0 predicts at every stage instead. */
int mgpu_set_selector_every_stage(mgpu_ctx* ctx, int every_stage);
/* Predict every `steps` CFL steps of mgpu_run (default 1; each call starts
 * with a prediction); the steps between reuse the last trusted predictions.
 * Information crosses at most CFL cells per step, so with CFL <= 0.5 an
 * interval of 2 stays inside the one-ring margin of the neighbour check. */
int mgpu_set_selector_interval(mgpu_ctx* ctx, uint32_t steps);
/* Counts over the last reconstruction with the selector: [0] cells,
 * [1] cells with every variable confident, [2] confident variables,
 * [3] stencils evaluated, [4] stencils full TENO evaluates, [5] error flag. */
int mgpu_selector_stats(mgpu_ctx* ctx, uint64_t* counts);
/* The selector's last predictions per cell and variable, caller order
 * [n_cells][4]: predicted TENO mask | 0x80 when confident; raw = 1 before
 * the neighbour check, 0 after it (what the reconstruction used). */
int mgpu_selector_predictions(mgpu_ctx* ctx, int raw, uint8_t* out);

/* ---- batched form -------------------------------------------------------
 * No counterpart in the reference.  Many independent cases on a few meshes
 * (n_groups <= 8; group g holds cases_per_group[g] cases on meshes[g]),
 * stepped together: one launch per kernel covers every case, each mesh's
 * TENO tables and face geometry exist once and are shared by its cases, and
 * every case has its own time step (its own CFL reduction), time and status
 * flags.  The FP32 form of corrected TENO at p = 3 only (cfg->precision =
 * MGPU_PREC_FP32); the boundary list applies to every case's zones.
 * Cases are addressed as (group, index within the group); states are in
 * the caller's cell order of the group's mesh. */
typedef struct mgpu_batch mgpu_batch;
int mgpu_batch_create(uint32_t n_groups, const mgpu_mesh* const* meshes, const uint32_t* cases_per_group,
                      const mgpu_config* cfg, mgpu_batch** out);
int mgpu_batch_add_boundary(mgpu_batch* b, uint32_t zone, int type, const double* data, int n_data);
int mgpu_batch_finalize(mgpu_batch* b);
void mgpu_batch_destroy(mgpu_batch* b);
uint32_t mgpu_batch_n_cases(const mgpu_batch* b);
/* Also resets the case's time and status flags; prim may be NULL. */
int mgpu_batch_set_state(mgpu_batch* b, uint32_t group, uint32_t index, const double* U, const double* prim);
/* prim: recovered from U after a step (as for the FP32 form's mgpu_get_state). */
int mgpu_batch_get_state(mgpu_batch* b, uint32_t group, uint32_t index, double* U, double* prim);
/* n_steps CFL steps of every case, each a replay of one captured CUDA graph
 * (spectral radius and dt per case, three SSPRK3 stages); asynchronous. */
int mgpu_batch_run(mgpu_batch* b, double cfl, uint32_t n_steps);
int mgpu_batch_synchronize(mgpu_batch* b);
/* Launch on the caller's stream (a cudaStream_t) from now on; NULL returns
 * to the batch's own stream. */
int mgpu_batch_set_stream(mgpu_batch* b, void* stream);
/* Per case (global order: group 0's cases first): status flags (bit 0
 * non-finite state, bit 1 invalid dt, bit 2 a bounded device wait ran out)
 * and time; either may be NULL. */
int mgpu_batch_status(mgpu_batch* b, uint32_t* flags, double* times);
/* Autotuner of the batched reconstruction: times the direct kernel's 4
 * launch shapes x 4 grid sizes (one thread per item, or a persistent grid of
 * 2, 4, 8 CTAs per SM), the staged kernel's 3 shapes (4-6, as mgpu_autotune
 * numbers them; one warp per item) and the resident kernel's 2 (7, 8: one
 * CTA of 4 or 8 warps per mesh tile, the tile's tables copied into shared
 * memory once and used for every case) on the current states and keeps the
 * fastest.  ms[36] receives the times (shape-major, 4 per shape, 0 where not
 * applicable); any output may be NULL. */
int mgpu_batch_autotune(mgpu_batch* b, double* ms, int* shape, int* blocks_per_sm);
/* Fix the batched reconstruction's launch shape (0-8) and grid (CTAs per
 * SM, 0 = one thread per item; the staged shapes ignore it). */
int mgpu_batch_set_launch_shape(mgpu_batch* b, int shape, int blocks_per_sm);

/* Diagnostics for measurement.  Kernel timing brackets every launch of the
 * reconstruction, flux, update, CFL and selector kernels with CUDA events on
 * the launching stream; mgpu_kernel_times returns, per kernel class
 * (0 recon, 1 flux, 2 update, 3 cfl, 4 selector), the summed milliseconds
 * and launch counts since the last reset (arrays of 5). */
int mgpu_enable_kernel_timing(mgpu_ctx* ctx, int enable);
int mgpu_kernel_times(mgpu_ctx* ctx, double* ms, uint32_t* launches);
/* Autotuner: times each launch shape of the reconstruction kernel (FP32
 * form at p = 3: 0-2 128-thread blocks with at most 128, 80 or 64 registers
 * per thread, 3 256-thread blocks with 64, 4-7 the staged kernel, whose
 * warps copy their tile's table blocks into shared memory with bulk async
 * copies, one stencil slot per warp: 4 warps per block with at most 80
 * registers, then 2, 1 and 4 warps per block with at most 72) on the
 * current state, three launches each after a warm-up, and keeps the
 * fastest for later launches.
 * ms[MGPU_AUTOTUNE_SHAPES] receives the average time per shape (0 where not
 * applicable), best the chosen shape.  Both may be NULL.  Other forms have
 * a single shape. */
#define MGPU_AUTOTUNE_SHAPES 8
int mgpu_autotune(mgpu_ctx* ctx, double* ms, int* best);
/* Fix the reconstruction's launch shape (as mgpu_autotune numbers them);
 * every shape gives the same results. */
int mgpu_set_launch_shape(mgpu_ctx* ctx, int shape);
/* Algorithmic (compulsory) bytes one reconstruction launch and one full
 * stage move, from the actual table sizes. */
int mgpu_traffic_model(mgpu_ctx* ctx, double* recon_bytes, double* stage_bytes);
/* A copy of one reconstruction table as the kernels read it (tiled layout,
 * library cell order), to compare the GPU and host table builds.  dst null:
 * only *bytes is set.  MGPU_ERR_ARG for a table this form does not hold. */
enum {
    MGPU_TABLE_P = 0,     /* double: pseudo-inverse (FP64 forms)          */
    MGPU_TABLE_AREAS = 1, /* double: transformed areas (FP64 forms)       */
    MGPU_TABLE_P32 = 2,   /* float: pseudo-inverse x areas (FP32 form)    */
    MGPU_TABLE_NB = 3,    /* uint32: stencil neighbours (FP64 forms)      */
    MGPU_TABLE_NB32 = 4,  /* uint32: stencil neighbours (FP32 form)       */
    MGPU_TABLE_PHI = 5,   /* double: face-point basis shapes (FP64 forms) */
    MGPU_TABLE_PHI32 = 6  /* uint16: per cell, 3 bits per face slot: the
                           * reference edge whose shape set the FP32 form's
                           * face points use (7: none)                    */
};
int mgpu_get_table(mgpu_ctx* ctx, int field, void* dst, uint64_t* bytes);
/* Wall seconds of mgpu_finalize's phases, seconds[7]: 0 face and cell
 * numbering, 1 geometry and gather lists, 2 TENO stencil search (on the GPU
 * with MGPU_TABLES_GPU, else on the host; includes the neighbourhood graph
 * and the stencils' host copy), 3 table pack (host; includes the host least
 * squares when built there) and upload, 4 least squares on the GPU, 5 other
 * TENO setup, 6 the remaining uploads. */
int mgpu_build_times(mgpu_ctx* ctx, double* seconds);
uint32_t mgpu_n_cells(const mgpu_ctx* ctx);

/* ---- unit-level GPU entry points (known-answer tests) ------------------ */
/* n independent Riemann problems; arrays: n_unit [n][2], u_l/u_r [n][2],
 * scalars [n]; flux [n][4].  Host buffers.  solver: MGPU_RIEMANN_*, with
 * MGPU_RIEMANN_GUARD or'ed in for the robust variant's guarded star
 * pressure (a NaN star pressure counts as zero). */
#define MGPU_RIEMANN_GUARD 16
int mgpu_riemann_flux_batch(int solver, uint32_t n, const double* n_unit, const double* rho_l, const double* u_l,
                            const double* p_l, const double* gamma_l, const double* h_l, const double* rho_r,
                            const double* u_r, const double* p_r, const double* gamma_r, const double* h_r,
                            double* flux);
/* Euler primitive recovery for n states on the GPU. */
int mgpu_primitives_batch(double gamma, double p_ref, double T_ref, double rho_ref, double p_min, double p_max,
                          uint32_t n, const double* U, double* primitives);
/* ---- output ------------------------------------------------------------- */
/* VTU output of the solution in the reference's format (DataWriter::write_vtu,
 * src/io/data_writer.cpp:93-244: VTK XML UnstructuredGrid, raw appended
 * data, Float64 cell arrays, files <prefix>_<step, 6 digits>.vtu), written
 * asynchronously.  variables: comma-separated [[write_data]] names among RHO,
 * RHOU_X, RHOU_Y, RHOE, U_X, U_Y, P, T, H, CFL (CFL = dt x the spectral radius
 * of the last time step).  mgpu_writer_write writes when step % interval ==
 * 0 or force: it snapshots the arrays on the device (ordered after the work
 * queued on the context's stream, which waits for the snapshot only) and
 * returns; a copy stream and a worker thread copy them to pinned memory and
 * write the file while the solver goes on.  mgpu_writer_flush waits for every
 * queued file and reports the first I/O error; destroy flushes. */
typedef struct mgpu_writer mgpu_writer;
int mgpu_writer_create(mgpu_ctx* ctx, const char* prefix, const char* variables, uint32_t interval,
                       mgpu_writer** out);
int mgpu_writer_write(mgpu_writer* w, uint32_t step, int force);
int mgpu_writer_flush(mgpu_writer* w);
void mgpu_writer_destroy(mgpu_writer* w);
/* The same file format from host arrays: data [n_vars][n_cells] in the
 * mesh's cell order (host only). */
int mgpu_vtu_write(const mgpu_mesh_buf* mesh, const char* path, uint32_t n_vars, const char* const* names,
                   const double* data);

/* FP64 FMA throughput probe: returns measured GFLOP/s (2 flops per FMA). */
int mgpu_probe_fp64_gflops(int device, double* gflops);
/* The FP32 form's integer-pipe conversions on the device, for testing:
 * out32[i] = in64[i] rounded to FP32 (nearest even; magnitudes below FP32's
 * smallest normal give a signed zero), out64[i] = in32[i] exactly. */
int mgpu_probe_conversions(int device, const double* in64, float* out32, const float* in32, double* out64, uint64_t n);

const char* mgpu_last_error(void);
int mgpu_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MALLARD_GB300_H */
