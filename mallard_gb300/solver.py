"""Host-side mirror of the reference's solver interfaces over the GPU path.

``Solver`` keeps the names, argument meaning and error behaviour of the
reference's hot-path methods (MatthewBonanni/Mallard src/solver/solver.h:47-108):

    calc_face_values(U)  -> FaceReconstruction::calc_face_values
    calc_rhs(U)          -> Solver::calc_rhs
    calc_dt(cfl)         -> Solver::calc_dt (+ the cfl_local field)
    take_step(dt)        -> SSPRK3::take_step + Solver::update_primitives
    run(cfl, n_steps)    -> the loop of Solver::run without output or checks

Every compute call goes through the C ABI into the CUDA kernels; errors come
back as ``MgpuError`` (a RuntimeError) carrying the reference's message where
the reference has one.
"""

import ctypes as C
import re

import numpy as np

from . import _native as N
from .mesh import Mesh

try:  # Python >= 3.11
    import tomllib
except ImportError:  # pragma: no cover
    tomllib = None


def gas_constants(gamma, p_ref, T_ref, rho_ref):
    """Euler::set_R_cp_cv (src/physics/physics.cpp:69-73)."""
    R = p_ref / (T_ref * rho_ref)
    cp = R * gamma / (gamma - 1.0)
    cv = cp / gamma
    return R, cp, cv


def state_from_primitives(rho, u, v, p, gamma=1.4, p_ref=101325.0, T_ref=298.15, rho_ref=1.225):
    """Conservatives and primitives from (rho, u, v, p) per cell, as the
    reference's analytical initialisation computes them
    (src/solver/solver_initialize.cpp:159-185)."""
    R, _, cv = gas_constants(gamma, p_ref, T_ref, rho_ref)
    rho, u, v, p = (np.asarray(x, dtype=np.float64) for x in (rho, u, v, p))
    T = p / (rho * R)
    e = cv * T
    E = e + 0.5 * (u * u + v * v)
    h = e + p / rho
    U = np.stack([rho, rho * u, rho * v, rho * E], 1)
    W = np.stack([u, v, p, T, h], 1)
    return np.ascontiguousarray(U), np.ascontiguousarray(W)


def eval_exprtk(expr, x, y):
    """Evaluate the subset of exprtk used by the reference's example inputs:
    ``var name := expr;`` assignments followed by one expression over x, y,
    comparisons, + - * / and numbers (src/solver/solver_initialize.cpp:125-157)."""
    env = {"x": np.asarray(x, dtype=np.float64), "y": np.asarray(y, dtype=np.float64)}
    parts = [s.strip() for s in expr.replace("\\\n", " ").split(";") if s.strip()]
    allowed = re.compile(r"^[\w\s.+\-*/()<>=!:]*$")
    for part in parts:
        if not allowed.match(part):
            raise RuntimeError(f"unsupported initial-condition expression: {part}")
        m = re.match(r"^var\s+(\w+)\s*:=\s*(.*)$", part, re.S)
        target, rhs = (m.group(1), m.group(2)) if m else (None, part)
        val = eval(rhs, {"__builtins__": {}}, env)  # restricted: names are x, y and earlier vars
        val = np.asarray(val, dtype=np.float64) if np.asarray(val).dtype == bool else np.asarray(val)
        if target:
            env[target] = val
        else:
            out = np.broadcast_to(np.asarray(val, dtype=np.float64), env["x"].shape)
            return np.array(out, dtype=np.float64)
    raise RuntimeError("initial-condition expression has no value")


class Solver:
    """The residual-and-update path of one case on one GPU."""

    def __init__(self, mesh, face_reconstruction="TENO", basis_type="legendre", basis_order=3,
                 max_stencil_size_factor=2.0, quadrature_order_cell=0, quadrature_order_face=0,
                 riemann_solver="HLLC", time_integrator="SSPRK3", gamma=1.4, p_ref=101325.0, T_ref=298.15,
                 rho_ref=1.225, p_min=-1e20, p_max=1e20, boundaries=(), teno_variant="reference", reorder=True,
                 device=0, precision="fp64", viscous=None, table_build="gpu"):
        """viscous: None for the Euler path, or a dict with mu_ref and
        optionally T_mu_ref, sutherland_S, prandtl and gradients ("recon":
        the reconstructed polynomials' gradients, the default; or
        "green_gauss") -- the viscous face flux, no counterpart in the
        reference; walls become no-slip.
        table_build: "gpu" (least-squares tables built by a kernel; Legendre
        basis) or "host"; both give the same bits."""
        self._lib = N.lib()
        self.mesh = mesh
        self.gas = dict(gamma=gamma, p_ref=p_ref, T_ref=T_ref, rho_ref=rho_ref)
        self.p_min, self.p_max = p_min, p_max
        if face_reconstruction not in N.RECON:
            raise RuntimeError(f"Unknown face reconstruction type: {face_reconstruction}.")
        if riemann_solver not in N.RIEMANN:
            raise RuntimeError(f"Unknown Riemann solver type: {riemann_solver}.")
        if time_integrator not in N.INTEGRATORS:
            raise RuntimeError(f"Unknown time integrator type: {time_integrator}.")
        cfg = N.Config()
        self._lib.mgpu_config_defaults(C.byref(cfg))
        cfg.recon = N.RECON[face_reconstruction]
        cfg.basis = N.BASIS[basis_type]
        cfg.poly_order = int(basis_order)
        cfg.max_stencil_size_factor = float(max_stencil_size_factor)
        cfg.quadrature_order_cell = int(quadrature_order_cell)
        cfg.quadrature_order_face = int(quadrature_order_face)
        cfg.riemann_solver = N.RIEMANN[riemann_solver]
        cfg.time_integrator = N.INTEGRATORS[time_integrator]
        cfg.gamma, cfg.p_ref, cfg.T_ref, cfg.rho_ref = gamma, p_ref, T_ref, rho_ref
        cfg.p_min, cfg.p_max = p_min, p_max
        cfg.teno_variant = N.TENO_VARIANTS[teno_variant]
        if precision not in N.PRECISIONS:
            raise RuntimeError(f"Unknown precision: {precision}.")
        cfg.precision = N.PRECISIONS[precision]
        self.precision = precision
        cfg.reorder = 1 if reorder else 0
        cfg.device = int(device)
        if table_build not in ("gpu", "host"):
            raise RuntimeError(f"Unknown table build: {table_build}.")
        cfg.table_build = 0 if table_build == "gpu" else 1
        if viscous:
            cfg.viscous = 1
            cfg.mu_ref = float(viscous["mu_ref"])
            cfg.T_mu_ref = float(viscous.get("T_mu_ref", 1.0))
            cfg.sutherland_S = float(viscous.get("sutherland_S", 0.0))
            cfg.prandtl = float(viscous.get("prandtl", 0.72))
            grads = viscous.get("gradients", "recon")
            if grads not in N.VISC_GRADIENTS:
                raise RuntimeError(f"Unknown viscous gradients: {grads}.")
            cfg.viscous_gradients = N.VISC_GRADIENTS[grads]
        self.cfg = cfg
        self.nq = 1 if face_reconstruction == "FO" else (
            quadrature_order_face if quadrature_order_face > 0 else (basis_order + 1) // 2)
        v = mesh.view()
        h = C.c_void_p()
        N.check(self._lib.mgpu_create(C.byref(v), C.byref(cfg), C.byref(h)))
        self._h = h
        try:
            for b in boundaries:
                self.add_boundary(**b)
            N.check(self._lib.mgpu_finalize(self._h))
        except Exception:
            self.close()
            raise
        self.n_cells, self.n_faces = mesh.n_cells, mesh.n_faces

    # ---- lifecycle ----------------------------------------------------------
    def add_boundary(self, name, type, u=None, p=None, T=None):
        """Boundary::init for the five reference BCs (src/boundary/boundary_*.cpp)."""
        if type not in N.BC_TYPES:
            raise RuntimeError(f"Unknown boundary type: {type}.")
        zone = self.mesh.zone_index(name)
        if type == "upt":
            if u is None or p is None or T is None:
                raise RuntimeError(f"Missing u, p or T for boundary: {name}.")
            if len(u) != 2:
                raise RuntimeError(f"Invalid u for boundary: {name}.")
            data = np.array([u[0], u[1], p, T], dtype=np.float64)
        elif type == "p_out":
            if p is None:
                raise RuntimeError(f"Missing p for boundary: {name}.")
            data = np.array([p], dtype=np.float64)
        else:
            data = np.zeros(0)
        N.check(self._lib.mgpu_add_boundary(self._h, zone, N.BC_TYPES[type], N.ptr(data) if data.size else None,
                                            int(data.size)))

    def close(self):
        # output writers snapshot this context: finish and release them first
        for w in getattr(self, "_writers", []):
            w.close()
        self._writers = []
        h = getattr(self, "_h", None)
        if h:
            self._lib.mgpu_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- state --------------------------------------------------------------
    def set_state(self, U, primitives=None):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(self.n_cells, 4)
        W = None if primitives is None else np.ascontiguousarray(primitives, dtype=np.float64).reshape(self.n_cells, 5)
        N.check(self._lib.mgpu_set_state(self._h, N.ptr(U), N.ptr(W)))

    def get_state(self, U=None, W=None, primitives=True):
        """Conservatives and primitives in the caller's cell order; pass
        (e.g. pinned) output arrays to receive them in place.  primitives
        False: the conservatives alone (W is None)."""
        U = np.empty((self.n_cells, 4)) if U is None else U
        if primitives:
            W = np.empty((self.n_cells, 5)) if W is None else W
        else:
            W = None
        for a, w in ((U, 4), (W, 5)):
            if a is None:
                continue
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != self.n_cells * w:
                raise ValueError("state buffers must be contiguous float64 of the mesh size")
        N.check(self._lib.mgpu_get_state(self._h, N.ptr(U), N.ptr(W)))
        return U, W

    # ---- hot path -----------------------------------------------------------
    def calc_face_values(self, U, masks=False):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(self.n_cells, 4)
        F = np.empty((self.n_faces, self.nq, 2, 4))
        M = np.empty((self.n_cells, 4), dtype=np.uint8) if masks else None
        N.check(self._lib.mgpu_calc_face_values(self._h, N.ptr(U), N.ptr(F), N.ptr(M)))
        return (F, M) if masks else F

    def calc_rhs(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(self.n_cells, 4)
        R = np.empty((self.n_cells, 4))
        N.check(self._lib.mgpu_calc_rhs(self._h, N.ptr(U), N.ptr(R)))
        return R

    def calc_dt(self, cfl):
        dt = C.c_double()
        cl = np.empty(self.n_cells)
        N.check(self._lib.mgpu_calc_dt(self._h, float(cfl), C.byref(dt), N.ptr(cl)))
        return dt.value, cl

    def take_step(self, dt):
        N.check(self._lib.mgpu_take_step(self._h, float(dt)))

    def run(self, cfl, n_steps):
        t = C.c_double()
        N.check(self._lib.mgpu_run(self._h, float(cfl), int(n_steps), C.byref(t)))
        return t.value

    def launch(self, cfl, n_steps):
        """Enqueue n_steps CFL steps without waiting (for timing)."""
        N.check(self._lib.mgpu_run(self._h, float(cfl), int(n_steps), None))

    def synchronize(self):
        N.check(self._lib.mgpu_synchronize(self._h))

    def status(self):
        f = C.c_uint32()
        rc = self._lib.mgpu_status(self._h, C.byref(f))
        if rc not in (N.MGPU_OK, 3):
            N.check(rc)
        return f.value

    # ---- measurement --------------------------------------------------------
    def set_stream(self, stream_handle):
        N.check(self._lib.mgpu_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None))

    def kernel_timing(self, enable=True):
        N.check(self._lib.mgpu_enable_kernel_timing(self._h, 1 if enable else 0))

    def kernel_times(self):
        """{class: (ms total, launches)} for recon, flux, update, cfl, selector."""
        ms = np.zeros(5)
        n = np.zeros(5, dtype=np.uint32)
        N.check(self._lib.mgpu_kernel_times(self._h, N.ptr(ms), N.ptr(n)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(("recon", "flux", "update", "cfl", "selector"))}

    # ---- learned stencil selector (FP32 form) --------------------------------
    def attach_selector(self, selector, threshold=0.995, directional_threshold=2.0, every_stage=False, interval=1):
        """Drive this FP32-form solver's TENO decisions with a trained
        selector: a variable predicted central with probability >= threshold
        skips the smoothness indicators and the directional stencils; a
        directional prediction is trusted only at >= directional_threshold
        (the default 2 trusts none).  Predictions are made once per time step
        (every interval steps in run()) unless every_stage.  selector None
        detaches."""
        N.check(self._lib.mgpu_set_selector(self._h, selector._h if selector is not None else None,
                                            float(threshold) if selector is not None else 0.0,
                                            float(directional_threshold)))
        if selector is not None:
            N.check(self._lib.mgpu_set_selector_every_stage(self._h, 1 if every_stage else 0))
            N.check(self._lib.mgpu_set_selector_interval(self._h, int(interval)))

    def selector_predictions(self, raw=True):
        """[n_cells][4] uint8: the selector's last predictions (mask | 0x80
        when confident), before (raw) or after the neighbour check."""
        out = np.zeros((self.mesh.n_cells, 4), dtype=np.uint8)
        N.check(self._lib.mgpu_selector_predictions(self._h, 1 if raw else 0, N.ptr(out)))
        return out

    def selector_stats(self):
        """Counts over the last reconstruction with the selector attached."""
        c = np.zeros(6, dtype=np.uint64)
        N.check(self._lib.mgpu_selector_stats(self._h, N.ptr(c)))
        keys = ("cells", "confident_cells", "confident_variables", "stencils_evaluated", "stencils_full", "error")
        return {k: int(c[i]) for i, k in enumerate(keys)}

    def autotune(self):
        """Pick the fastest launch shape of the reconstruction kernel on the
        current state; returns (chosen shape, ms per shape)."""
        ms = np.zeros(N.AUTOTUNE_SHAPES)
        best = C.c_int()
        N.check(self._lib.mgpu_autotune(self._h, N.ptr(ms), C.byref(best)))
        return best.value, ms

    def set_launch_shape(self, shape):
        """Fix the reconstruction kernel's launch shape (autotune numbering)."""
        N.check(self._lib.mgpu_set_launch_shape(self._h, int(shape)))

    def traffic_model(self):
        r, s = C.c_double(), C.c_double()
        N.check(self._lib.mgpu_traffic_model(self._h, C.byref(r), C.byref(s)))
        return r.value, s.value

    BUILD_PHASES = ("numbering", "geometry", "stencil_search", "table_pack", "gpu_least_squares", "teno_other",
                    "uploads")

    def build_times(self):
        """Seconds of each phase of the solver's setup (mgpu_finalize)."""
        t = np.zeros(7)
        N.check(self._lib.mgpu_build_times(self._h, N.ptr(t)))
        return dict(zip(self.BUILD_PHASES, t.tolist()))

    TABLES = {"P": (0, np.float64), "areas": (1, np.float64), "P32": (2, np.float32), "nb": (3, np.uint32),
              "nb32": (4, np.uint32), "phi": (5, np.float64), "phi32": (6, np.uint16)}

    def get_table(self, name):
        """One reconstruction table as the kernels read it (tiled layout,
        library cell order), as a flat array."""
        field, dt = self.TABLES[name]
        n = C.c_uint64()
        N.check(self._lib.mgpu_get_table(self._h, field, None, C.byref(n)))
        out = np.zeros(n.value // np.dtype(dt).itemsize, dtype=dt)
        N.check(self._lib.mgpu_get_table(self._h, field, out.ctypes.data_as(C.c_void_p), C.byref(n)))
        return out

    # ---- construction from the reference's TOML input -------------------------
    @classmethod
    def from_toml(cls, source, teno_variant="reference", reorder=True, device=0):
        """Build from a reference input file (path, TOML text or dict) and
        return (solver, U0, W0, run) where run holds the [run] table.
        Mirrors Solver::init (src/solver/solver.cpp:39-80)."""
        if isinstance(source, dict):
            inp = source
        else:
            if tomllib is None:
                raise RuntimeError("tomllib unavailable")
            text = source if "\n" in str(source) else open(source, "rb").read().decode()
            inp = tomllib.loads(text)
        m = inp.get("mesh", {})
        mtype = m.get("type", "file")
        if mtype == "file":
            # the reference's [mesh] filename key and default (mesh.cpp:41-43);
            # relative to the input file when one was given
            fname = m.get("filename", "mesh.msh")
            import os
            if not os.path.isabs(fname) and isinstance(source, (str, os.PathLike)) and "\n" not in str(source) \
                    and os.path.exists(str(source)):
                fname = os.path.join(os.path.dirname(os.path.abspath(str(source))), fname)
            mesh = Mesh.read_file(fname)
        else:
            mesh = Mesh.generate(mtype, m.get("Nx", 100), m.get("Ny", 100), m.get("Lx", 1.0), m.get("Ly", 1.0))
        phys = inp["physics"]
        for key in ("gamma", "p_ref", "T_ref", "rho_ref"):
            if key not in phys:
                raise RuntimeError(f"Missing {key} for physics: euler.")
        num = inp.get("numerics", {})
        fr = num.get("face_reconstruction", {})
        kw = dict(face_reconstruction=fr.get("type", "FO"), basis_type=fr.get("basis_type", "monomial"),
                  basis_order=fr.get("basis_order", 3), max_stencil_size_factor=fr.get("max_stencil_size_factor", 2.0),
                  quadrature_order_cell=fr.get("quadrature_order_cell", 0),
                  quadrature_order_face=fr.get("quadrature_order_face", 0),
                  riemann_solver=num.get("riemann_solver", "HLLC"),
                  time_integrator=num.get("time_integrator", "LSSSPRK3"),
                  gamma=phys["gamma"], p_ref=phys["p_ref"], T_ref=phys["T_ref"], rho_ref=phys["rho_ref"],
                  p_min=phys.get("p_min", -1e20), p_max=phys.get("p_max", 1e20))
        bnds = []
        for b in inp.get("boundaries", []):
            if "name" not in b:
                raise RuntimeError("Boundary name not specified.")
            if "type" not in b:
                raise RuntimeError("Boundary type not specified.")
            bnds.append({k: b[k] for k in ("name", "type", "u", "p", "T") if k in b})
        solver = cls(mesh, boundaries=bnds, teno_variant=teno_variant, reorder=reorder, device=device, **kw)
        U0, W0 = initial_state(mesh, inp.get("initialize", {}), solver.gas)
        # [[write_data]] (DataWriter::init, data_writer.cpp:29-75): VTU writers in solver.writers
        from .output import VtuWriter
        solver.writers = []
        for wd in inp.get("write_data", []):
            for key in ("prefix", "format", "interval", "variables"):
                if key not in wd:
                    raise RuntimeError(f"DataWriter: {key} not specified.")
            if wd["format"] == "tecplot":
                raise RuntimeError("DataWriter::write_tecplot not implemented.")
            if wd["format"] != "vtu":
                raise RuntimeError(f"DataWriter: Unknown format type: {wd['format']}.")
            solver.writers.append(VtuWriter(solver, wd["prefix"], wd["variables"], wd["interval"]))
        return solver, U0, W0, inp.get("run", {})


def initial_state(mesh, init, gas):
    """Solver::init_solution (src/solver/solver_initialize.cpp:35-187)."""
    kind = init.get("type", "constant")
    R, _, cv = gas_constants(gas["gamma"], gas["p_ref"], gas["T_ref"], gas["rho_ref"])
    x, y = mesh.cell_coords[:, 0], mesh.cell_coords[:, 1]
    if kind == "constant":
        u = init.get("u")
        if u is None:
            raise RuntimeError("Missing u for initialization: constant.")
        if len(u) != 2:
            raise RuntimeError("u must be a 2-element array for initialization: constant.")
        if "p" not in init:
            raise RuntimeError("Missing p for initialization: constant.")
        if "T" not in init:
            raise RuntimeError("Missing T for initialization: constant.")
        p, T = float(init["p"]), float(init["T"])
        rho = p / (R * T)
        e = cv * T
        E = e + 0.5 * (u[0] * u[0] + u[1] * u[1])
        h = e + p / rho
        n = mesh.n_cells
        U = np.tile(np.array([rho, rho * u[0], rho * u[1], rho * E]), (n, 1))
        W = np.tile(np.array([u[0], u[1], p, T, h]), (n, 1))
        return U, W
    if kind != "analytical":
        raise RuntimeError(f"Unknown initialization type: {kind}.")
    u = init.get("u")
    if u is None:
        raise RuntimeError("Missing u for initialization: analytical.")
    have = [k for k in ("rho", "p", "T") if k in init]
    if len(have) != 2:
        raise RuntimeError("Exactly two of rho, p, and T must be specified for initialization: analytical.")
    ux, uy = eval_exprtk(str(u[0]), x, y), eval_exprtk(str(u[1]), x, y)
    val = {k: eval_exprtk(str(init[k]), x, y) for k in have}
    if "rho" in val and "p" in val:
        rho, p = val["rho"], val["p"]
        T = p / (rho * R)
    elif "rho" in val:
        rho, T = val["rho"], val["T"]
        p = rho * R * T
    else:
        p, T = val["p"], val["T"]
        rho = p / (R * T)
    e = cv * T
    E = e + 0.5 * (ux * ux + uy * uy)
    h = e + p / rho
    U = np.stack([rho, rho * ux, rho * uy, rho * E], 1)
    W = np.stack([ux, uy, p, T, h], 1)
    return np.ascontiguousarray(U), np.ascontiguousarray(W)


def riemann_flux(solver, n_unit, rho_l, u_l, p_l, gamma_l, h_l, rho_r, u_r, p_r, gamma_r, h_r, guard=False):
    """RiemannSolver::calc_flux on the GPU for arrays of problems; guard: the
    robust variant's star pressure (a NaN star pressure counts as zero)."""
    arrs = [np.ascontiguousarray(np.atleast_1d(np.asarray(a, dtype=np.float64)))
            for a in (n_unit, rho_l, u_l, p_l, gamma_l, h_l, rho_r, u_r, p_r, gamma_r, h_r)]
    n = arrs[1].size
    arrs[0] = arrs[0].reshape(n, 2)
    arrs[2] = arrs[2].reshape(n, 2)
    arrs[7] = arrs[7].reshape(n, 2)
    F = np.empty((n, 4))
    N.check(N.lib().mgpu_riemann_flux_batch(N.RIEMANN[solver] | (16 if guard else 0), n, *[N.ptr(a) for a in arrs], N.ptr(F)))
    return F


def primitives(U, gamma=1.4, p_ref=101325.0, T_ref=298.15, rho_ref=1.225, p_min=-1e20, p_max=1e20):
    """Physics::compute_primitives_from_conservatives on the GPU."""
    U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1, 4)
    W = np.empty((len(U), 5))
    N.check(N.lib().mgpu_primitives_batch(gamma, p_ref, T_ref, rho_ref, p_min, p_max, len(U), N.ptr(U), N.ptr(W)))
    return W


def fp64_peak_gflops(device=0):
    g = C.c_double()
    N.check(N.lib().mgpu_probe_fp64_gflops(int(device), C.byref(g)))
    return g.value
