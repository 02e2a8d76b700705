"""ctypes binding of libmallard_gb300.so (declarations in include/mallard_gb300.h).

The library is the product: the CUDA kernels and the host C++ behind the C
ABI.  There is no Python or CPU fallback for any compute entry point; if the
library is missing, importing the solver raises.
"""

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("MALLARD_GB300_LIB", _PKG / "_build" / "libmallard_gb300.so"))

MGPU_OK = 0
ERRORS = {1: "MGPU_ERR_ARG", 2: "MGPU_ERR_CUDA", 3: "MGPU_ERR_NAN", 4: "MGPU_ERR_TIMEOUT", 5: "MGPU_ERR_STATE",
          6: "MGPU_ERR_UNSUPPORTED", 7: "MGPU_ERR_HOST"}

MESH_TYPES = {"cartesian": 0, "cartesian_tri": 1, "wedge": 2}
RECON = {"FO": 0, "TENO": 1}
BASIS = {"monomial": 0, "legendre": 1}
RIEMANN = {"Rusanov": 0, "HLL": 1, "HLLC": 2}
INTEGRATORS = {"SSPRK3": 0, "FE": 1, "RK4": 2}
BC_TYPES = {"symmetry": 0, "extrapolation": 1, "wall_adiabatic": 2, "upt": 3, "p_out": 4}
TENO_VARIANTS = {"reference": 0, "corrected": 1, "robust": 2}
PRECISIONS = {"fp64": 0, "fp64_fast": 1, "fp32": 2}
VISC_GRADIENTS = {"recon": 0, "green_gauss": 1}
AUTOTUNE_SHAPES = 8  # MGPU_AUTOTUNE_SHAPES

TENO_FIELDS = {
    "offsets_stencil_groups": (0, "uint32"),
    "offsets_stencils": (1, "uint32"),
    "stencils": (2, "uint32"),
    "offsets_reconstruction_matrices": (3, "uint32"),
    "reconstruction_matrices": (4, "float64"),
    "transformed_areas": (5, "float64"),
    "integral_psi_target": (6, "float64"),
    "oscillation_indicator": (7, "float64"),
    "poly_indices": (8, "int32"),
}


class MgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class MeshView(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_uint32), ("n_cells", C.c_uint32), ("n_faces", C.c_uint32),
        ("node_coords", C.c_void_p), ("cell_coords", C.c_void_p), ("cell_volume", C.c_void_p),
        ("face_area", C.c_void_p), ("face_normals", C.c_void_p),
        ("offsets_nodes_of_cell", C.c_void_p), ("nodes_of_cell", C.c_void_p),
        ("offsets_faces_of_cell", C.c_void_p), ("faces_of_cell", C.c_void_p),
        ("offsets_nodes_of_face", C.c_void_p), ("nodes_of_face", C.c_void_p),
        ("cells_of_face", C.c_void_p),
        ("n_zones", C.c_uint32), ("zone_offsets", C.c_void_p), ("zone_faces", C.c_void_p),
    ]


class Config(C.Structure):
    _fields_ = [
        ("recon", C.c_int), ("basis", C.c_int), ("poly_order", C.c_int), ("max_stencil_size_factor", C.c_double),
        ("quadrature_order_cell", C.c_int), ("quadrature_order_face", C.c_int), ("riemann_solver", C.c_int),
        ("time_integrator", C.c_int), ("gamma", C.c_double), ("p_ref", C.c_double), ("T_ref", C.c_double),
        ("rho_ref", C.c_double), ("p_min", C.c_double), ("p_max", C.c_double), ("teno_variant", C.c_int),
        ("precision", C.c_int), ("reorder", C.c_int), ("device", C.c_int),
        ("viscous", C.c_int), ("mu_ref", C.c_double), ("T_mu_ref", C.c_double), ("sutherland_S", C.c_double),
        ("prandtl", C.c_double), ("table_build", C.c_int), ("viscous_gradients", C.c_int),
    ]


_lib = None


def lib():
    """Load the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"libmallard_gb300.so not built ({LIB_PATH}); run python -m mallard_gb300.build")
    L = C.CDLL(str(LIB_PATH))
    vp, i32, u32, u64, f64 = C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.c_double
    P = C.POINTER
    sig = {
        "mgpu_last_error": (C.c_char_p, []),
        "mgpu_version": (i32, []),
        "mgpu_mesh_generate": (i32, [i32, u32, u32, f64, f64, P(vp)]),
        "mgpu_mesh_generate_ramp": (i32, [u32, u32, f64, f64, f64, f64, f64, u64, P(vp)]),
        "mgpu_mesh_from_connectivity": (i32, [u32, vp, u32, vp, vp, vp, vp, u32, vp, vp, vp, u32, vp, vp, P(vp)]),
        "mgpu_mesh_permute_cells": (i32, [vp, u64, vp]),
        "mgpu_mesh_view": (i32, [vp, P(MeshView)]),
        "mgpu_mesh_free": (None, [vp]),
        "mgpu_teno_tables_build": (i32, [P(MeshView), i32, i32, f64, i32, i32, P(vp)]),
        "mgpu_teno_tables_len": (u64, [vp, i32]),
        "mgpu_teno_tables_copy": (i32, [vp, i32, vp]),
        "mgpu_teno_tables_free": (None, [vp]),
        "mgpu_config_defaults": (None, [P(Config)]),
        "mgpu_create": (i32, [P(MeshView), P(Config), P(vp)]),
        "mgpu_add_boundary": (i32, [vp, u32, i32, vp, i32]),
        "mgpu_finalize": (i32, [vp]),
        "mgpu_destroy": (i32, [vp]),
        "mgpu_set_stream": (i32, [vp, vp]),
        "mgpu_synchronize": (i32, [vp]),
        "mgpu_set_state": (i32, [vp, vp, vp]),
        "mgpu_get_state": (i32, [vp, vp, vp]),
        "mgpu_calc_face_values": (i32, [vp, vp, vp, vp]),
        "mgpu_calc_rhs": (i32, [vp, vp, vp]),
        "mgpu_calc_dt": (i32, [vp, f64, P(f64), vp]),
        "mgpu_take_step": (i32, [vp, f64]),
        "mgpu_run": (i32, [vp, f64, u32, P(f64)]),
        "mgpu_status": (i32, [vp, P(u32)]),
        "mgpu_calc_dt_noalloc": (i32, [vp, f64, vp, vp]),
        "mgpu_enable_kernel_timing": (i32, [vp, i32]),
        "mgpu_kernel_times": (i32, [vp, vp, vp]),
        "mgpu_traffic_model": (i32, [vp, P(f64), P(f64)]),
        "mgpu_get_table": (i32, [vp, i32, vp, P(C.c_uint64)]),
        "mgpu_set_launch_shape": (i32, [vp, i32]),
        "mgpu_batch_set_launch_shape": (i32, [vp, i32, i32]),
        "mgpu_mesh_read_gmsh": (i32, [C.c_char_p, P(vp)]),
        "mgpu_writer_create": (i32, [vp, C.c_char_p, C.c_char_p, u32, P(vp)]),
        "mgpu_writer_write": (i32, [vp, u32, i32]),
        "mgpu_writer_flush": (i32, [vp]),
        "mgpu_writer_destroy": (None, [vp]),
        "mgpu_vtu_write": (i32, [vp, C.c_char_p, u32, vp, vp]),
        "mgpu_mesh_read": (i32, [C.c_char_p, P(vp)]),
        "mgpu_mesh_write": (i32, [vp, C.c_char_p]),
        "mgpu_mesh_zone_name": (i32, [vp, u32, C.c_char_p, u32]),
        "mgpu_mesh_set_zone_name": (i32, [vp, u32, C.c_char_p]),
        "mgpu_probe_conversions": (i32, [i32, vp, vp, vp, vp, C.c_uint64]),
        "mgpu_build_times": (i32, [vp, vp]),
        "mgpu_autotune": (i32, [vp, vp, P(i32)]),
        "mgpu_batch_create": (i32, [u32, vp, vp, P(Config), P(vp)]),
        "mgpu_batch_add_boundary": (i32, [vp, u32, i32, vp, i32]),
        "mgpu_batch_finalize": (i32, [vp]),
        "mgpu_batch_destroy": (None, [vp]),
        "mgpu_batch_n_cases": (u32, [vp]),
        "mgpu_batch_set_state": (i32, [vp, u32, u32, vp, vp]),
        "mgpu_batch_get_state": (i32, [vp, u32, u32, vp, vp]),
        "mgpu_batch_run": (i32, [vp, f64, u32]),
        "mgpu_batch_synchronize": (i32, [vp]),
        "mgpu_batch_set_stream": (i32, [vp, vp]),
        "mgpu_batch_status": (i32, [vp, vp, vp]),
        "mgpu_batch_autotune": (i32, [vp, vp, P(i32), P(i32)]),
        "mgpu_n_cells": (u32, [vp]),
        "mgpu_riemann_flux_batch": (i32, [i32, u32] + [vp] * 12),
        "mgpu_primitives_batch": (i32, [f64, f64, f64, f64, f64, f64, u32, vp, vp]),
        "mgpu_probe_fp64_gflops": (i32, [i32, P(f64)]),
        "mgpu_selector_create": (i32, [i32, u64, P(vp)]),
        "mgpu_selector_destroy": (None, [vp]),
        "mgpu_selector_get_params": (i32, [vp, vp]),
        "mgpu_selector_set_params": (i32, [vp, vp]),
        "mgpu_selector_dataset_size": (i32, [vp, P(u64)]),
        "mgpu_selector_clear": (i32, [vp]),
        "mgpu_selector_add_samples": (i32, [vp, vp, vp, u64]),
        "mgpu_selector_get_samples": (i32, [vp, u64, u64, vp, vp]),
        "mgpu_selector_harvest": (i32, [vp, vp, f64, u64, P(u64)]),
        "mgpu_selector_gradient": (i32, [vp, vp, vp, u32, vp, P(C.c_float)]),
        "mgpu_selector_train": (i32, [vp, u32, u32, C.c_float, u64, vp]),
        "mgpu_selector_infer": (i32, [vp, vp, u32, C.c_float, C.c_float, vp, vp]),
        "mgpu_set_selector": (i32, [vp, vp, C.c_float, C.c_float]),
        "mgpu_selector_stats": (i32, [vp, vp]),
        "mgpu_selector_predictions": (i32, [vp, i32, vp]),
        "mgpu_set_selector_interval": (i32, [vp, u32]),
        "mgpu_set_selector_every_stage": (i32, [vp, i32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != MGPU_OK:
        raise MgpuError(rc, lib().mgpu_last_error().decode(errors="replace"))
    return rc


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def exported_symbols():
    """Names declared in include/mallard_gb300.h (for the ABI test)."""
    import re
    hdr = (_PKG.parent / "include" / "mallard_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(mgpu_\w+)\s*\(", hdr)))
