"""ctypes wrapper around oracle/_build/liboracle.so (the CPU restatement).

Test infrastructure: the checker for the GPU path and the timed CPU baseline.
Build it with ``make -C oracle`` (``__graft_entry__.build()`` does this).
"""

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "liboracle.so"
_lib = None

MESH_TYPES = {"cartesian": 0, "cartesian_tri": 1, "wedge": 2}
RECON = {"FO": 0, "TENO": 1}
BASIS = {"monomial": 0, "legendre": 1}
RIEMANN = {"Rusanov": 0, "HLL": 1, "HLLC": 2}
BC_TYPES = {"symmetry": 0, "extrapolation": 1, "wall_adiabatic": 2, "upt": 3, "p_out": 4}

_MESH_FIELDS = [
    ("node_coords", np.float64, 2),
    ("cell_coords", np.float64, 2),
    ("cell_volume", np.float64, 1),
    ("face_area", np.float64, 1),
    ("face_normals", np.float64, 2),
    ("offsets_nodes_of_cell", np.uint32, 1),
    ("nodes_of_cell", np.uint32, 1),
    ("offsets_faces_of_cell", np.uint32, 1),
    ("faces_of_cell", np.uint32, 1),
    ("offsets_nodes_of_face", np.uint32, 1),
    ("nodes_of_face", np.uint32, 1),
    ("cells_of_face", np.int32, 2),
    ("zone_offsets", np.uint32, 1),
    ("zone_faces", np.uint32, 1),
]

_TENO_FIELDS = [
    ("offsets_stencil_groups", np.uint32),
    ("offsets_stencils", np.uint32),
    ("stencils", np.uint32),
    ("offsets_reconstruction_matrices", np.uint32),
    ("reconstruction_matrices", np.float64),
    ("transformed_areas", np.float64),
    ("integral_psi_target", np.float64),
    ("oscillation_indicator", np.float64),
    ("poly_indices", np.int32),
]


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise RuntimeError(f"oracle library not built: {_LIB_PATH} (run make -C oracle)")
    lib = C.CDLL(str(_LIB_PATH))
    vp, u32, i32, f64, u64 = C.c_void_p, C.c_uint32, C.c_int, C.c_double, C.c_uint64
    sig = {
        "orc_last_error": (C.c_char_p, []),
        "orc_set_threads": (None, [i32]),
        "orc_max_threads": (i32, []),
        "orc_mesh_generate": (vp, [i32, u32, u32, f64, f64]),
        "orc_mesh_from_arrays": (vp, [u32, vp, u32, vp, vp, vp, vp, u32, vp, vp, vp, u32, vp, vp]),
        "orc_mesh_free": (None, [vp]),
        "orc_mesh_permute_cells": (i32, [vp, u64, vp]),
        "orc_mesh_len": (u64, [vp, i32]),
        "orc_mesh_copy": (None, [vp, i32, vp]),
        "orc_mesh_counts": (u32, [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]),
        "orc_case_create": (vp, [vp, i32, i32, i32, f64, i32, i32, i32, f64, f64, f64, f64, f64, f64]),
        "orc_case_free": (None, [vp]),
        "orc_case_add_boundary": (i32, [vp, u32, i32, vp, i32]),
        "orc_case_set_state": (None, [vp, vp, vp]),
        "orc_case_get_state": (None, [vp, vp, vp]),
        "orc_case_nq": (i32, [vp]),
        "orc_case_set_teno_variant": (None, [vp, i32]),
        "orc_case_set_viscous": (None, [vp, i32, f64, f64, f64, f64]),
        "orc_case_set_viscous_gradients": (None, [vp, i32]),
        "orc_case_viscous_gradients": (i32, [vp, vp, vp]),
        "orc_case_set_integrator": (None, [vp, i32]),
        "orc_fe_const_rhs": (None, [vp, vp, u32, f64]),
        "orc_rk4_const_rhs": (None, [vp, vp, u32, f64]),
        "orc_case_face_values": (i32, [vp, vp, vp, vp]),
        "orc_case_calc_rhs": (i32, [vp, vp, vp]),
        "orc_case_calc_dt": (i32, [vp, f64, C.POINTER(f64), vp]),
        "orc_case_take_step": (i32, [vp, f64]),
        "orc_case_run": (i32, [vp, f64, u32, C.POINTER(f64)]),
        "orc_teno_len": (u64, [vp, i32]),
        "orc_teno_copy": (None, [vp, i32, vp]),
        "orc_riemann_flux": (None, [i32, vp, f64, vp, f64, f64, f64, f64, vp, f64, f64, f64, vp]),
        "orc_gas_constants": (None, [f64, f64, f64, f64, vp]),
        "orc_primitives": (None, [f64, f64, f64, f64, f64, f64, vp, vp, u32]),
        "orc_qr_householder": (i32, [vp, vp, i32, i32]),
        "orc_forward_substitution": (None, [vp, vp, vp, i32, i32, i32, i32, i32]),
        "orc_back_substitution": (None, [vp, vp, vp, i32, i32, i32, i32, i32]),
        "orc_triangle_jac": (None, [vp, vp, vp, vp, vp]),
        "orc_triangle_area": (f64, [vp, vp, vp]),
        "orc_ssprk3_const_rhs": (None, [vp, vp, u32, f64]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _err(lib):
    return lib.orc_last_error().decode()


class OracleMesh:
    """A mesh held by the oracle: generated (reference generators) or from arrays."""

    def __init__(self, handle):
        self._lib = load()
        if not handle:
            raise RuntimeError(_err(self._lib))
        self.h = handle
        self._load()

    def _load(self):
        nn, nc, nf = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self.n_zones = self._lib.orc_mesh_counts(self.h, C.byref(nn), C.byref(nc), C.byref(nf))
        self.n_nodes, self.n_cells, self.n_faces = nn.value, nc.value, nf.value
        for i, (name, dt, width) in enumerate(_MESH_FIELDS):
            n = self._lib.orc_mesh_len(self.h, i)
            a = np.empty(n, dtype=dt)
            if n:
                self._lib.orc_mesh_copy(self.h, i, _p(a))
            if width > 1:
                a = a.reshape(-1, width)
            setattr(self, name, a)

    def permute_cells(self, seed):
        """Relabel the cells by the seeded permutation the GPU library's mesh
        helper applies (see the C source); returns new_of_old."""
        perm = np.empty(self.n_cells, dtype=np.uint32)
        if self._lib.orc_mesh_permute_cells(self.h, int(seed), _p(perm)) != 0:
            raise RuntimeError(_err(self._lib))
        self._load()
        return perm

    @classmethod
    def generate(cls, mesh_type, nx, ny, Lx=1.0, Ly=1.0):
        return cls(load().orc_mesh_generate(MESH_TYPES[mesh_type], nx, ny, Lx, Ly))

    @classmethod
    def from_arrays(cls, m):
        """m: any object with the connectivity attributes of a mesh (numpy)."""
        arr = {k: np.ascontiguousarray(getattr(m, k)) for k in (
            "node_coords", "offsets_nodes_of_cell", "nodes_of_cell", "offsets_faces_of_cell", "faces_of_cell",
            "offsets_nodes_of_face", "nodes_of_face", "cells_of_face", "zone_offsets", "zone_faces")}
        n_cells = len(arr["offsets_nodes_of_cell"]) - 1
        n_faces = len(arr["offsets_nodes_of_face"]) - 1
        h = load().orc_mesh_from_arrays(
            len(arr["node_coords"]), _p(arr["node_coords"]), n_cells, _p(arr["offsets_nodes_of_cell"]),
            _p(arr["nodes_of_cell"]), _p(arr["offsets_faces_of_cell"]), _p(arr["faces_of_cell"]), n_faces,
            _p(arr["offsets_nodes_of_face"]), _p(arr["nodes_of_face"]), _p(arr["cells_of_face"]),
            len(arr["zone_offsets"]) - 1, _p(arr["zone_offsets"]), _p(arr["zone_faces"]))
        return cls(h)

    def __del__(self):
        if getattr(self, "h", None) and self._lib is not None:
            self._lib.orc_mesh_free(self.h)
            self.h = None


class OracleCase:
    """One solver case: mesh + numerics + state, with the hot-path methods."""

    def __init__(self, mesh, recon="TENO", basis="legendre", poly_order=3, stencil_factor=2.0, q_cell=0, q_face=0,
                 riemann="HLLC", gamma=1.4, p_ref=101325.0, T_ref=298.15, rho_ref=1.225, p_min=-1e20, p_max=1e20):
        self._lib = load()
        self.mesh = mesh
        self.h = self._lib.orc_case_create(mesh.h, RECON[recon], BASIS[basis], poly_order, stencil_factor, q_cell,
                                           q_face, RIEMANN[riemann], gamma, p_ref, T_ref, rho_ref, p_min, p_max)
        if not self.h:
            raise RuntimeError(_err(self._lib))
        self.nq = self._lib.orc_case_nq(self.h)
        self.n_cells, self.n_faces = mesh.n_cells, mesh.n_faces

    def __del__(self):
        if getattr(self, "h", None) and self._lib is not None:
            self._lib.orc_case_free(self.h)
            self.h = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(_err(self._lib))

    def set_teno_variant(self, variant):
        """0: the reference's weighting; 1: cut-off weighting; 2: robust (cut-off
        weighting, first-order boundary cells, range scaling and positivity
        fallback per cell, guarded star pressure); see the C source."""
        self._lib.orc_case_set_teno_variant(self.h, int(variant))

    def set_integrator(self, name):
        """SSPRK3 (default), FE or RK4 (time_integrator.cpp)."""
        self._lib.orc_case_set_integrator(self.h, {"SSPRK3": 0, "FE": 1, "RK4": 2}[name])

    def set_viscous(self, mu_ref, T_mu_ref=1.0, sutherland_S=0.0, prandtl=0.72, viscous=True, gradients="recon"):
        """The viscous face flux (no reference counterpart; see the C source).
        gradients: "recon" (the reconstructed polynomials', with TENO) or
        "green_gauss"."""
        self._lib.orc_case_set_viscous(self.h, 1 if viscous else 0, float(mu_ref), float(T_mu_ref),
                                       float(sutherland_S), float(prandtl))
        self._lib.orc_case_set_viscous_gradients(self.h, {"recon": 0, "green_gauss": 1}[gradients])

    def add_boundary(self, zone, bc_type, data=()):
        d = np.asarray(data, dtype=np.float64)
        self._check(self._lib.orc_case_add_boundary(self.h, zone, BC_TYPES[bc_type], _p(d) if d.size else None,
                                                    int(d.size)))

    def set_state(self, U, prim=None):
        U = np.ascontiguousarray(U, dtype=np.float64)
        P = None if prim is None else np.ascontiguousarray(prim, dtype=np.float64)
        self._lib.orc_case_set_state(self.h, _p(U), _p(P))

    def get_state(self):
        U = np.empty((self.n_cells, 4))
        P = np.empty((self.n_cells, 5))
        self._lib.orc_case_get_state(self.h, _p(U), _p(P))
        return U, P

    def face_values(self, U, masks=False):
        U = np.ascontiguousarray(U, dtype=np.float64)
        F = np.zeros((self.n_faces, self.nq, 2, 4))
        M = np.zeros((self.n_cells, 4), dtype=np.uint8) if masks else None
        self._check(self._lib.orc_case_face_values(self.h, _p(U), _p(F), _p(M)))
        return (F, M) if masks else F

    def calc_rhs(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        R = np.empty((self.n_cells, 4))
        self._check(self._lib.orc_case_calc_rhs(self.h, _p(U), _p(R)))
        return R

    def viscous_gradients(self, U):
        """The viscous flux's cell gradients of U, [n_cells][6]: du/dx,
        du/dy, dv/dx, dv/dy, dT/dx, dT/dy."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        G = np.empty((self.n_cells, 6))
        self._check(self._lib.orc_case_viscous_gradients(self.h, _p(U), _p(G)))
        return G

    def calc_dt(self, cfl):
        dt = C.c_double()
        cl = np.empty(self.n_cells)
        self._check(self._lib.orc_case_calc_dt(self.h, cfl, C.byref(dt), _p(cl)))
        return dt.value, cl

    def take_step(self, dt):
        self._check(self._lib.orc_case_take_step(self.h, dt))

    def run(self, cfl, n_steps):
        t = C.c_double()
        self._check(self._lib.orc_case_run(self.h, cfl, n_steps, C.byref(t)))
        return t.value

    def teno_tables(self):
        out = {}
        for i, (name, dt) in enumerate(_TENO_FIELDS):
            n = self._lib.orc_teno_len(self.h, i)
            a = np.empty(n, dtype=dt)
            if n:
                self._lib.orc_teno_copy(self.h, i, _p(a))
            out[name] = a
        return out


class Oracle:
    """Unit-level oracle routines (known-answer tests)."""

    def __init__(self):
        self.lib = load()

    def set_threads(self, n):
        self.lib.orc_set_threads(int(n))

    def max_threads(self):
        return self.lib.orc_max_threads()

    def riemann_flux(self, kind, n_unit, rho_l, u_l, p_l, gamma_l, h_l, rho_r, u_r, p_r, gamma_r, h_r, guard=False):
        n = np.asarray(n_unit, dtype=np.float64)
        ul = np.asarray(u_l, dtype=np.float64)
        ur = np.asarray(u_r, dtype=np.float64)
        F = np.empty(4)
        self.lib.orc_riemann_flux(RIEMANN[kind] | (16 if guard else 0), _p(n), rho_l, _p(ul), p_l, gamma_l, h_l, rho_r, _p(ur), p_r,
                                  gamma_r, h_r, _p(F))
        return F

    def gas_constants(self, gamma, p_ref, T_ref, rho_ref):
        out = np.empty(3)
        self.lib.orc_gas_constants(gamma, p_ref, T_ref, rho_ref, _p(out))
        return out

    def primitives(self, U, gamma, p_ref, T_ref, rho_ref, p_min=-1e20, p_max=1e20):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1, 4)
        W = np.empty((len(U), 5))
        self.lib.orc_primitives(gamma, p_ref, T_ref, rho_ref, p_min, p_max, _p(U), _p(W), len(U))
        return W

    def qr_householder(self, A, m, n):
        A = np.ascontiguousarray(A, dtype=np.float64)
        R = np.empty(m * n)
        if self.lib.orc_qr_householder(_p(A), _p(R), m, n) != 0:
            raise RuntimeError(_err(self.lib))
        return R

    def forward_substitution(self, L, B, m, n, p, tL, tB):
        L = np.ascontiguousarray(L, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        X = np.zeros(m * p)
        self.lib.orc_forward_substitution(_p(L), _p(B), _p(X), m, n, p, int(tL), int(tB))
        return X

    def back_substitution(self, U, B, m, n, p, tU, tB):
        U = np.ascontiguousarray(U, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        X = np.zeros(m * p)
        self.lib.orc_back_substitution(_p(U), _p(B), _p(X), m, n, p, int(tU), int(tB))
        return X

    def triangle_jac(self, a, b, c):
        a, b, c = (np.asarray(v, dtype=np.float64) for v in (a, b, c))
        J, Ji = np.empty(4), np.empty(4)
        self.lib.orc_triangle_jac(_p(a), _p(b), _p(c), _p(J), _p(Ji))
        return J, Ji

    def triangle_area(self, a, b, c):
        a, b, c = (np.asarray(v, dtype=np.float64) for v in (a, b, c))
        return self.lib.orc_triangle_area(_p(a), _p(b), _p(c))

    def ssprk3_const_rhs(self, U, rhs, dt):
        return self._const_rhs(self.lib.orc_ssprk3_const_rhs, U, rhs, dt)

    def fe_const_rhs(self, U, rhs, dt):
        return self._const_rhs(self.lib.orc_fe_const_rhs, U, rhs, dt)

    def rk4_const_rhs(self, U, rhs, dt):
        return self._const_rhs(self.lib.orc_rk4_const_rhs, U, rhs, dt)

    @staticmethod
    def _const_rhs(fn, U, rhs, dt):
        U = np.ascontiguousarray(U, dtype=np.float64).copy()
        R = np.ascontiguousarray(rhs, dtype=np.float64)
        fn(_p(U), _p(R), len(U) // 4 if U.ndim == 1 else len(U), dt)
        return U


def threads_available():
    return max(1, os.cpu_count() or 1)
