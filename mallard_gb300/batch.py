"""The batched form: many independent cases on a few meshes, stepped
together by one launch per kernel (no counterpart in the reference).

    b = Batch([mesh_a, mesh_b], [64, 32], boundaries=[...], riemann_solver="HLLC")
    b.set_state(0, 5, U, W)              # group 0, case 5, caller cell order
    b.autotune()
    b.run(0.5, 100)
    flags, times = b.status()            # per case
    U, W = b.get_state(0, 5)

Each mesh's TENO tables and face geometry are built once and shared by its
cases; every case has its own time step.  FP32 form of corrected (or
robust) TENO, p = 3.
"""

import ctypes as C

import numpy as np

from . import _native as N


class Batch:
    def __init__(self, meshes, cases_per_group, boundaries=(), riemann_solver="HLLC", gamma=1.4, p_ref=101325.0,
                 T_ref=298.15, rho_ref=1.225, device=0, teno_variant="corrected"):
        self._lib = N.lib()
        self.meshes = list(meshes)
        self.C = [int(c) for c in cases_per_group]
        cfg = N.Config()
        self._lib.mgpu_config_defaults(C.byref(cfg))
        cfg.riemann_solver = N.RIEMANN[riemann_solver]
        cfg.gamma, cfg.p_ref, cfg.T_ref, cfg.rho_ref = gamma, p_ref, T_ref, rho_ref
        cfg.teno_variant = N.TENO_VARIANTS[teno_variant]
        cfg.precision = N.PRECISIONS["fp32"]
        cfg.device = int(device)
        self._views = [m.view() for m in self.meshes]
        arr = (C.POINTER(N.MeshView) * len(self._views))(*[C.pointer(v) for v in self._views])
        cases = np.asarray(self.C, dtype=np.uint32)
        h = C.c_void_p()
        N.check(self._lib.mgpu_batch_create(len(self.meshes), C.cast(arr, C.c_void_p), N.ptr(cases), C.byref(cfg),
                                            C.byref(h)))
        self._h = h
        try:
            for bnd in boundaries:
                self._add_boundary(**bnd)
            N.check(self._lib.mgpu_batch_finalize(self._h))
        except Exception:
            self.close()
            raise
        self.n_cases = int(self._lib.mgpu_batch_n_cases(self._h))

    def _add_boundary(self, name, type, u=None, p=None, T=None):
        zone = self.meshes[0].zone_index(name)
        if type == "upt":
            data = np.array([u[0], u[1], p, T], dtype=np.float64)
        elif type == "p_out":
            data = np.array([p], dtype=np.float64)
        else:
            data = np.zeros(0)
        N.check(self._lib.mgpu_batch_add_boundary(self._h, zone, N.BC_TYPES[type], N.ptr(data) if data.size else None,
                                                  int(data.size)))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_state(self, group, index, U, primitives=None):
        U = np.ascontiguousarray(U, dtype=np.float64)
        W = None if primitives is None else np.ascontiguousarray(primitives, dtype=np.float64)
        N.check(self._lib.mgpu_batch_set_state(self._h, group, index, N.ptr(U), N.ptr(W)))

    def get_state(self, group, index):
        n = self.meshes[group].n_cells
        U = np.empty((n, 4))
        W = np.empty((n, 5))
        N.check(self._lib.mgpu_batch_get_state(self._h, group, index, N.ptr(U), N.ptr(W)))
        return U, W

    def run(self, cfl, n_steps):
        N.check(self._lib.mgpu_batch_run(self._h, float(cfl), int(n_steps)))

    def set_stream(self, stream_handle):
        N.check(self._lib.mgpu_batch_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None))

    def synchronize(self):
        N.check(self._lib.mgpu_batch_synchronize(self._h))

    def status(self):
        f = np.zeros(self.n_cases, dtype=np.uint32)
        t = np.zeros(self.n_cases)
        N.check(self._lib.mgpu_batch_status(self._h, N.ptr(f), N.ptr(t)))
        return f, t

    def set_launch_shape(self, shape, blocks_per_sm=0):
        """Fix the batched reconstruction's launch shape (autotune numbering)."""
        N.check(self._lib.mgpu_batch_set_launch_shape(self._h, int(shape), int(blocks_per_sm)))

    def autotune(self):
        """(shape, CTAs per SM or 0, ms[9][4]) of the batched reconstruction
        (shapes 4-8, the staged and resident kernels, have one grid: ms[s][0])."""
        ms = np.zeros(36)
        sh, bps = C.c_int(), C.c_int()
        N.check(self._lib.mgpu_batch_autotune(self._h, N.ptr(ms), C.byref(sh), C.byref(bps)))
        return sh.value, bps.value, ms.reshape(9, 4)
