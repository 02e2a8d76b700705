"""The learned TENO stencil selector (no counterpart in the reference).

A 96-64-64-32 MLP predicts, per cell and conserved variable, the stencil
decision of the corrected TENO form: class 0 = central stencil only, class
m = 1..7 = the directional stencils whose bit is set in m.  It is trained on
the GPU from (features, decision) pairs harvested from the FP64 solver's own
runs and evaluated on the tcgen05 tensor cores inside the FP32 form's
reconstruction, where a variable whose predicted class reaches the
probability threshold skips the smoothness indicators and the cell reads
only the stencil tables it needs.

    sel = Selector(seed=1)
    sel.harvest(fp64_solver, keep_central=0.05, seed=2)   # as often as wanted
    sel.train(epochs=8)
    fp32_solver.attach_selector(sel, threshold=0.9)
"""

import ctypes as C
from pathlib import Path

import numpy as np

from . import _native as N

IN, OUT, NCLS, N_PARAMS = 96, 32, 8, 12448


class Selector:
    def __init__(self, device=0, seed=0):
        self._lib = N.lib()
        h = C.c_void_p()
        N.check(self._lib.mgpu_selector_create(int(device), int(seed), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mgpu_selector_destroy(self._h)
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

    # ---- parameters -----------------------------------------------------------
    @property
    def params(self):
        p = np.empty(N_PARAMS, dtype=np.float32)
        N.check(self._lib.mgpu_selector_get_params(self._h, N.ptr(p)))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.shape != (N_PARAMS,):
            raise ValueError(f"expected {N_PARAMS} parameters")
        N.check(self._lib.mgpu_selector_set_params(self._h, N.ptr(p)))

    def save(self, path, **meta):
        np.savez(path, params=self.params, **meta)

    def load(self, path):
        with np.load(path) as z:
            self.params = z["params"]

    # ---- data -----------------------------------------------------------------
    def __len__(self):
        n = C.c_uint64()
        N.check(self._lib.mgpu_selector_dataset_size(self._h, C.byref(n)))
        return n.value

    def clear(self):
        N.check(self._lib.mgpu_selector_clear(self._h))

    def add_samples(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.uint8)
        if X.ndim != 2 or X.shape[1] != IN or Y.shape != (X.shape[0], 4):
            raise ValueError("X must be [n][96] and Y [n][4]")
        N.check(self._lib.mgpu_selector_add_samples(self._h, N.ptr(X), N.ptr(Y), X.shape[0]))

    def samples(self, first=0, n=None):
        n = len(self) - first if n is None else n
        X = np.empty((n, IN), dtype=np.float32)
        Y = np.empty((n, 4), dtype=np.uint8)
        N.check(self._lib.mgpu_selector_get_samples(self._h, first, n, N.ptr(X), N.ptr(Y)))
        return X, Y

    def harvest(self, solver, keep_central=0.05, seed=0):
        """Append the current state of an FP64 TENO solver; returns rows added."""
        n = C.c_uint64()
        N.check(self._lib.mgpu_selector_harvest(self._h, solver._h, float(keep_central), int(seed), C.byref(n)))
        return n.value

    # ---- training and inference -------------------------------------------------
    def gradient(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.uint8)
        g = np.empty(N_PARAMS, dtype=np.float32)
        loss = C.c_float()
        N.check(self._lib.mgpu_selector_gradient(self._h, N.ptr(X), N.ptr(Y), X.shape[0], N.ptr(g), C.byref(loss)))
        return g, loss.value

    def train(self, epochs=8, batch=4096, lr=2e-3, seed=0):
        losses = np.zeros(epochs, dtype=np.float32)
        N.check(self._lib.mgpu_selector_train(self._h, int(epochs), int(batch), float(lr), int(seed), N.ptr(losses)))
        return losses

    def infer(self, X, threshold=0.9, directional_threshold=None):
        """(logits [n][32], predictions [n][4]) from the tensor-core kernel.
        directional_threshold defaults to threshold."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        L = np.empty((X.shape[0], OUT), dtype=np.float32)
        P = np.empty((X.shape[0], 4), dtype=np.uint8)
        td = threshold if directional_threshold is None else directional_threshold
        N.check(self._lib.mgpu_selector_infer(self._h, N.ptr(X), X.shape[0], float(threshold), float(td), N.ptr(L),
                                              N.ptr(P)))
        return L, P


def default_weights_path():
    return Path(__file__).resolve().parent / "data" / "selector_p3.npz"
