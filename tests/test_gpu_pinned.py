"""State transfers from and to pinned host memory: the device reads and
writes such buffers in one kernel pass that also permutes the rows (and
writes the FP32 copy), instead of a copy through the staging array.  The
results must be the pageable path's, bit for bit: the state read back, and
the states after a few steps, on a permuted, RCM-ordered mesh, FP64 and
FP32 forms, with and without primitives."""

import numpy as np
import pytest

import mallard_gb300 as mg
from cases import GAS, explosion

pytestmark = pytest.mark.gpu


def _pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def _solver(mesh, precision):
    blist = [{"name": z, "type": "extrapolation"} for z in mesh.zone_names[1:]]
    return mg.Solver(mesh, face_reconstruction="TENO", basis_type="legendre", basis_order=3, riemann_solver="HLLC",
                     boundaries=blist, teno_variant="robust", precision=precision, **GAS)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pinned_transfers_equal_pageable(precision):
    m = mg.Mesh.generate("cartesian_tri", 40, 36, 1.0, 1.0)
    m.permute_cells(9)
    U, W = explosion(m)
    n = m.n_cells
    Up, Wp = _pinned((n, 4)), _pinned((n, 5))
    Up[:] = U
    Wp[:] = W
    out = {}
    with _solver(m, precision) as s:
        for kind, (Uin, Win) in (("pageable", (U, W)), ("pinned", (Up, Wp))):
            s.set_state(Uin)
            back = _pinned((n, 4)) if kind == "pinned" else np.empty((n, 4))
            s.get_state(back, primitives=False)
            np.testing.assert_array_equal(back, U)
            s.set_state(Uin, Win)
            s.run(0.5, 6)
            Ue = _pinned((n, 4)) if kind == "pinned" else np.empty((n, 4))
            We = _pinned((n, 5)) if kind == "pinned" else np.empty((n, 5))
            s.get_state(Ue, We)
            assert s.status() == 0
            out[kind] = (Ue.copy(), We.copy())
    np.testing.assert_array_equal(out["pinned"][0], out["pageable"][0])
    np.testing.assert_array_equal(out["pinned"][1], out["pageable"][1])
