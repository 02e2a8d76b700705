"""Properties of the GPU path at the benchmark's full size (cartesian_tri
1024 x 1024 quads, 2,097,152 cells, seeded permutation + RCM), where the
oracle is too slow to run: size-independent checks of the kind the domain
offers.

* a uniform state stays uniform (every form);
* mass and energy are conserved in a closed box (symmetry walls) to
  round-off, for the FP64, FP64-fast and FP32 + learned forms;
* TENO (corrected weighting) reconstructs a linear field exactly at every
  face point of every face;
* an explosion centred in the unit square keeps the mesh's point symmetry
  (x, y) -> (1 - x, 1 - y) (first order).
"""

import numpy as np
import pytest

import mallard_gb300 as mg
from cases import BC_DATA, GAS, explosion, uniform

pytestmark = pytest.mark.gpu

N = 1024


@pytest.fixture(scope="module")
def mesh():
    m = mg.Mesh.generate("cartesian_tri", N, N, 1.0, 1.0)
    m.permute_cells(20261203)
    assert m.n_cells == 2 * N * N
    return m


def gpu_solver(mesh, recon="TENO", bcs=None, precision="fp64"):
    """The GPU solver alone (no oracle case: the CPU table build at this
    size would take far longer than the checks)."""
    bcs = bcs or {name: "extrapolation" for name in mesh.zone_names[1:]}
    blist = [dict(name=n, type=t, **BC_DATA[t]) for n, t in bcs.items()]
    return mg.Solver(mesh, face_reconstruction=recon, basis_type="legendre", basis_order=3, riemann_solver="HLLC",
                     boundaries=blist, teno_variant="corrected", precision=precision, **GAS)


def _closed(mesh, precision, learned=False):
    bcs = {z: "symmetry" for z in mesh.zone_names[1:]}
    s = gpu_solver(mesh, bcs=bcs, precision=precision)
    if learned:
        from mallard_gb300.selector import Selector, default_weights_path
        sel = Selector()
        sel.load(default_weights_path())
        s.attach_selector(sel)
        s._sel = sel
    return s


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("fp64_fast", 1e-13), ("fp32", 1e-6)])
def test_uniform_state_fullsize(mesh, precision, tol):
    s = gpu_solver(mesh, precision=precision)
    U, W = uniform(mesh)
    s.set_state(U, W)
    s.run(0.5, 5)
    Ug, _ = s.get_state()
    assert s.status() == 0
    err = np.abs(Ug - U).max(axis=0) / np.abs(U).max(axis=0)
    assert err.max() < tol, err
    s.close()


@pytest.mark.parametrize("precision,learned", [("fp64", False), ("fp64_fast", False), ("fp32", True)])
def test_conservation_closed_box_fullsize(mesh, precision, learned):
    s = _closed(mesh, precision, learned)
    U, W = explosion(mesh)
    s.set_state(U, W)
    vol = mesh.cell_volume
    m0, e0 = (U[:, 0] * vol).sum(), (U[:, 3] * vol).sum()
    s.run(0.5, 10)
    assert s.status() == 0
    Ug, _ = s.get_state()
    m1, e1 = (Ug[:, 0] * vol).sum(), (Ug[:, 3] * vol).sum()
    assert abs(m1 - m0) <= 1e-12 * m0, (m1 - m0) / m0
    assert abs(e1 - e0) <= 1e-12 * e0, (e1 - e0) / e0
    assert np.abs(Ug - U).max() > 1e-3  # the state did evolve
    s.close()


def test_linear_field_reconstruction_fullsize(mesh):
    """Cell averages of a linear field are its values at the centroids; the
    reconstruction must return the field at every face point (both sides of
    interior faces), to round-off."""
    s = gpu_solver(mesh, precision="fp64")
    coef = np.array([[1.0, 0.3, -0.2], [0.5, -0.4, 0.25], [-0.3, 0.2, 0.6], [2.5, 0.7, -0.5]])
    x, y = mesh.cell_coords[:, 0], mesh.cell_coords[:, 1]
    U = coef[:, 0] + np.outer(x, coef[:, 1]) + np.outer(y, coef[:, 2])
    F = s.calc_face_values(U)
    s.close()
    # face points: Gauss-Legendre on the segment from the face's first to its second node
    nodes = mesh.nodes_of_face.reshape(-1, 2)
    p0, p1 = mesh.node_coords[nodes[:, 0]], mesh.node_coords[nodes[:, 1]]
    interior = np.zeros(mesh.n_faces, dtype=bool)
    interior[mesh.zone("interior")] = True
    real = np.zeros(mesh.n_faces, dtype=bool)
    real[mesh.zone_faces] = True
    worst = 0.0
    for q, xi in enumerate((-1.0 / np.sqrt(3.0), 1.0 / np.sqrt(3.0))):
        t = (xi + 1.0) * 0.5
        xq = p0 + t * (p1 - p0)
        exact = coef[:, 0] + np.outer(xq[:, 0], coef[:, 1]) + np.outer(xq[:, 1], coef[:, 2])
        for side, sel in ((0, real), (1, interior)):
            err = np.abs(F[sel, q, side, :] - exact[sel]).max()
            worst = max(worst, err)
    assert worst < 1e-12 * np.abs(coef).sum(), worst


def test_point_symmetry_fullsize(mesh):
    """The cartesian_tri mesh is symmetric under (x, y) -> (1 - x, 1 - y)
    (each quad's diagonal maps onto itself); a centred explosion in a closed
    box keeps that symmetry to round-off over 20 first-order HLLC steps.
    (TENO stencils break distance ties by cell index, which the reflection
    does not preserve, so the check uses first order.)"""
    c = mesh.cell_coords
    key = np.round(c * 4 * N).astype(np.int64)
    mkey = np.round((1.0 - c) * 4 * N).astype(np.int64)
    order = np.lexsort((key[:, 1], key[:, 0]))
    morder = np.lexsort((mkey[:, 1], mkey[:, 0]))
    partner = np.empty(mesh.n_cells, dtype=np.int64)
    partner[morder] = order
    np.testing.assert_array_equal(key[partner], mkey)
    U, W = explosion(mesh)
    first = np.arange(mesh.n_cells) < partner
    U[~first], W[~first] = U[partner[~first]], W[partner[~first]]  # exactly symmetric start
    W[~first, :2] = -W[partner[~first], :2]
    U[~first, 1:3] = -U[partner[~first], 1:3]
    bcs = {z: "symmetry" for z in mesh.zone_names[1:]}
    s = gpu_solver(mesh, recon="FO", bcs=bcs, precision="fp64")
    s.set_state(U, W)
    s.run(0.5, 20)
    Ug, _ = s.get_state()
    assert s.status() == 0
    s.close()
    rho = Ug[:, 0]
    assert np.abs(rho - U[:, 0]).max() > 1e-3  # the state did evolve
    assert np.abs(rho - rho[partner]).max() < 1e-11 * rho.max()
    # momentum is odd under the point reflection
    assert np.abs(Ug[:, 1] + Ug[partner, 1]).max() < 1e-11 * np.abs(Ug[:, 1]).max()
