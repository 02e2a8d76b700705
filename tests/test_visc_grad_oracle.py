"""The viscous flux's cell gradients from the reconstruction, in the oracle
(the library's own definition; the reference solves the Euler equations).

Each cell's TENO polynomials are differentiated at its centroid, the
conserved variables' gradients turned into those of (u, v, T) by the
quotient rule with the cell averages.  For linear conserved fields every
candidate polynomial is the field itself, so the gradients are exact; the
robust variant zeroes them in cells with a boundary face (first order
there); Green-Gauss remains selectable.
"""

import numpy as np

import mallard_gb300 as mg
from cases import GAS, make_pair

R = GAS["p_ref"] / (GAS["T_ref"] * GAS["rho_ref"])
CV = R / (GAS["gamma"] - 1.0)

# linear conserved fields a + b x + c y: rho, rho u, rho v, rho E
COEF = np.array([[1.0, 0.10, -0.05], [0.3, 0.02, 0.04], [-0.2, 0.03, 0.01], [2.5, 0.15, -0.08]])


def _linear_state(mesh):
    X = mesh.cell_coords
    return COEF[:, 0][None, :] + X[:, :1] * COEF[:, 1][None, :] + X[:, 1:2] * COEF[:, 2][None, :]


def _exact_gradients(mesh):
    U = _linear_state(mesh)
    rho, m0, m1, Et = U.T
    g = COEF[:, 1:]  # [var][x, y]
    u, v, E = m0 / rho, m1 / rho, Et / rho
    ux = (g[1][0] - u * g[0][0]) / rho
    uy = (g[1][1] - u * g[0][1]) / rho
    vx = (g[2][0] - v * g[0][0]) / rho
    vy = (g[2][1] - v * g[0][1]) / rho
    ex = (g[3][0] - E * g[0][0]) / rho - (u * ux + v * vx)
    ey = (g[3][1] - E * g[0][1]) / rho - (u * uy + v * vy)
    return np.stack([ux, uy, vx, vy, ex / CV, ey / CV], axis=1)


def _boundary_cells(mesh):
    b = np.zeros(mesh.n_cells, dtype=bool)
    cof = mesh.cells_of_face
    b[cof[cof[:, 1] < 0, 0]] = True
    return b


def _case(mesh, variant):
    _, oc = make_pair(mesh, variant=variant, gpu=False)
    oc.set_viscous(1e-3, 1.0, 0.0, 0.72, gradients="recon")
    return oc


def test_reconstructed_gradients_are_exact_for_linear_fields():
    m = mg.Mesh.generate("cartesian_tri", 12, 10, 1.0, 1.0)
    m.permute_cells(3)
    oc = _case(m, "corrected")
    G = oc.viscous_gradients(_linear_state(m))
    ref = _exact_gradients(m)
    scale = np.abs(ref).max(axis=0)
    assert np.abs(G - ref).max(axis=0).max() < 1e-9 * scale.max(), np.abs(G - ref).max(axis=0) / scale


def test_reconstructed_gradients_on_a_delaunay_mesh():
    m = mg.Mesh.ramp_channel(24, 8, 3.0, 1.0, 0.5, 15.0, 0.2, seed=5)
    oc = _case(m, "corrected")
    G = oc.viscous_gradients(_linear_state(m))
    ref = _exact_gradients(m)
    assert np.abs(G - ref).max() < 1e-8 * np.abs(ref).max()


def test_robust_variant_zeroes_boundary_cells():
    """Robust: first order in cells with a boundary face, so zero gradients
    there; linear data stays within the central stencils' range elsewhere,
    so the interior gradients are the exact ones."""
    m = mg.Mesh.generate("cartesian_tri", 12, 10, 1.0, 1.0)
    oc = _case(m, "robust")
    G = oc.viscous_gradients(_linear_state(m))
    b = _boundary_cells(m)
    assert b.any() and (~b).any()
    assert np.all(G[b] == 0.0)
    ref = _exact_gradients(m)
    assert np.abs(G[~b] - ref[~b]).max() < 1e-9 * np.abs(ref).max()


def test_green_gauss_stays_selectable():
    """Green-Gauss of a linear field on interior cells of a uniform mesh is
    first-order accurate, not exact: the two definitions differ, and the
    option picks between them."""
    m = mg.Mesh.generate("cartesian_tri", 12, 10, 1.0, 1.0)
    _, oc = make_pair(m, variant="corrected", gpu=False)
    oc.set_viscous(1e-3, 1.0, 0.0, 0.72, gradients="green_gauss")
    U = _linear_state(m)
    Ggg = oc.viscous_gradients(U)
    oc.set_viscous(1e-3, 1.0, 0.0, 0.72, gradients="recon")
    Grc = oc.viscous_gradients(U)
    ref = _exact_gradients(m)
    b = _boundary_cells(m)
    assert np.abs(Grc - ref).max() < 1e-9 * np.abs(ref).max()
    assert np.abs(Ggg[~b] - ref[~b]).max() > 1e-6 * np.abs(ref).max()
