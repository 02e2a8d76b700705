"""Case builders shared by the tests: the same mesh, numerics, boundaries and
initial state handed to the GPU path (mallard_gb300.Solver) and the oracle.

Initial states are seeded or analytic stand-ins for the benchmark configs
(four-quadrant Riemann problem, Sod tube, smooth density wave, the wedge
inflow); no external dataset is involved.
"""

import numpy as np

import mallard_gb300 as mg
from oracle import OracleCase, OracleMesh

GAS = dict(gamma=1.4, p_ref=101325.0, T_ref=298.15, rho_ref=1.225)

# 2D four-quadrant Riemann problem, split at x = y = 0.8 (rho, u, v, p)
QUADRANTS = {
    "UR": (1.5, 0.0, 0.0, 1.5),
    "UL": (0.532258064516129, 1.206045378311055, 0.0, 0.3),
    "LL": (0.137992831541219, 1.206045378311055, 1.206045378311055, 0.029032258064516),
    "LR": (0.532258064516129, 0.0, 1.206045378311055, 0.3),
}


def four_quadrant(mesh, split=0.8, states=None):
    """states: optional (rho, u, v, p) for UR, UL, LL, LR."""
    x, y = mesh.cell_coords[:, 0], mesh.cell_coords[:, 1]
    r, t = x >= split, y >= split
    prim = np.zeros((mesh.n_cells, 4))
    for i, (key, sel) in enumerate((("UR", r & t), ("UL", ~r & t), ("LL", ~r & ~t), ("LR", r & ~t))):
        prim[sel] = QUADRANTS[key] if states is None else states[i]
    return mg.state_from_primitives(prim[:, 0], prim[:, 1], prim[:, 2], prim[:, 3], **GAS)


def explosion(mesh, center=(0.5, 0.5), radius=0.2, inside=(1.0, 1.0), outside=(0.125, 0.1)):
    """Cylindrical Sod problem: (rho, p) inside and outside a circle, at rest."""
    x, y = mesh.cell_coords[:, 0] - center[0], mesh.cell_coords[:, 1] - center[1]
    inn = x * x + y * y < radius * radius
    rho = np.where(inn, inside[0], outside[0])
    p = np.where(inn, inside[1], outside[1])
    z = np.zeros(mesh.n_cells)
    return mg.state_from_primitives(rho, z, z, p, **GAS)


def sod(mesh, split=0.5):
    x = mesh.cell_coords[:, 0]
    left = x < split
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    return mg.state_from_primitives(rho, 0 * x, 0 * x, p, **GAS)


def smooth(mesh, amp=0.2, u=0.3, v=0.2):
    x, y = mesh.cell_coords[:, 0], mesh.cell_coords[:, 1]
    rho = 1.0 + amp * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y)
    p = 1.0 + 0.1 * np.cos(2 * np.pi * x)
    return mg.state_from_primitives(rho, 0 * x + u, 0 * x + v, p, **GAS)


def pulse(mesh, amp=0.2, width2=0.02):
    """An acoustic pulse at rest in the centre of the unit square."""
    x, y = mesh.cell_coords[:, 0], mesh.cell_coords[:, 1]
    g = np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / width2)
    return mg.state_from_primitives(1.0 + amp * g, 0 * x, 0 * x, 1.0 + amp * g, **GAS)


def uniform(mesh, rho=1.3, u=0.4, v=-0.25, p=0.9):
    n = mesh.n_cells
    return mg.state_from_primitives(np.full(n, rho), np.full(n, u), np.full(n, v), np.full(n, p), **GAS)


def perturbed(mesh, seed=1234, base=smooth, scale=0.05):
    """A seeded random perturbation of a base state (cell-wise, positive)."""
    rng = np.random.default_rng(seed)
    U, _ = base(mesh)
    rho = U[:, 0] * (1.0 + scale * rng.uniform(-1, 1, mesh.n_cells))
    u = U[:, 1] / U[:, 0] + scale * rng.uniform(-1, 1, mesh.n_cells)
    v = U[:, 2] / U[:, 0] + scale * rng.uniform(-1, 1, mesh.n_cells)
    p = 1.0 + scale * rng.uniform(-1, 1, mesh.n_cells)
    return mg.state_from_primitives(rho, u, v, p, **GAS)


BC_DATA = {
    "symmetry": {},
    "extrapolation": {},
    "wall_adiabatic": {},
    "upt": {"u": [0.9, 0.1], "p": 1.1, "T": 1.1 / (1.2 * (101325.0 / (298.15 * 1.225)))},
    "p_out": {"p": 0.95},
}


def make_pair(mesh, recon="TENO", riemann="HLLC", variant="reference", bcs=None, poly_order=3, p_min=-1e20,
              p_max=1e20, reorder=True, precision="fp64", integrator="SSPRK3", gpu=True):
    """A GPU solver and an oracle case on the same mesh and numerics (gpu
    False: the oracle case alone, the solver None)."""
    bcs = bcs or {name: "extrapolation" for name in mesh.zone_names[1:]}
    blist = []
    for name, typ in bcs.items():
        d = {"name": name, "type": typ}
        d.update(BC_DATA[typ])
        blist.append(d)
    s = mg.Solver(mesh, face_reconstruction=recon, basis_type="legendre", basis_order=poly_order,
                  riemann_solver=riemann, boundaries=blist, teno_variant=variant, reorder=reorder, p_min=p_min,
                  p_max=p_max, precision=precision, time_integrator=integrator, **GAS) if gpu else None
    om = OracleMesh.from_arrays(mesh)
    oc = OracleCase(om, recon=recon, basis="legendre", poly_order=poly_order, riemann=riemann, p_min=p_min,
                    p_max=p_max, **GAS)
    oc.set_teno_variant({"reference": 0, "corrected": 1, "robust": 2}[variant])
    oc.set_integrator(integrator)
    for b in blist:
        data = ()
        if b["type"] == "upt":
            data = (b["u"][0], b["u"][1], b["p"], b["T"])
        elif b["type"] == "p_out":
            data = (b["p"],)
        oc.add_boundary(mesh.zone_index(b["name"]), b["type"], data)
    oc._om = om  # keep the oracle mesh alive
    return s, oc


def real_faces(mesh):
    """(face ids, side-1 valid) over faces in any zone."""
    f = mesh.zone_faces
    interior = np.zeros(mesh.n_faces, dtype=bool)
    interior[mesh.zone(mesh.zone_names[0])] = True
    return f, interior[f]
