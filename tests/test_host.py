"""CPU tests of the host side: meshes, TENO tables, the C ABI surface,
argument checking and input parsing.  No GPU is touched here."""

import ctypes
import re
import subprocess

import numpy as np
import pytest

import mallard_gb300 as mg
from mallard_gb300 import _native as N
from mallard_gb300.solver import eval_exprtk, initial_state
from oracle import OracleCase, OracleMesh

MESH_FIELDS = ["node_coords", "cell_coords", "cell_volume", "face_area", "face_normals", "offsets_nodes_of_cell",
               "nodes_of_cell", "offsets_faces_of_cell", "faces_of_cell", "offsets_nodes_of_face", "nodes_of_face",
               "cells_of_face", "zone_offsets", "zone_faces"]


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    declared = N.exported_symbols()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(lib, name), name
    # and nm agrees that they are defined, exported functions
    out = subprocess.run(["nm", "-D", "--defined-only", str(N.LIB_PATH)], capture_output=True, text=True).stdout
    defined = set(re.findall(r" T (mgpu_\w+)", out))
    assert set(declared) <= defined


def test_library_has_sm103a_code():
    out = subprocess.run(["nm", "-D", str(N.LIB_PATH)], capture_output=True, text=True).stdout
    assert "cudaLaunchKernel" in out or "__cudaRegisterFatBinary" in out or "cudaGetLastError" in out


@pytest.mark.parametrize("mesh_type,nx,ny", [("cartesian_tri", 12, 10), ("cartesian", 7, 5), ("wedge", 9, 4),
                                              ("cartesian_tri", 40, 4), ("cartesian_tri", 1, 1)])
def test_mesh_generators_match_reference(mesh_type, nx, ny):
    a = mg.Mesh.generate(mesh_type, nx, ny, 1.3, 0.7)
    b = OracleMesh.generate(mesh_type, nx, ny, 1.3, 0.7)
    for f in MESH_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


def test_cartesian_tri_unused_faces_are_outside_zones():
    m = mg.Mesh.generate("cartesian_tri", 6, 5)
    used = np.zeros(m.n_faces, dtype=bool)
    used[m.zone_faces] = True
    assert m.n_faces == 3 * m.n_cells + 6 + 5
    assert used.sum() == 3 * m.n_cells // 2 + 6 + 5
    assert np.isnan(m.face_normals[~used]).all()


def test_permutation_is_a_relabelling():
    m = mg.Mesh.generate("cartesian_tri", 10, 8)
    ref = mg.Mesh.generate("cartesian_tri", 10, 8)
    perm = m.permute_cells(20261203)
    assert sorted(perm.tolist()) == list(range(m.n_cells))
    np.testing.assert_array_equal(m.cell_coords[perm], ref.cell_coords)
    np.testing.assert_array_equal(m.cell_volume[perm], ref.cell_volume)
    zf = ref.zone_faces
    cof = ref.cells_of_face[zf]
    mapped = np.where(cof >= 0, perm.astype(np.int64)[np.maximum(cof, 0)], -1)
    np.testing.assert_array_equal(m.cells_of_face[zf], mapped)
    # geometry re-derived from the permuted connectivity is unchanged
    g = OracleMesh.from_arrays(m)
    for f in MESH_FIELDS:
        np.testing.assert_array_equal(getattr(m, f), getattr(g, f), err_msg=f)


def test_permutation_is_seeded():
    a = mg.Mesh.generate("cartesian_tri", 9, 9)
    b = mg.Mesh.generate("cartesian_tri", 9, 9)
    np.testing.assert_array_equal(a.permute_cells(5), b.permute_cells(5))


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("seed", [None, 7])
def test_teno_tables_bit_identical_to_oracle(p, seed):
    m = mg.Mesh.generate("cartesian_tri", 16, 12)
    if seed is not None:
        m.permute_cells(seed)
    ta = mg.teno_tables(m, poly_order=p)
    tb = OracleCase(OracleMesh.from_arrays(m), poly_order=p).teno_tables()
    for k in ta:
        np.testing.assert_array_equal(ta[k], tb[k], err_msg=k)


def test_teno_tables_monomial_basis():
    m = mg.Mesh.generate("cartesian_tri", 10, 9)
    ta = mg.teno_tables(m, basis="monomial", poly_order=2)
    tb = OracleCase(OracleMesh.from_arrays(m), basis="monomial", poly_order=2).teno_tables()
    for k in ta:
        np.testing.assert_array_equal(ta[k], tb[k], err_msg=k)


def test_teno_table_structure():
    """Appendix facts the GPU layout relies on: dof 0 row and stencil column 0
    of every pseudo-inverse are exact zeros; stencils are full or empty."""
    m = mg.Mesh.generate("cartesian_tri", 14, 11)
    t = mg.teno_tables(m)
    K, M = 10, 20
    sizes = np.diff(t["offsets_stencils"])
    assert set(np.unique(sizes)) <= {0, M}
    assert (sizes.reshape(-1, 4)[:, 0] == M).all()
    mats = t["reconstruction_matrices"].reshape(-1, K, M)
    assert (mats[:, 0, :] == 0).all() and (mats[:, :, 0] == 0).all()
    st = t["stencils"].reshape(-1, M)
    first = np.repeat(np.arange(m.n_cells), 4)[sizes > 0]
    np.testing.assert_array_equal(st[:, 0], first)


def test_teno_rejects_quads():
    m = mg.Mesh.generate("cartesian", 6, 6)
    with pytest.raises(mg.MgpuError, match="triangular"):
        mg.teno_tables(m)


def test_teno_tables_on_a_delaunay_mesh():
    """Unstructured (jittered Delaunay) triangles through the FILE-style entry."""
    spatial = pytest.importorskip("scipy.spatial")
    m = delaunay_mesh(14, 9, seed=3)
    ta = mg.teno_tables(m)
    tb = OracleCase(OracleMesh.from_arrays(m)).teno_tables()
    for k in ta:
        np.testing.assert_array_equal(ta[k], tb[k], err_msg=k)
    assert spatial is not None


def delaunay_mesh(nx, ny, seed=0, Lx=1.0, Ly=1.0, jitter=0.2):
    """Jittered-lattice Delaunay triangulation with 4 boundary zones
    (right, top, left, bottom), as a mesh given by connectivity."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    xs, ys = np.meshgrid(np.linspace(0, Lx, nx + 1), np.linspace(0, Ly, ny + 1), indexing="ij")
    pts = np.stack([xs.ravel(), ys.ravel()], 1)
    h = min(Lx / nx, Ly / ny)
    inner = (pts[:, 0] > 0) & (pts[:, 0] < Lx) & (pts[:, 1] > 0) & (pts[:, 1] < Ly)
    pts[inner] += rng.uniform(-jitter, jitter, (inner.sum(), 2)) * h
    tri = Delaunay(pts).simplices.astype(np.int64)
    # counter-clockwise orientation
    a, b, c = pts[tri[:, 0]], pts[tri[:, 1]], pts[tri[:, 2]]
    cw = ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])) < 0
    tri[cw] = tri[cw][:, [0, 2, 1]]
    faces, cof, foc = {}, [], []
    for ci, t in enumerate(tri):
        fl = []
        for k in range(3):
            n0, n1 = int(t[k]), int(t[(k + 1) % 3])
            key = (min(n0, n1), max(n0, n1))
            if key not in faces:
                faces[key] = len(faces)
                cof.append([ci, -1])
            else:
                cof[faces[key]][1] = ci
            fl.append(faces[key])
        foc.append(fl)
    nof = np.array(list(faces.keys()), dtype=np.uint32)
    cof = np.array(cof, dtype=np.int32)
    bnd = np.where(cof[:, 1] < 0)[0]
    mid = pts[nof[bnd]].mean(1)
    zones = [np.where(cof[:, 1] >= 0)[0]]
    eps = 1e-9
    zones.append(bnd[np.abs(mid[:, 0] - Lx) < eps])
    zones.append(bnd[np.abs(mid[:, 1] - Ly) < eps])
    zones.append(bnd[np.abs(mid[:, 0]) < eps])
    zones.append(bnd[np.abs(mid[:, 1]) < eps])
    zoff = np.cumsum([0] + [len(z) for z in zones]).astype(np.uint32)
    n = len(tri)
    return mg.Mesh.from_connectivity(
        pts, np.arange(0, 3 * n + 1, 3), tri.ravel(), np.arange(0, 3 * n + 1, 3), np.array(foc).ravel(),
        np.arange(0, 2 * len(nof) + 1, 2), nof.ravel(), cof, zoff, np.concatenate(zones),
        zone_names=["interior", "right", "top", "left", "bottom"])


def test_from_connectivity_rejects_bad_indices():
    m = mg.Mesh.generate("cartesian_tri", 3, 3)
    bad = m.faces_of_cell.copy()
    bad[0] = m.n_faces + 5
    with pytest.raises(mg.MgpuError):
        mg.Mesh.from_connectivity(m.node_coords, m.offsets_nodes_of_cell, m.nodes_of_cell, m.offsets_faces_of_cell,
                                  bad, m.offsets_nodes_of_face, m.nodes_of_face, m.cells_of_face, m.zone_offsets,
                                  m.zone_faces)


def test_solver_argument_errors_match_reference_messages():
    m = mg.Mesh.generate("cartesian_tri", 4, 4)
    with pytest.raises(RuntimeError, match="Unknown Riemann solver type"):
        mg.Solver(m, riemann_solver="Roe")
    with pytest.raises(RuntimeError, match="Unknown face reconstruction type"):
        mg.Solver(m, face_reconstruction="WENO")
    with pytest.raises(RuntimeError, match="Unknown time integrator type"):
        mg.Solver(m, time_integrator="LSSSPRK3")


def test_config_defaults_are_the_reference_defaults():
    cfg = N.Config()
    N.lib().mgpu_config_defaults(ctypes.byref(cfg))
    assert (cfg.recon, cfg.basis, cfg.poly_order, cfg.max_stencil_size_factor) == (1, 1, 3, 2.0)
    assert (cfg.riemann_solver, cfg.gamma, cfg.p_min, cfg.p_max) == (2, 1.4, -1e20, 1e20)


def test_gas_constants_match_physics_test(golden):
    t = {x["name"]: x for x in golden["files"]["test/physics_test.cpp"]}["SetRCpCv"]
    s = t["scalars"]
    R, cp, cv = mg.gas_constants(s["gamma"], s["p_ref"], s["T_ref"], s["rho_ref"])
    exp = {e["args"][0]: float(e["args"][1]) for e in t["expects"] if not e["args"][1].strip().isidentifier()}
    assert abs(R - exp["physics.get_h_R()"]) < 1e-6
    assert abs(cp - exp["physics.get_h_Cp()"]) < 1e-6
    assert abs(cv - exp["physics.get_h_Cv()"]) < 1e-6


def test_exprtk_subset():
    x = np.array([0.1, 0.6, 0.9])
    y = np.array([0.9, 0.2, 0.85])
    expr = """var l := x <  0.8; \\
    var r := x >= 0.8; \\
    var b := y <  0.8; \\
    var t := y >= 0.8; \\
    1.5 * r * t + 0.5 * l * t + 0.1 * l * b + 0.3 * r * b"""
    np.testing.assert_array_equal(eval_exprtk(expr, x, y), [0.5, 0.1, 1.5])
    np.testing.assert_array_equal(eval_exprtk("0.0", x, y), [0.0, 0.0, 0.0])
    with pytest.raises(RuntimeError):
        eval_exprtk("__import__('os')", x, y)


def test_initial_state_matches_reference_formulas():
    m = mg.Mesh.generate("cartesian", 5, 1, 1.0, 0.2)
    gas = dict(gamma=1.4, p_ref=101325.0, T_ref=298.15, rho_ref=1.225)
    U, W = initial_state(m, {"type": "analytical", "rho": "var l := x < 0.5; 1.0 * l + 0.125 * (1 - l)",
                             "u": ["0.0", "0.0"], "p": "var l := x < 0.5; 1.0 * l + 0.1 * (1 - l)"}, gas)
    R, _, cv = mg.gas_constants(**gas)
    assert U[0, 0] == 1.0 and U[-1, 0] == 0.125
    T = 0.1 / (0.125 * R)
    assert W[-1, 3] == T and U[-1, 3] == 0.125 * (cv * T)
    Uc, Wc = initial_state(m, {"type": "constant", "u": [600.0, 0.0], "p": 101325.0, "T": 300.0}, gas)
    assert np.allclose(Uc[:, 1] / Uc[:, 0], 600.0)
    with pytest.raises(RuntimeError, match="Missing T"):
        initial_state(m, {"type": "constant", "u": [1.0, 0.0], "p": 1.0}, gas)


@pytest.mark.parametrize("which", ["cartesian_tri", "permuted", "ramp"])
def test_face_points_sit_on_reference_edges(which):
    """The FP32 form stores a 3-bit code per face slot instead of per-cell
    face shapes: mapped into its triangle's reference frame (nodes 0, 1, 2 at
    (0,0), (1,0), (0,1)), a face's Gauss points are those of the reference
    edge from node i0 to node i1, so six shape sets serve every cell.  Check
    that premise on the meshes the tests and benchmark use: every face of a
    cell joins two of its nodes, and the mapped points match the edge's."""
    if which == "ramp":
        m = mg.Mesh.ramp_channel(45, 15, 3.0, 1.0, 0.5, 15.0, 0.2, seed=7)
    else:
        m = mg.Mesh.generate("cartesian_tri", 17, 13, 1.0, 1.0)
        if which == "permuted":
            m.permute_cells(5)
    ref = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    gl = np.array([-1.0, 1.0]) / np.sqrt(3.0)  # two-point Gauss-Legendre on [-1, 1]
    X = m.node_coords
    codes = np.zeros(6, dtype=int)
    worst = 0.0
    for c in range(m.n_cells):
        nc = m.nodes_of_cell[m.offsets_nodes_of_cell[c]:m.offsets_nodes_of_cell[c + 1]]
        assert len(nc) == 3
        J = np.column_stack((X[nc[1]] - X[nc[0]], X[nc[2]] - X[nc[0]]))
        Ji = np.linalg.inv(J)
        for f in m.faces_of_cell[m.offsets_faces_of_cell[c]:m.offsets_faces_of_cell[c + 1]]:
            fn = m.nodes_of_face[m.offsets_nodes_of_face[f]:m.offsets_nodes_of_face[f + 1]]
            i0, i1 = int(np.flatnonzero(nc == fn[0])[0]), int(np.flatnonzero(nc == fn[1])[0])
            assert i0 != i1
            code = 2 * i0 if i1 == (i0 + 1) % 3 else 2 * i0 + 1
            codes[code] += 1
            x0, x1 = Ji @ (X[fn[0]] - X[nc[0]]), Ji @ (X[fn[1]] - X[nc[0]])
            for t in (gl + 1.0) * 0.5:
                mapped = x0 + t * (x1 - x0)
                edge = ref[i0] + t * (ref[i1] - ref[i0])
                worst = max(worst, np.abs(mapped - edge).max())
    assert worst < 1e-12, worst
    assert codes.sum() == 3 * m.n_cells


def test_oracle_permutation_equals_the_library_mesh_helper():
    """The oracle's seeded cell relabelling (used by the benchmark's CPU legs,
    which build the benchmark mesh without the GPU library) gives the
    library's permuted mesh array for array."""
    from oracle import OracleMesh
    for kind, nx, ny in (("cartesian_tri", 37, 23), ("cartesian", 20, 9), ("wedge", 30, 10)):
        m = mg.Mesh.generate(kind, nx, ny, 1.0, 1.0)
        p_lib = m.permute_cells(20261203)
        om = OracleMesh.generate(kind, nx, ny, 1.0, 1.0)
        p_ora = om.permute_cells(20261203)
        np.testing.assert_array_equal(p_lib, p_ora)
        for k in ("node_coords", "cell_coords", "cell_volume", "offsets_nodes_of_cell", "nodes_of_cell",
                  "offsets_faces_of_cell", "faces_of_cell", "cells_of_face", "zone_offsets", "zone_faces"):
            np.testing.assert_array_equal(np.asarray(getattr(m, k)), np.asarray(getattr(om, k)), err_msg=f"{kind} {k}")
