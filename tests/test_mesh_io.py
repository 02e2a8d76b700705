"""Mesh ingest (host only): the Gmsh reader (MSH 2.2 and 4.1 ASCII) for the
reference's unimplemented "file" mesh type (src/mesh/mesh.cpp:41-43), the
library's binary mesh format, zone names, and the TOML front end's
[mesh] type = "file"."""

import numpy as np
import pytest

import mallard_gb300 as mg
from cases import GAS
from oracle import OracleCase, OracleMesh


def _square_parts(n=3):
    """Nodes (tag -> x, y), triangles (node tags) and boundary lines (tag
    pairs with a physical group) of the unit square split into 2 n^2
    triangles; groups 1 left "inlet", 2 right "outlet", 3 bottom and top
    "walls"."""
    tag = lambda i, j: 1 + i * (n + 1) + j  # noqa: E731
    nodes = {tag(i, j): (i / n, j / n) for i in range(n + 1) for j in range(n + 1)}
    tris = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = tag(i, j), tag(i + 1, j), tag(i + 1, j + 1), tag(i, j + 1)
            tris += [(a, b, c), (a, c, d)]
    lines = []
    for j in range(n):
        lines.append((tag(0, j), tag(0, j + 1), 1))
        lines.append((tag(n, j), tag(n, j + 1), 2))
    for i in range(n):
        lines.append((tag(i, 0), tag(i + 1, 0), 3))
        lines.append((tag(i, n), tag(i + 1, n), 3))
    return nodes, tris, lines, {1: "inlet", 2: "outlet", 3: "walls"}


def _write_v2(path, nodes, tris, lines, names):
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$PhysicalNames\n%d\n" % (len(names) + 1))
        for t, nm in names.items():
            f.write(f'1 {t} "{nm}"\n')
        f.write('2 10 "fluid"\n$EndPhysicalNames\n')
        f.write("$Nodes\n%d\n" % len(nodes))
        for t, (x, y) in nodes.items():
            f.write(f"{t} {x!r} {y!r} 0\n")
        f.write("$EndNodes\n$Elements\n%d\n" % (len(lines) + len(tris)))
        e = 1
        for a, b, g in lines:
            f.write(f"{e} 1 2 {g} {g} {a} {b}\n")
            e += 1
        for a, b, c in tris:
            f.write(f"{e} 2 2 10 1 {a} {b} {c}\n")
            e += 1
        f.write("$EndElements\n")


def _write_v4(path, nodes, tris, lines, names):
    # one curve entity per physical group, one surface
    groups = sorted(names)
    with open(path, "w") as f:
        f.write("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n$PhysicalNames\n%d\n" % (len(names) + 1))
        for t in groups:
            f.write(f'1 {t} "{names[t]}"\n')
        f.write('2 10 "fluid"\n$EndPhysicalNames\n')
        f.write(f"$Entities\n0 {len(groups)} 1 0\n")
        for t in groups:
            f.write(f"{t} 0 0 0 1 1 0 1 {t} 0\n")
        f.write("1 0 0 0 1 1 0 1 10 0\n$EndEntities\n")
        tags = list(nodes)
        f.write(f"$Nodes\n1 {len(nodes)} {min(tags)} {max(tags)}\n2 1 0 {len(nodes)}\n")
        for t in tags:
            f.write(f"{t}\n")
        for t in tags:
            x, y = nodes[t]
            f.write(f"{x!r} {y!r} 0\n")
        f.write("$EndNodes\n")
        n_el = len(lines) + len(tris)
        f.write(f"$Elements\n{len(groups) + 1} {n_el} 1 {n_el}\n")
        e = 1
        for t in groups:
            ls = [ln for ln in lines if ln[2] == t]
            f.write(f"1 {t} 1 {len(ls)}\n")
            for a, b, _ in ls:
                f.write(f"{e} {a} {b}\n")
                e += 1
        f.write(f"2 1 2 {len(tris)}\n")
        for a, b, c in tris:
            f.write(f"{e} {a} {b} {c}\n")
            e += 1
        f.write("$EndElements\n")


def _check_mesh(m, n):
    assert m.n_cells == 2 * n * n
    assert m.zone_names == ["interior", "inlet", "outlet", "walls"]
    np.testing.assert_allclose(m.cell_volume.sum(), 1.0, rtol=1e-14)
    sizes = np.diff(m.zone_offsets)
    assert list(sizes[1:]) == [n, n, 2 * n]
    # every face is in exactly one zone, interior faces have two cells
    zf = np.sort(m.zone_faces)
    np.testing.assert_array_equal(zf, np.arange(m.n_faces))
    assert (m.cells_of_face[m.zone("interior")][:, 1] >= 0).all()
    for z in ("inlet", "outlet", "walls"):
        assert (m.cells_of_face[m.zone(z)][:, 1] == -1).all()
    # faces_of_cell and cells_of_face agree
    for c in range(m.n_cells):
        for f in m.faces_of_cell[m.offsets_faces_of_cell[c]:m.offsets_faces_of_cell[c + 1]]:
            assert c in m.cells_of_face[f]
    # outward normals of each cell sum to zero (closed cells)
    for c in range(m.n_cells):
        s = np.zeros(2)
        for f in m.faces_of_cell[m.offsets_faces_of_cell[c]:m.offsets_faces_of_cell[c + 1]]:
            s += m.face_normals[f] * (1 if m.cells_of_face[f][0] == c else -1)
        assert np.abs(s).max() < 1e-14


@pytest.mark.parametrize("version", ["2.2", "4.1"])
def test_gmsh_square(tmp_path, version):
    parts = _square_parts(3)
    p = tmp_path / f"square{version}.msh"
    (_write_v2 if version == "2.2" else _write_v4)(p, *parts)
    m = mg.Mesh.read_gmsh(p)
    _check_mesh(m, 3)


def test_gmsh_versions_agree(tmp_path):
    parts = _square_parts(4)
    _write_v2(tmp_path / "a.msh", *parts)
    _write_v4(tmp_path / "b.msh", *parts)
    a, b = mg.Mesh.read_gmsh(tmp_path / "a.msh"), mg.Mesh.read_gmsh(tmp_path / "b.msh")
    for k in ("node_coords", "nodes_of_cell", "faces_of_cell", "nodes_of_face", "cells_of_face", "zone_offsets",
              "zone_faces", "face_normals", "cell_volume"):
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)


def test_gmsh_of_a_generated_mesh_gives_the_same_residual(tmp_path):
    """A cartesian_tri mesh written as Gmsh and read back: same cells, and a
    first-order residual equal to the generated mesh's (oracle) up to the
    order of each cell's face sums."""
    g = mg.Mesh.generate("cartesian_tri", 8, 6, 1.0, 0.75)
    nodes = {i + 1: (float(xy[0]), float(xy[1])) for i, xy in enumerate(g.node_coords)}
    tris = [tuple(int(x) + 1 for x in g.nodes_of_cell[g.offsets_nodes_of_cell[c]:g.offsets_nodes_of_cell[c + 1]])
            for c in range(g.n_cells)]
    lines, names = [], {}
    for zi, z in enumerate(g.zone_names[1:], start=1):
        names[zi] = z
        for f in g.zone(z):
            a, b = g.nodes_of_face[g.offsets_nodes_of_face[f]:g.offsets_nodes_of_face[f + 1]]
            lines.append((int(a) + 1, int(b) + 1, zi))
    _write_v2(tmp_path / "g.msh", nodes, tris, lines, names)
    r = mg.Mesh.read_gmsh(tmp_path / "g.msh")
    assert r.zone_names == g.zone_names
    np.testing.assert_array_equal(r.cell_coords, g.cell_coords)
    np.testing.assert_array_equal(r.cell_volume, g.cell_volume)
    rng = np.random.default_rng(3)
    U, _ = mg.state_from_primitives(1 + 0.1 * rng.random(g.n_cells), 0.2 * rng.random(g.n_cells),
                                    0.1 * rng.random(g.n_cells), 1 + 0.1 * rng.random(g.n_cells), **GAS)
    res = []
    for m in (g, r):
        om = OracleMesh.from_arrays(m)
        oc = OracleCase(om, recon="FO", basis="legendre", poly_order=1, riemann="HLLC", **GAS)
        for z in m.zone_names[1:]:
            oc.add_boundary(m.zone_index(z), "extrapolation", ())
        res.append(oc.calc_rhs(U))
    np.testing.assert_allclose(res[1], res[0], rtol=1e-12, atol=1e-12 * np.abs(res[0]).max())


@pytest.mark.parametrize("kind", ["cartesian_tri", "ramp"])
def test_binary_round_trip(tmp_path, kind):
    m = (mg.Mesh.generate("cartesian_tri", 7, 5, 2.0, 1.0) if kind == "cartesian_tri" else
         mg.Mesh.ramp_channel(12, 5, 3.0, 1.0, 0.5, 15.0, 0.2, seed=2))
    m.permute_cells(4)
    m.write(tmp_path / "m.mgm")
    r = mg.Mesh.read_file(tmp_path / "m.mgm")
    assert r.zone_names == m.zone_names
    for k in ("node_coords", "cell_coords", "cell_volume", "face_area", "face_normals", "offsets_nodes_of_cell",
              "nodes_of_cell", "offsets_faces_of_cell", "faces_of_cell", "offsets_nodes_of_face", "nodes_of_face",
              "cells_of_face", "zone_offsets", "zone_faces"):
        a, b = getattr(m, k), getattr(r, k)
        assert a.dtype == b.dtype and a.shape == b.shape, k
        assert a.tobytes() == b.tobytes(), k


def test_zone_names_and_errors(tmp_path):
    m = mg.Mesh.ramp_channel(6, 3, seed=1)
    assert m.zone_names == ["interior", "inflow", "outflow", "wall", "top"]
    assert mg.Mesh.generate("cartesian", 3, 2).zone_names == ["interior", "right", "top", "left", "bottom"]
    with pytest.raises(mg.MgpuError):
        mg.Mesh.read_gmsh(tmp_path / "missing.msh")
    (tmp_path / "bin.msh").write_text("$MeshFormat\n4.1 1 8\n$EndMeshFormat\n")
    with pytest.raises(mg.MgpuError):
        mg.Mesh.read_gmsh(tmp_path / "bin.msh")
    (tmp_path / "bad.mgm").write_bytes(b"MGPUMSH1" + b"\0" * 7)
    with pytest.raises(mg.MgpuError):
        mg.Mesh.read(tmp_path / "bad.mgm")


def test_toml_file_mesh(tmp_path):
    """[mesh] type = "file" reads the Gmsh file named by filename (relative
    to the input file), as the reference's input format has it."""
    _write_v2(tmp_path / "mesh.msh", *_square_parts(3))
    toml = tmp_path / "input.toml"
    toml.write_text('[mesh]\ntype = "file"\nfilename = "mesh.msh"\n')
    import tomllib
    inp = tomllib.loads(toml.read_text())
    assert inp["mesh"]["filename"] == "mesh.msh"
    m = mg.Mesh.read_file(tmp_path / inp["mesh"]["filename"])
    _check_mesh(m, 3)


@pytest.mark.gpu
def test_solver_from_toml_with_a_file_mesh(tmp_path):
    """Solver.from_toml with [mesh] type = "file": the Gmsh mesh is read
    relative to the input file, its zones take the [[boundaries]], and the
    solver runs first-order steps that keep a uniform state uniform."""
    _write_v2(tmp_path / "channel.msh", *_square_parts(6))
    toml = tmp_path / "input.toml"
    toml.write_text("\n".join([
        '[mesh]', 'type = "file"', 'filename = "channel.msh"',
        '[physics]', 'type = "euler"', 'gamma = 1.4', 'p_ref = 101325.0', 'T_ref = 298.15', 'rho_ref = 1.225',
        '[numerics]', 'riemann_solver = "HLLC"', 'time_integrator = "SSPRK3"',
        '[numerics.face_reconstruction]', 'type = "FO"',
        '[[boundaries]]', 'name = "inlet"', 'type = "extrapolation"',
        '[[boundaries]]', 'name = "outlet"', 'type = "extrapolation"',
        '[[boundaries]]', 'name = "walls"', 'type = "symmetry"',
        '[initialize]', 'type = "constant"', 'u = [0.3, 0.0]', 'p = 1.0', 'T = 0.003',
    ]) + "\n")
    solver, U0, W0, run = mg.Solver.from_toml(str(toml))
    assert solver.mesh.n_cells == 72
    solver.set_state(U0, W0)
    solver.run(0.5, 10)
    U, _ = solver.get_state()
    assert solver.status() == 0
    np.testing.assert_allclose(U, U0, rtol=1e-12, atol=1e-12 * np.abs(U0).max())
    solver.close()
