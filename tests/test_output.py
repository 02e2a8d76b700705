"""VTU output in the reference's format (DataWriter::write_vtu,
src/io/data_writer.cpp:93-244): the host writer on CPU, the asynchronous
device writer on the GPU."""

import numpy as np
import pytest

import mallard_gb300 as mg
from cases import GAS, explosion


def _check_layout(path, mesh):
    raw = open(path, "rb").read()
    head = raw[:raw.index(b"<AppendedData")].decode()
    assert head.startswith('<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="0.1" '
                           'byte_order="LittleEndian">\n')
    assert f'<Piece NumberOfPoints="{mesh.n_nodes}" NumberOfCells="{mesh.n_cells}">' in head
    assert raw.endswith(b"\n</AppendedData>\n</VTKFile>\n")
    pts, conn, offs, types, cells = mg.read_vtu(path)
    np.testing.assert_array_equal(pts[:, :2], mesh.node_coords)
    assert (pts[:, 2] == 0).all()
    np.testing.assert_array_equal(conn, mesh.nodes_of_cell)
    np.testing.assert_array_equal(offs, mesh.offsets_nodes_of_cell[1:])
    assert (types == 7).all()
    return cells


@pytest.mark.parametrize("kind", ["cartesian_tri", "cartesian"])
def test_host_vtu_file(tmp_path, kind):
    m = mg.Mesh.generate(kind, 9, 7, 1.0, 0.5)
    r = np.random.default_rng(2)
    arrays = {"RHO": r.random(m.n_cells), "P": r.random(m.n_cells) * 1e5, "CFL": r.random(m.n_cells)}
    mg.write_vtu(m, tmp_path / "x_000000.vtu", arrays)
    cells = _check_layout(tmp_path / "x_000000.vtu", m)
    assert list(cells) == ["RHO", "P", "CFL"]
    for k, v in arrays.items():
        np.testing.assert_array_equal(cells[k], v)


@pytest.mark.gpu
def test_async_writer_matches_state(tmp_path):
    """Files written while the solver keeps stepping hold the state of the
    step they were taken at: the snapshot is ordered after that step and
    before the next."""
    m = mg.Mesh.generate("cartesian_tri", 24, 24, 1.0, 1.0)
    m.permute_cells(3)
    blist = [{"name": z, "type": "symmetry"} for z in m.zone_names[1:]]
    s = mg.Solver(m, face_reconstruction="TENO", basis_type="legendre", basis_order=3, riemann_solver="HLLC",
                  boundaries=blist, teno_variant="corrected", precision="fp32", **GAS)
    U, W = explosion(m)
    s.set_state(U, W)
    w = mg.VtuWriter(s, str(tmp_path / "sol"), ["RHO", "RHOU_X", "RHOE", "U_Y", "P", "T", "H", "CFL"], interval=5)
    expect = {}
    for step in range(0, 16):
        if step % 5 == 0:
            dt, cfl = s.calc_dt(0.5)
            Us, Ws = s.get_state()
            expect[step] = (Us, Ws, cfl)
        w.write(step)                 # no file for steps that are not multiples of 5
        s.run(0.5, 1)                 # the solver goes on while files are written
    w.flush()
    files = sorted(p.name for p in tmp_path.iterdir())
    assert files == ["sol_000000.vtu", "sol_000005.vtu", "sol_000010.vtu", "sol_000015.vtu"]
    for step, (Us, Ws, cfl) in expect.items():
        cells = _check_layout(tmp_path / f"sol_{step:06d}.vtu", m)
        np.testing.assert_array_equal(cells["RHO"], Us[:, 0])
        np.testing.assert_array_equal(cells["RHOU_X"], Us[:, 1])
        np.testing.assert_array_equal(cells["RHOE"], Us[:, 3])
        np.testing.assert_array_equal(cells["U_Y"], Ws[:, 1])
        np.testing.assert_array_equal(cells["P"], Ws[:, 2])
        np.testing.assert_array_equal(cells["T"], Ws[:, 3])
        np.testing.assert_array_equal(cells["H"], Ws[:, 4])
        np.testing.assert_array_equal(cells["CFL"], cfl)
    w.write(16, force=True)
    s.close()                          # closes (flushes) the writer first
    assert (tmp_path / "sol_000016.vtu").exists()
    with pytest.raises(mg.MgpuError):
        s2 = mg.Solver(m, face_reconstruction="FO", boundaries=blist, **GAS)
        try:
            mg.VtuWriter(s2, str(tmp_path / "bad"), ["RHO", "VORTICITY"])
        finally:
            s2.close()
