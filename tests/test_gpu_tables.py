"""The TENO least-squares tables built on the GPU (teno_tables.cu) against
the host build (host_teno.cpp, itself bit-identical to the oracle's
restatement of face_reconstruction.cpp:477-741): every table the kernels
read must agree bit for bit, in the FP64 and FP32 layouts, for p = 1..3 on
structured, permuted and Delaunay meshes."""

import numpy as np
import pytest

import mallard_gb300 as mg
from cases import GAS, explosion

pytestmark = pytest.mark.gpu


def _solver(mesh, precision, p, build, variant="corrected"):
    blist = [{"name": z, "type": "extrapolation"} for z in mesh.zone_names[1:]]
    return mg.Solver(mesh, face_reconstruction="TENO", basis_type="legendre", basis_order=p, riemann_solver="HLLC",
                     boundaries=blist, teno_variant=variant, precision=precision, table_build=build, **GAS)


def _meshes():
    a = mg.Mesh.generate("cartesian_tri", 24, 20, 1.0, 1.0)
    b = mg.Mesh.generate("cartesian_tri", 24, 24, 1.0, 1.0)
    b.permute_cells(5)
    c = mg.Mesh.ramp_channel(45, 15, 3.0, 1.0, 0.5, 15.0, 0.2, seed=7)
    return {"tri": a, "permuted": b, "ramp": c}


MESHES = _meshes()


@pytest.mark.parametrize("mesh", list(MESHES))
@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_tables_equal_host_tables(mesh, p, precision):
    if precision == "fp32" and p != 3:
        pytest.skip("the FP32 form is built for p = 3")
    m = MESHES[mesh]
    names = ["P32", "nb32", "phi32"] if precision == "fp32" else ["P", "areas", "nb", "phi"]
    with _solver(m, precision, p, "host") as sh, _solver(m, precision, p, "gpu") as sg:
        for name in names:
            th, tg = sh.get_table(name), sg.get_table(name)
            assert th.shape == tg.shape, name
            assert th.any(), name
            diff = np.flatnonzero(th.view(np.uint8) != tg.view(np.uint8))
            assert diff.size == 0, f"{name}: {diff.size} bytes differ"


def test_gpu_tables_same_run():
    """A GPU-built and a host-built solver give identical states after 10
    steps of the explosion (FP64 form)."""
    m = MESHES["permuted"]
    out = []
    for build in ("host", "gpu"):
        with _solver(m, "fp64", 3, build) as s:
            U, W = explosion(m)
            s.set_state(U, W)
            s.run(0.5, 10)
            out.append(s.get_state()[0])
    np.testing.assert_array_equal(out[0], out[1])


def test_monomial_basis_builds_on_the_host():
    """table_build="gpu" with the monomial basis (std::pow) takes the host
    path and so still equals the host build."""
    m = MESHES["tri"]
    blist = [{"name": z, "type": "extrapolation"} for z in m.zone_names[1:]]
    kw = dict(face_reconstruction="TENO", basis_type="monomial", basis_order=2, riemann_solver="HLLC",
              boundaries=blist, precision="fp64", **GAS)
    with mg.Solver(m, table_build="host", **kw) as sh, mg.Solver(m, table_build="gpu", **kw) as sg:
        np.testing.assert_array_equal(sh.get_table("P"), sg.get_table("P"))


def test_gpu_stencil_search_on_a_tied_mesh():
    """The stencil search on the GPU (stencil_search.cu) against the host's
    (host_teno.cpp): on a permuted 96x96 cartesian_tri mesh, where almost
    every ring of more than 16 cells holds equal distances, the neighbour
    tables -- every stencil's cells in order -- agree, so std::sort's order
    among ties is the host's."""
    m = mg.Mesh.generate("cartesian_tri", 96, 96, 1.0, 1.0)
    m.permute_cells(11)
    with _solver(m, "fp32", 3, "host") as sh, _solver(m, "fp32", 3, "gpu") as sg:
        th, tg = sh.get_table("nb32"), sg.get_table("nb32")
        assert th.shape == tg.shape
        np.testing.assert_array_equal(th, tg)


def test_gpu_stencil_search_errors_as_the_host():
    """A mesh too small for the stencil: the cells the GPU cannot fill go
    back to the host search, which raises the reference's error."""
    m = mg.Mesh.generate("cartesian_tri", 3, 2, 1.0, 1.0)
    for build in ("host", "gpu"):
        with pytest.raises(mg.MgpuError, match="Mesh too small for the TENO stencil size"):
            _solver(m, "fp64", 3, build)


def test_gpu_stencil_search_time():
    """At 1024x1024 (2,097,152 cells) the search on the GPU, with the
    neighbourhood graph and the stencil layout on the host, takes about
    0.16 s on a GB300 (the host search takes 1.4 s on its 16 cores)."""
    m = mg.Mesh.generate("cartesian_tri", 1024, 1024, 1.0, 1.0)
    with _solver(m, "fp32", 3, "gpu") as s:
        t = s.build_times()
    print("build times", t)
    assert t["stencil_search"] < 0.4, t
