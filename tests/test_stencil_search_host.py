"""The GPU stencil search's logic on the CPU: search_cell (stencil_search.cu)
compiled for the host -- with the same libstdc++ std::sort the device code
instantiates -- against the library's host search (host_teno.cpp, itself
bit-identical to the oracle): every stencil's cells in order, on a
tie-heavy structured mesh (equal distances in almost every ring of more
than 16 cells), a permuted one, a Delaunay mesh and p = 1..3."""

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import mallard_gb300 as mg
from mallard_gb300.mesh import teno_tables

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("no nvcc")
    out = tmp_path_factory.mktemp("search") / "libsearch_host.so"
    subprocess.run([nvcc, "-std=c++20", "--expt-relaxed-constexpr", "-fmad=false", "-Xcompiler",
                    "-fPIC,-ffp-contract=off", "-shared", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", str(ROOT / "include"), str(ROOT / "tests" / "stencil_search_host.cu"), "-o", str(out),
                    "-lcudart"], check=True)
    return C.CDLL(str(out))


def _graph(m):
    """First-order neighbourhoods (the cell itself included), sorted."""
    off, nb = [0], []
    for c in range(m.n_cells):
        t = {c}
        for k in range(m.offsets_faces_of_cell[c], m.offsets_faces_of_cell[c + 1]):
            a, b = m.cells_of_face[m.faces_of_cell[k]]
            if b >= 0:
                t.add(int(b if a == c else a))
        nb += sorted(t)
        off.append(len(nb))
    return np.array(off, np.uint32), np.array(nb, np.uint32)


def _check(lib, m, p):
    t = teno_tables(m, poly_order=p)
    K = (p + 1) * (p + 2) // 2
    M = 2 * K
    off, nb = _graph(m)
    n = m.n_cells
    flat = np.zeros(n * 4 * M, np.uint32)
    sizes = np.zeros(n * 4, np.uint8)
    status = np.zeros(n, np.uint8)
    v = m.view()
    p_ = lambda a: a.ctypes.data_as(C.c_void_p)
    redo = lib.search_host(C.byref(v), p_(off), p_(nb), M, p_(flat), p_(sizes), p_(status))
    assert redo == 0
    so, st = t["offsets_stencils"], t["stencils"]
    for i in range(n * 4):
        ref = st[so[i]:so[i + 1]]
        got = flat[i * M:i * M + int(sizes[i])]
        assert len(ref) == len(got) and (ref == got).all(), (i // 4, i % 4)


def test_structured_mesh_with_ties(harness):
    _check(harness, mg.Mesh.generate("cartesian_tri", 24, 20, 1.0, 1.0), 3)


def test_permuted_mesh(harness):
    m = mg.Mesh.generate("cartesian_tri", 24, 24, 1.0, 1.0)
    m.permute_cells(5)
    _check(harness, m, 3)


def test_delaunay_mesh(harness):
    _check(harness, mg.Mesh.ramp_channel(45, 15, 3.0, 1.0, 0.5, 15.0, 0.2, seed=7), 3)


@pytest.mark.parametrize("p", [1, 2])
def test_lower_orders(harness, p):
    _check(harness, mg.Mesh.generate("cartesian_tri", 20, 20, 1.0, 1.0), p)
