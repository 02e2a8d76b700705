"""The drop-in boundary from C: tests/abi_check.c includes
include/mallard_gb300.h as C99, links the library and calls its host-only
entry points (mesh generation and I/O, the TENO table build, VTU output,
error reporting) without a GPU."""

import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_c_client(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = ROOT / "mallard_gb300" / "_build" / "libmallard_gb300.so"
    if not lib.exists():
        pytest.skip("library not built")
    exe = tmp_path / "abi_check"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "abi_check.c"), "-o", str(exe), "-L", str(lib.parent), "-lmallard_gb300",
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    out = subprocess.run([str(exe), str(tmp_path)], check=True, capture_output=True, text=True).stdout
    fields = dict(kv.split("=", 1) for kv in out.split())
    assert fields["cells"] == "512" and fields["zones"] == "5" and fields["zone1"] == "right"
    assert int(fields["matrices"]) > 0 and fields["read_cells"] == "512" and fields["bad_arg"] == "1"
    assert (tmp_path / "mesh.mgm").exists() and (tmp_path / "rho_000000.vtu").stat().st_size > 1000
    import mallard_gb300 as mg
    m = mg.Mesh.generate("cartesian_tri", 16, 16, 1.0, 1.0)
    _, _, _, _, cells = mg.read_vtu(tmp_path / "rho_000000.vtu")
    assert abs(cells["RHO"] - (1.0 + m.cell_coords[:, 0])).max() == 0.0
