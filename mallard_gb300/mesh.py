"""Meshes for the GPU path: the reference's generators (built by the native
library) and meshes given as connectivity arrays.

Array names follow the reference Mesh (src/mesh/mesh.h:228-253).  Zone 0 is
"interior"; generated meshes add "right", "top", "left", "bottom" in that
order (src/mesh/mesh.cpp:408-498, 671-767).
"""

import ctypes as C

import numpy as np

from . import _native as N

GENERATED_ZONES = ["interior", "right", "top", "left", "bottom"]


def _arr(ptr, n, dtype, width=1):
    if n == 0:
        return np.zeros((0, width) if width > 1 else 0, dtype=dtype)
    ctype = {np.float64: C.c_double, np.uint32: C.c_uint32, np.int32: C.c_int32}[dtype]
    a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(n * width,)).copy()
    return a.reshape(-1, width) if width > 1 else a


class Mesh:
    """An owning host mesh (numpy copies of the native arrays)."""

    def __init__(self, handle, zone_names=None):
        self._h = handle
        self._lib = N.lib()
        v = N.MeshView()
        N.check(self._lib.mgpu_mesh_view(self._h, C.byref(v)))
        self._load(v)
        if zone_names:
            self.zone_names = list(zone_names)
            for i, name in enumerate(self.zone_names):
                N.check(self._lib.mgpu_mesh_set_zone_name(self._h, i, name.encode()))
        else:
            buf = C.create_string_buffer(4096)
            self.zone_names = []
            for i in range(self.n_zones):
                N.check(self._lib.mgpu_mesh_zone_name(self._h, i, buf, len(buf)))
                self.zone_names.append(buf.value.decode())

    def _load(self, v):
        self.n_nodes, self.n_cells, self.n_faces, self.n_zones = v.n_nodes, v.n_cells, v.n_faces, v.n_zones
        self.node_coords = _arr(v.node_coords, v.n_nodes, np.float64, 2)
        self.cell_coords = _arr(v.cell_coords, v.n_cells, np.float64, 2)
        self.cell_volume = _arr(v.cell_volume, v.n_cells, np.float64)
        self.face_area = _arr(v.face_area, v.n_faces, np.float64)
        self.face_normals = _arr(v.face_normals, v.n_faces, np.float64, 2)
        self.offsets_nodes_of_cell = _arr(v.offsets_nodes_of_cell, v.n_cells + 1, np.uint32)
        self.nodes_of_cell = _arr(v.nodes_of_cell, int(self.offsets_nodes_of_cell[-1]), np.uint32)
        self.offsets_faces_of_cell = _arr(v.offsets_faces_of_cell, v.n_cells + 1, np.uint32)
        self.faces_of_cell = _arr(v.faces_of_cell, int(self.offsets_faces_of_cell[-1]), np.uint32)
        self.offsets_nodes_of_face = _arr(v.offsets_nodes_of_face, v.n_faces + 1, np.uint32)
        self.nodes_of_face = _arr(v.nodes_of_face, int(self.offsets_nodes_of_face[-1]), np.uint32)
        self.cells_of_face = _arr(v.cells_of_face, v.n_faces, np.int32, 2)
        self.zone_offsets = _arr(v.zone_offsets, v.n_zones + 1, np.uint32)
        self.zone_faces = _arr(v.zone_faces, int(self.zone_offsets[-1]), np.uint32)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.mgpu_mesh_free(h)
            self._h = None

    @classmethod
    def generate(cls, mesh_type, nx, ny, Lx=1.0, Ly=1.0):
        """Mesh::init_cart / init_cart_tri / init_wedge (src/mesh/mesh.cpp:305-848)."""
        h = C.c_void_p()
        N.check(N.lib().mgpu_mesh_generate(N.MESH_TYPES[mesh_type], nx, ny, float(Lx), float(Ly), C.byref(h)))
        return cls(h)

    @classmethod
    def ramp_channel(cls, nx, ny, Lx=3.0, Ly=1.0, x0=0.5, ramp_deg=15.0, jitter=0.2, seed=0):
        """Jittered-lattice Delaunay triangulation of a channel with a ramp
        (2 nx ny triangles); zones interior, inflow, outflow, wall, top."""
        h = C.c_void_p()
        N.check(N.lib().mgpu_mesh_generate_ramp(nx, ny, float(Lx), float(Ly), float(x0), float(ramp_deg),
                                                float(jitter), int(seed), C.byref(h)))
        return cls(h)

    @classmethod
    def from_connectivity(cls, node_coords, offsets_nodes_of_cell, nodes_of_cell, offsets_faces_of_cell,
                          faces_of_cell, offsets_nodes_of_face, nodes_of_face, cells_of_face, zone_offsets,
                          zone_faces, zone_names=None):
        """A mesh from arrays (the reference's FILE type); geometry is derived."""
        a = [np.ascontiguousarray(x, dtype=d) for x, d in (
            (node_coords, np.float64), (offsets_nodes_of_cell, np.uint32), (nodes_of_cell, np.uint32),
            (offsets_faces_of_cell, np.uint32), (faces_of_cell, np.uint32), (offsets_nodes_of_face, np.uint32),
            (nodes_of_face, np.uint32), (cells_of_face, np.int32), (zone_offsets, np.uint32),
            (zone_faces, np.uint32))]
        h = C.c_void_p()
        N.check(N.lib().mgpu_mesh_from_connectivity(
            len(a[0]), N.ptr(a[0]), len(a[1]) - 1, N.ptr(a[1]), N.ptr(a[2]), N.ptr(a[3]), N.ptr(a[4]),
            len(a[5]) - 1, N.ptr(a[5]), N.ptr(a[6]), N.ptr(a[7]), len(a[8]) - 1, N.ptr(a[8]), N.ptr(a[9]),
            C.byref(h)))
        return cls(h, zone_names)

    @classmethod
    def read_gmsh(cls, path):
        """A 2-D Gmsh mesh (ASCII MSH 2.2 or 4.1): triangles and quadrilaterals
        as cells, boundary zones named by the physical groups of the line
        elements (the reference's unimplemented "file" mesh type)."""
        h = C.c_void_p()
        N.check(N.lib().mgpu_mesh_read_gmsh(str(path).encode(), C.byref(h)))
        return cls(h)

    @classmethod
    def read(cls, path):
        """A mesh in the library's binary format (Mesh.write)."""
        h = C.c_void_p()
        N.check(N.lib().mgpu_mesh_read(str(path).encode(), C.byref(h)))
        return cls(h)

    @classmethod
    def read_file(cls, path):
        """Gmsh (.msh) or the library's binary format, by the file's first bytes."""
        with open(path, "rb") as f:
            head = f.read(8)
        return cls.read(path) if head == b"MGPUMSH1" else cls.read_gmsh(path)

    def write(self, path):
        """Save in the library's binary format (connectivity, zones, names)."""
        N.check(self._lib.mgpu_mesh_write(self._h, str(path).encode()))

    def permute_cells(self, seed):
        """Relabel cells with a seeded random permutation; returns new_of_old."""
        perm = np.empty(self.n_cells, dtype=np.uint32)
        N.check(self._lib.mgpu_mesh_permute_cells(self._h, int(seed), N.ptr(perm)))
        v = N.MeshView()
        N.check(self._lib.mgpu_mesh_view(self._h, C.byref(v)))
        self._load(v)
        return perm

    def view(self):
        v = N.MeshView()
        N.check(self._lib.mgpu_mesh_view(self._h, C.byref(v)))
        return v

    def zone_index(self, name):
        try:
            return self.zone_names.index(name)
        except ValueError:
            raise RuntimeError(f"Boundary name {name} not found in mesh.") from None

    def zone(self, name):
        z = self.zone_index(name)
        return self.zone_faces[self.zone_offsets[z]:self.zone_offsets[z + 1]]


def teno_tables(mesh, basis="legendre", poly_order=3, stencil_factor=2.0, q_cell=0, q_face=0):
    """The tables TENO::init builds, in the reference's layout (host only)."""
    h = C.c_void_p()
    v = mesh.view()
    L = N.lib()
    N.check(L.mgpu_teno_tables_build(C.byref(v), N.BASIS[basis], poly_order, stencil_factor, q_cell, q_face,
                                     C.byref(h)))
    try:
        out = {}
        for name, (fid, dt) in N.TENO_FIELDS.items():
            n = L.mgpu_teno_tables_len(h, fid)
            a = np.empty(n, dtype=dt)
            if n:
                N.check(L.mgpu_teno_tables_copy(h, fid, N.ptr(a)))
            out[name] = a
        return out
    finally:
        L.mgpu_teno_tables_free(h)
