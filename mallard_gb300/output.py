"""VTU output of the solution (the reference's [[write_data]] with format
"vtu", src/io/data_writer.cpp:93-244), written asynchronously by the native
library: a write snapshots the requested arrays on the device and returns,
and a copy stream plus a worker thread produce <prefix>_<step:06d>.vtu while
the solver goes on."""

import ctypes as C

import numpy as np

from . import _native as N

VARIABLES = ("RHO", "RHOU_X", "RHOU_Y", "RHOE", "U_X", "U_Y", "P", "T", "H", "CFL")


class VtuWriter:
    """[[write_data]] of one solver: prefix, variables (names above) and
    interval as the reference's DataWriter::init (data_writer.cpp:29-75)."""

    def __init__(self, solver, prefix, variables, interval=1):
        self._lib = N.lib()
        self.prefix, self.variables, self.interval = prefix, list(variables), int(interval)
        if not self.variables:
            raise RuntimeError("DataWriter: No variables specified.")
        h = C.c_void_p()
        N.check(self._lib.mgpu_writer_create(solver._h, str(prefix).encode(), ",".join(self.variables).encode(),
                                             self.interval, C.byref(h)))
        self._h = h
        if not hasattr(solver, "_writers"):
            solver._writers = []
        solver._writers.append(self)  # closed before the solver's context

    def write(self, step, force=False):
        """DataWriter::write: when step % interval == 0 or force."""
        N.check(self._lib.mgpu_writer_write(self._h, int(step), 1 if force else 0))

    def flush(self):
        """Wait until every queued file is written."""
        N.check(self._lib.mgpu_writer_flush(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mgpu_writer_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()


def write_vtu(mesh, path, arrays):
    """The same file from host arrays: {name: [n_cells] values} in the mesh's
    cell order."""
    names = list(arrays)
    data = np.ascontiguousarray(np.stack([np.asarray(arrays[k], dtype=np.float64) for k in names]))
    cnames = (C.c_char_p * len(names))(*[n.encode() for n in names])
    N.check(N.lib().mgpu_vtu_write(mesh._h, str(path).encode(), len(names), C.cast(cnames, C.c_void_p),
                                   N.ptr(data)))


def read_vtu(path):
    """Read a file in this format back: (points [n][3], connectivity,
    offsets, types, {name: cell array}) -- for tests and post-processing."""
    import re
    raw = open(path, "rb").read()
    mark = raw.index(b'<AppendedData encoding="raw">\n_') + len(b'<AppendedData encoding="raw">\n_')
    head = raw[:mark].decode()
    blob = raw[mark:]
    out = {}
    arrays = re.findall(r'<DataArray type="(\w+)"(?: Name="(\w+)")?(?: NumberOfComponents="(\d)")? '
                        r'format="appended" offset="(\d+)">', head)
    types = {"Float64": np.float64, "UInt32": np.uint32, "UInt8": np.uint8}
    for typ, name, ncomp, off in arrays:
        off = int(off)
        n = int(np.frombuffer(blob[off:off + 4], dtype=np.uint32)[0])
        a = np.frombuffer(blob[off + 4:off + 4 + n], dtype=types[typ]).copy()
        out[name or "Points"] = a.reshape(-1, int(ncomp)) if ncomp else a
    cells = {k: v for k, v in out.items() if k not in ("Points", "connectivity", "offsets", "types")}
    return out["Points"], out["connectivity"], out["offsets"], out["types"], cells
