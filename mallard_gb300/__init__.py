"""mallard_gb300 -- GB300 (sm_103a) residual-and-update path for the Mallard
finite-volume Euler solver: TENO reconstruction, Riemann face flux with
boundary faces, deterministic residual gather and the SSPRK3 stage update
with primitive recovery and the CFL reduction, behind a C ABI
(include/mallard_gb300.h) whose kernels live in mallard_gb300/csrc.
"""

from ._native import MgpuError, lib  # noqa: F401
from .mesh import Mesh, teno_tables  # noqa: F401
from .output import VtuWriter, read_vtu, write_vtu  # noqa: F401
from .solver import (Solver, fp64_peak_gflops, gas_constants, initial_state, primitives,  # noqa: F401
                     riemann_flux, state_from_primitives)

__version__ = "0.1.0"
