"""mgpu_calc_dt_noalloc: the CFL time step for callers that must not allocate
device memory once they are stepping (an application whose device memory
all comes from its own pool, a real-time loop that cannot take the
device-wide synchronisation of cudaMalloc/cudaFree).  It must give the same
dt and per-cell spectral radius as mgpu_calc_dt, including on consecutive
calls that reuse its static scratch.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest

import mallard_gb300 as mg
from mallard_gb300 import _native as N
from cases import four_quadrant

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the per-stage tolerance of the parity tests


def _dev_ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_calc_dt_noalloc_matches_calc_dt_on_two_calls():
    torch = pytest.importorskip("torch")
    m = mg.Mesh.generate("cartesian_tri", 48, 40, 1.0, 1.0)
    m.permute_cells(11)
    s = mg.Solver(m, teno_variant="corrected", boundaries=[{"name": z, "type": "extrapolation"}
                                                          for z in ("right", "top", "left", "bottom")])
    U, W = four_quadrant(m)
    s.set_state(U, W)
    lib = N.lib()
    dt_dev = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    rho_dev = torch.full((m.n_cells,), -1.0, dtype=torch.float64, device="cuda")
    for call in range(2):
        dt_ref, cfl_local = s.calc_dt(0.5)
        N.check(lib.mgpu_calc_dt_noalloc(s._h, 0.5, _dev_ptr(dt_dev), _dev_ptr(rho_dev)))
        s.synchronize()
        dt = float(dt_dev.cpu().numpy()[0])
        rho = rho_dev.cpu().numpy()
        assert abs(dt - dt_ref) <= TOL * abs(dt_ref), (call, dt, dt_ref)
        np.testing.assert_allclose(dt_ref * rho, cfl_local, rtol=TOL, atol=0)
        s.take_step(dt_ref)  # the second call sees a new state in the same scratch
    s.close()


def test_calc_dt_noalloc_fp32_form_bit_for_bit():
    """The FP32 form: both entry points compute the radius in FP32 from the
    FP32 state rows, with the same roundings, after steps as before them."""
    torch = pytest.importorskip("torch")
    m = mg.Mesh.generate("cartesian_tri", 48, 40, 1.0, 1.0)
    m.permute_cells(11)
    s = mg.Solver(m, teno_variant="corrected", precision="fp32",
                  boundaries=[{"name": z, "type": "extrapolation"} for z in ("right", "top", "left", "bottom")])
    U, W = four_quadrant(m)
    s.set_state(U, W)
    lib = N.lib()
    dt_dev = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    rho_dev = torch.full((m.n_cells,), -1.0, dtype=torch.float64, device="cuda")
    for call in range(2):
        dt_ref, cfl_local = s.calc_dt(0.5)
        N.check(lib.mgpu_calc_dt_noalloc(s._h, 0.5, _dev_ptr(dt_dev), _dev_ptr(rho_dev)))
        s.synchronize()
        assert float(dt_dev.cpu().numpy()[0]) == dt_ref, call
        np.testing.assert_array_equal(dt_ref * rho_dev.cpu().numpy(), cfl_local)
        s.run(0.5, 3)
    s.close()


def test_calc_dt_noalloc_after_a_larger_mesh():
    """A smaller mesh after a larger one: stale partial slots are never read."""
    torch = pytest.importorskip("torch")
    lib = N.lib()
    dt_dev = torch.zeros(1, dtype=torch.float64, device="cuda")
    for n in (64, 12):
        m = mg.Mesh.generate("cartesian_tri", n, n, 1.0, 1.0)
        s = mg.Solver(m, teno_variant="corrected", boundaries=[{"name": "left", "type": "symmetry"}])
        U, W = four_quadrant(m)
        s.set_state(U, W)
        dt_ref, _ = s.calc_dt(0.3)
        N.check(lib.mgpu_calc_dt_noalloc(s._h, 0.3, _dev_ptr(dt_dev), None))
        s.synchronize()
        assert abs(float(dt_dev.cpu().numpy()[0]) - dt_ref) <= TOL * abs(dt_ref)
        s.close()


def test_calc_dt_noalloc_fp64_fast_form():
    """The FP64-fast form: mgpu_calc_dt uses reciprocals and FMA there, this
    entry point the plain divisions, so the two agree to 1e-12, not bit for
    bit."""
    torch = pytest.importorskip("torch")
    m = mg.Mesh.generate("cartesian_tri", 40, 40, 1.0, 1.0)
    m.permute_cells(5)
    s = mg.Solver(m, teno_variant="corrected", precision="fp64_fast",
                  boundaries=[{"name": z, "type": "extrapolation"} for z in ("right", "top", "left", "bottom")])
    U, W = four_quadrant(m)
    s.set_state(U, W)
    lib = N.lib()
    dt_dev = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    for call in range(2):
        dt_ref, _ = s.calc_dt(0.5)
        N.check(lib.mgpu_calc_dt_noalloc(s._h, 0.5, _dev_ptr(dt_dev), None))
        s.synchronize()
        dt = float(dt_dev.cpu().numpy()[0])
        assert abs(dt - dt_ref) <= TOL * abs(dt_ref), (call, dt, dt_ref)
        s.take_step(dt_ref)
    s.close()


def test_calc_dt_noalloc_flags_a_nan_state():
    """A non-finite cell gives a non-finite dt, which the status word reports
    (bit 1), as it does for the main path's time step."""
    torch = pytest.importorskip("torch")
    m = mg.Mesh.generate("cartesian_tri", 16, 16, 1.0, 1.0)
    s = mg.Solver(m, teno_variant="corrected",
                  boundaries=[{"name": z, "type": "extrapolation"} for z in ("right", "top", "left", "bottom")])
    U, W = four_quadrant(m)
    U[7, :] = np.nan
    W[7, :] = np.nan
    s.set_state(U, W)
    assert s.status() == 0
    dt_dev = torch.zeros(1, dtype=torch.float64, device="cuda")
    N.check(N.lib().mgpu_calc_dt_noalloc(s._h, 0.5, _dev_ptr(dt_dev), None))
    s.synchronize()
    assert not np.isfinite(float(dt_dev.cpu().numpy()[0])) or float(dt_dev.cpu().numpy()[0]) < 0
    assert s.status() & 2
    s.close()
