"""Parity at the benchmark's own configuration: the four-quadrant workload
on cartesian_tri 1024 x 1024 (2,097,152 cells, seed 20261203, RCM inside the
library), robust TENO + HLLC, transmissive boundaries, CFL 0.5; and one
residual of the 4M-cell supersonic wedge (ramp channel 2449 x 816).

The oracle builds its tables over all host threads (bit-identical to its
serial build) and scatters with atomics (Kokkos::OpenMP's order), so the
comparison is at the parity bar, not bit for bit:
* FP64 path: decision masks exact; one stage residual 1e-12; 8 SSPRK3 steps
  1e-10 (relative to max(|ref|, 1e-3 max|ref| of the variable));
* FP32 + learned form (the headline): density L1 <= 1e-3 against the FP64
  path after the same 8 steps, with the location of the largest difference
  reported.
"""

import os

import numpy as np
import pytest

import mallard_gb300 as mg
from cases import four_quadrant, make_pair
from conftest import rel_err

pytestmark = pytest.mark.gpu

N = 1024
SEED = 20261203
STEPS = 8


@pytest.fixture(scope="module")
def threads():
    from oracle import Oracle
    o = Oracle()
    o.set_threads(max(1, os.cpu_count() or 1))
    yield
    o.set_threads(1)


@pytest.fixture(scope="module")
def bench_case(threads):
    m = mg.Mesh.generate("cartesian_tri", N, N, 1.0, 1.0)
    m.permute_cells(SEED)
    s, oc = make_pair(m, variant="robust")
    U, W = four_quadrant(m)
    yield m, s, oc, U, W
    s.close()


def test_bench_mesh_stage_residual_and_masks(bench_case):
    m, s, oc, U, W = bench_case
    _, M = s.calc_face_values(U, masks=True)
    _, Mo = oc.face_values(U, masks=True)
    np.testing.assert_array_equal(M, Mo, err_msg="TENO decision masks differ")
    r, ro = s.calc_rhs(U), oc.calc_rhs(U)
    err = rel_err(r, ro)
    print(f"bench mesh: stage residual max rel err {err.max():.2e}, bit-identical {np.mean(r == ro):.4f}")
    assert err.max() <= 1e-12


def test_bench_mesh_8_steps_and_learned_error(bench_case):
    m, s, oc, U, W = bench_case
    s.set_state(U, W)
    oc.set_state(U, W)
    t_gpu = s.run(0.5, STEPS)
    t_ora = oc.run(0.5, STEPS)
    assert abs(t_gpu - t_ora) <= 1e-12 * t_ora
    Ug, _ = s.get_state()
    Uo, _ = oc.get_state()
    assert np.isfinite(Uo).all() and s.status() == 0
    err = rel_err(Ug, Uo)
    print(f"bench mesh: {STEPS} steps max rel err {err.max():.2e}")
    assert err.max() <= 1e-10
    from mallard_gb300.selector import Selector, default_weights_path
    path = default_weights_path()
    if not path.exists():
        pytest.skip("no shipped selector weights")
    with Selector() as sel:
        sel.load(path)
        f32, _ = make_pair(m, variant="robust", precision="fp32", gpu=True)
        f32.attach_selector(sel, interval=4)
        f32.set_state(U, W)
        f32.run(0.5, STEPS)
        Ul, _ = f32.get_state()
        assert f32.status() == 0
        f32.close()
    vol = m.cell_volume
    d = np.abs(Ul[:, 0] - Ug[:, 0])
    l1 = float(np.sum(vol * d) / np.sum(vol * np.abs(Ug[:, 0])))
    i = int(np.argmax(d))
    print(f"bench mesh: learned form density L1 {l1:.2e}, L-inf {d.max() / np.abs(Ug[:, 0]).max():.2e} at "
          f"{m.cell_coords[i].round(4)} (rho {Ug[i, 0]:.4f})")
    assert l1 <= 1e-3


def test_wedge_4m_residual(threads):
    """One FP64 residual of the 4M-cell viscous wedge (Delaunay ramp channel,
    corrected TENO + Rusanov, no-slip walls, Re 1e5, cell gradients of the
    reconstructed polynomials) against the oracle, within 2e-12 relative.
    The viscous flux has no reference counterpart; the bar is twice the
    inviscid one because the two sides sum a cell's face fluxes in different
    orders (the oracle scatters face by face, the GPU gathers per cell) and
    the rounding of fluxes that largely cancel reaches 1.2e-12 of the
    residual in one entry of the 16M."""
    from cases import GAS
    from mallard_gb300.train_selector import wedge_setup, wedge_viscosity
    from oracle import OracleCase, OracleMesh
    m = mg.Mesh.ramp_channel(3 * 816 + 1, 816, 3.0, 1.0, 0.5, 15.0, 0.2, seed=SEED)
    s, U, W = wedge_setup(m, mach=2.5, precision="fp64", reynolds=1e5)
    oc = OracleCase(OracleMesh.from_arrays(m), recon="TENO", basis="legendre", poly_order=3, riemann="Rusanov", **GAS)
    oc.set_teno_variant(1)
    visc = wedge_viscosity(2.5, 1.4, 1.0, 1e5)
    oc.set_viscous(visc["mu_ref"], visc.get("T_mu_ref", 1.0), visc.get("sutherland_S", 0.0),
                   visc.get("prandtl", 0.72))
    R = GAS["p_ref"] / (GAS["T_ref"] * GAS["rho_ref"])
    u = 2.5 * float(np.sqrt(GAS["gamma"] * 1.0 / 1.4))
    for name, bc, data in (("inflow", "upt", (u, 0.0, 1.0, 1.0 / (1.4 * R))), ("outflow", "p_out", (1.0,)),
                           ("wall", "wall_adiabatic", ()), ("top", "wall_adiabatic", ())):
        oc.add_boundary(m.zone_index(name), bc, data)
    # a developed-looking state: the uniform inflow with a seeded perturbation
    r = np.random.default_rng(3)
    U = U * (1.0 + 0.02 * r.uniform(-1, 1, U.shape))
    err = rel_err(s.calc_rhs(U), oc.calc_rhs(U))
    print(f"wedge 4M: residual max rel err {err.max():.2e}, entries above 1e-12: {(err > 1e-12).sum()}")
    assert err.max() <= 2e-12
    s.close()
