"""The FP32-bulk form against the FP64 oracle (corrected TENO weighting).

Reported and bounded: relative errors of face states and residuals per
stage, and the L1 / L-infinity density error, mass and energy drift after
100 steps.  Bounds are loose multiples of FP32 round-off; the benchmark's
bar is 1e-3 relative L1 density error.
"""

import numpy as np
import pytest

import mallard_gb300 as mg
from cases import GAS, explosion, four_quadrant, make_pair, perturbed, pulse, real_faces
from test_gpu_parity import tri_mesh
from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ic", [four_quadrant, perturbed])
def test_fp32_face_values(ic):
    m = tri_mesh(24, seed=20261203)
    s, oc = make_pair(m, variant="corrected", precision="fp32")
    U, _ = ic(m)
    F, M = s.calc_face_values(U, masks=True)
    Fo, Mo = oc.face_values(U, masks=True)
    assert (M == Mo).mean() > 0.99
    f, _ = real_faces(m)
    agree = (M == Mo).all(1)
    cells_ok = np.zeros(m.n_faces, dtype=bool)
    cof = m.cells_of_face[f, 0]
    cells_ok[f] = agree[cof]
    sel = f[cells_ok[f]]
    err = rel_err(F[sel][:, :, 0].reshape(len(sel), -1), Fo[sel][:, :, 0].reshape(len(sel), -1))
    assert err.max() < 1e-4, err.max()


@pytest.mark.parametrize("riemann", ["Rusanov", "HLLC"])
def test_fp32_residual(riemann):
    m = tri_mesh(24, seed=20261203)
    s, oc = make_pair(m, riemann=riemann, variant="corrected", precision="fp32")
    U, _ = perturbed(m)
    err = rel_err(s.calc_rhs(U), oc.calc_rhs(U))
    assert np.median(err) < 1e-5 and err.max() < 1e-2, (np.median(err), err.max())


def test_fp32_100_steps_errors():
    m = tri_mesh(32, seed=20261203)
    bcs = {z: "symmetry" for z in ("left", "right", "top", "bottom")}
    s, oc = make_pair(m, variant="corrected", bcs=bcs, precision="fp32")
    U, W = pulse(m)
    s.set_state(U, W)
    oc.set_state(U, W)
    s.run(0.5, 100)
    oc.run(0.5, 100)
    Ug, _ = s.get_state()
    Uo, _ = oc.get_state()
    vol = m.cell_volume
    l1 = np.sum(vol * np.abs(Ug[:, 0] - Uo[:, 0])) / np.sum(vol * np.abs(Uo[:, 0]))
    linf = np.max(np.abs(Ug[:, 0] - Uo[:, 0])) / np.max(np.abs(Uo[:, 0]))
    mass0 = np.sum(vol * U[:, 0])
    drift32 = abs(np.sum(vol * Ug[:, 0]) - mass0) / mass0
    drift64 = abs(np.sum(vol * Uo[:, 0]) - mass0) / mass0
    e_drift = abs(np.sum(vol * Ug[:, 3]) - np.sum(vol * Uo[:, 3])) / np.sum(vol * Uo[:, 3])
    print(f"fp32 vs fp64 after 100 steps: L1 {l1:.2e} Linf {linf:.2e} mass drift fp32 {drift32:.2e} "
          f"fp64 {drift64:.2e} energy diff {e_drift:.2e}")
    assert l1 < 1e-5 and linf < 1e-4
    assert drift32 < 1e-6 and e_drift < 1e-6


def test_fp32_primitives_and_time_step():
    """The FP32 form's steps carry no FP64 primitives: get_state recovers
    them from the conserved state it returns (bit for bit the primitive
    recovery of that state), and leaves the ones set_state was given alone
    until a step runs.  Its time step, computed in FP32 from the FP32 state
    copy, is the FP64 forms' to FP32 round-off."""
    m = tri_mesh(24, seed=20261203)
    s, _ = make_pair(m, variant="corrected", precision="fp32")
    U, W = explosion(m)
    s.set_state(U, W)
    np.testing.assert_array_equal(s.get_state()[1], W)
    s.run(0.5, 5)
    assert s.status() == 0
    Ug, Wg = s.get_state()
    np.testing.assert_array_equal(Wg, mg.primitives(Ug, **GAS))
    dt32, cfl32 = s.calc_dt(0.5)
    s64, _ = make_pair(m, variant="corrected", precision="fp64")
    s64.set_state(Ug)
    dt64, cfl64 = s64.calc_dt(0.5)
    print(f"FP32 time step vs FP64: {abs(dt32 - dt64) / dt64:.2e}")
    assert abs(dt32 - dt64) <= 1e-6 * dt64
    np.testing.assert_allclose(cfl32, cfl64, rtol=1e-5)
    s.close()
    s64.close()


@pytest.mark.parametrize("learned,variant", [(False, "corrected"), (True, "corrected"), (True, "robust")])
def test_launch_shapes_agree(learned, variant):
    """Every launch shape of the FP32 reconstruction (including the staged
    kernel, which reads its tables from shared memory filled by bulk async
    copies) gives the same bits, with and without the learned selector; a
    mesh whose cell count is not a multiple of the 8-cell tile exercises the
    staged kernel's idle lanes."""
    from mallard_gb300.selector import Selector, default_weights_path
    m = mg.Mesh.generate("cartesian_tri", 41, 39, 1.0, 1.0)
    m.permute_cells(9)
    assert m.n_cells % 8 != 0
    sel = Selector()
    sel.load(default_weights_path())
    out = []
    for shape in range(8):
        s, _ = make_pair(m, variant=variant, precision="fp32")
        if learned:
            s.attach_selector(sel)
        s.set_launch_shape(shape)
        U, W = explosion(m)
        s.set_state(U, W)
        s.run(0.5, 6)
        assert s.status() == 0
        out.append(s.get_state()[0])
        s.close()
    sel.close()
    for shape in range(1, 8):
        np.testing.assert_array_equal(out[shape], out[0], err_msg=f"shape {shape}")
