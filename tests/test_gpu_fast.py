"""The FP64 fast form (FMA contraction, symmetric smoothness indicator)
against the oracle: same decisions; face states within 1e-12; residuals
within FAST_STAGE_TOL = 1e-11 relative to max(|ref|, 1e-3 max|ref|): in
cells whose face fluxes nearly cancel, FMA round-off of a few ulps of the
flux shows up at ~2e-12 of that floor (the exact form is bit-identical)."""

import numpy as np
import pytest

import mallard_gb300 as mg
from cases import four_quadrant, make_pair, perturbed, pulse, real_faces
from test_gpu_parity import RUN_TOL, STAGE_TOL, assert_close, tri_mesh

FAST_STAGE_TOL = 1e-11

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("variant", ["reference", "corrected"])
@pytest.mark.parametrize("ic", [four_quadrant, perturbed])
def test_fast_face_values_and_masks(variant, ic):
    m = tri_mesh(24, seed=20261203)
    s, oc = make_pair(m, variant=variant, precision="fp64_fast")
    U, _ = ic(m)
    F, M = s.calc_face_values(U, masks=True)
    Fo, Mo = oc.face_values(U, masks=True)
    np.testing.assert_array_equal(M, Mo)
    f, _ = real_faces(m)
    assert_close(F[f][:, :, 0], Fo[f][:, :, 0], STAGE_TOL, what="fast face values")


@pytest.mark.parametrize("riemann", ["Rusanov", "HLLC"])
def test_fast_residual(riemann):
    m = tri_mesh(24, seed=20261203)
    s, oc = make_pair(m, riemann=riemann, variant="corrected", precision="fp64_fast")
    for ic in (four_quadrant, perturbed):
        U, _ = ic(m)
        assert_close(s.calc_rhs(U), oc.calc_rhs(U), FAST_STAGE_TOL, what=f"fast {riemann}")


def test_fast_100_steps_pulse():
    m = tri_mesh(16, seed=20261203)
    bcs = {z: "symmetry" for z in ("left", "right", "top", "bottom")}
    s, oc = make_pair(m, variant="corrected", bcs=bcs, precision="fp64_fast")
    U, W = pulse(m)
    s.set_state(U, W)
    oc.set_state(U, W)
    s.run(0.5, 100)
    oc.run(0.5, 100)
    assert_close(s.get_state()[0], oc.get_state()[0], RUN_TOL, what="fast 100 steps")


def test_unknown_precision_rejected():
    m = mg.Mesh.generate("cartesian_tri", 4, 4)
    with pytest.raises(RuntimeError, match="precision"):
        mg.Solver(m, precision="fp16")
