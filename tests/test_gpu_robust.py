"""The robust TENO variant on the GPU (no reference counterpart): the FP64
path against the oracle's restatement at the parity bar (1e-12 per stage,
1e-10 after 100 steps), the guarded star pressure against the oracle, the
FP32 and learned forms against the FP64 path at the spec bar (density
L1 <= 1e-3), and the batched form against single-case runs, bit for bit."""

import numpy as np
import pytest

import mallard_gb300 as mg
from cases import GAS, four_quadrant, make_pair, perturbed
from test_gpu_parity import RUN_TOL, STAGE_TOL, assert_close, tri_mesh
from test_robust_oracle import EXPANSION, GAMMA, _h

pytestmark = pytest.mark.gpu


def _l1(m, U, Uref):
    vol = m.cell_volume
    return float(np.sum(vol * np.abs(U[:, 0] - Uref[:, 0])) / np.sum(vol * np.abs(Uref[:, 0])))


@pytest.mark.parametrize("kind", ["HLL", "HLLC"])
def test_guarded_star_pressure_matches_oracle(kind):
    from oracle import Oracle
    o = Oracle()
    r = np.random.default_rng(11)
    cases = [EXPANSION] + [dict(rl=r.uniform(0.1, 2), ul=r.uniform(-1.5, 1.5, 2), pl=r.uniform(1e-5, 2),
                                rr=r.uniform(0.1, 2), ur=r.uniform(-1.5, 1.5, 2), pr=r.uniform(1e-5, 2))
                           for _ in range(200)]
    n = np.tile([1.0, 0.0], (len(cases), 1))
    arr = lambda key: np.array([np.asarray(c[key], dtype=float) for c in cases])  # noqa: E731
    rl, ul, pl, rr, ur, pr = (arr(k) for k in ("rl", "ul", "pl", "rr", "ur", "pr"))
    g = np.full(len(cases), GAMMA)
    args = (n, rl, ul, pl, g, _h(rl, 0, pl), rr, ur, pr, g, _h(rr, 0, pr))
    F_plain = mg.riemann_flux(kind, *args)
    F_guard = mg.riemann_flux(kind, *args, guard=True)
    assert np.isnan(F_plain[0]).all() and np.isfinite(F_guard).all()
    ref = np.array([o.riemann_flux(kind, n[i], rl[i], ul[i], pl[i], GAMMA, _h(rl[i], 0, pl[i]), rr[i], ur[i], pr[i],
                                   GAMMA, _h(rr[i], 0, pr[i]), guard=True) for i in range(len(cases))])
    np.testing.assert_allclose(F_guard, ref, rtol=1e-12, atol=1e-14)
    fin = np.isfinite(F_plain).all(axis=1)
    np.testing.assert_array_equal(F_guard[fin], F_plain[fin])


@pytest.mark.parametrize("ic", [four_quadrant, perturbed])
def test_face_values_and_residual(ic):
    m = tri_mesh(24, seed=20261203)
    s, oc = make_pair(m, variant="robust")
    U, _ = ic(m)
    F, M = s.calc_face_values(U, masks=True)
    Fo, Mo = oc.face_values(U, masks=True)
    np.testing.assert_array_equal(M, Mo, err_msg="TENO decision masks differ")
    from cases import real_faces
    f, interior = real_faces(m)
    a = np.concatenate([F[f][:, :, 0].reshape(len(f), -1), F[f[interior]][:, :, 1].reshape(interior.sum(), -1)])
    b = np.concatenate([Fo[f][:, :, 0].reshape(len(f), -1), Fo[f[interior]][:, :, 1].reshape(interior.sum(), -1)])
    assert_close(a, b, STAGE_TOL, min_exact=0.99, what="face values")
    for riemann in ("Rusanov", "HLLC"):
        s2, oc2 = make_pair(m, variant="robust", riemann=riemann)
        assert_close(s2.calc_rhs(U), oc2.calc_rhs(U), STAGE_TOL, min_exact=0.95, what=riemann)
        s2.close()
    s.close()


def test_100_steps_four_quadrant():
    """100 CFL steps of the four-quadrant problem (transmissive boundaries,
    HLLC): the corrected weighting goes non-finite within ~15 steps here."""
    m = tri_mesh(32, seed=20261203)
    s, oc = make_pair(m, variant="robust")
    U, W = four_quadrant(m)
    s.set_state(U, W)
    oc.set_state(U, W)
    t_gpu = s.run(0.5, 100)
    t_ora = oc.run(0.5, 100)
    assert abs(t_gpu - t_ora) <= 1e-12 * t_ora
    Ug, _ = s.get_state()
    Uo, _ = oc.get_state()
    assert np.isfinite(Uo).all()
    assert_close(Ug, Uo, RUN_TOL, what="U after 100 steps")
    assert s.status() == 0
    s.close()


@pytest.mark.parametrize("precision", ["fp64_fast", "fp32"])
def test_fast_forms_to_the_end_time(precision):
    """The four-quadrant problem at 64 x 64 to t = 0.3 (the FP64 form's step
    count) in the FMA and FP32 forms against the FP64 form: density L1 within
    the spec bar 1e-3 (a TENO decision within round-off of its
    threshold can flip at a shock, so neither is bit-close over a whole run),
    and the same time within 1e-3 (each form takes its own CFL steps, whose
    sizes follow the largest wave speed of its own state)."""
    m = tri_mesh(64, seed=20261203)
    U, W = four_quadrant(m)
    s, _ = make_pair(m, variant="robust", precision="fp64")
    s.set_state(U, W)
    t, steps = 0.0, 0
    while t < 0.3:
        t += s.run(0.5, 1)
        steps += 1
    assert s.status() == 0
    ref = s.get_state()[0]
    s.close()
    s, _ = make_pair(m, variant="robust", precision=precision)
    s.set_state(U, W)
    t2 = s.run(0.5, steps)
    assert s.status() == 0
    out = s.get_state()[0]
    s.close()
    l1 = _l1(m, out, ref)
    print(f"robust {precision} vs fp64, t = {t:.4f} ({steps} steps, {precision} t = {t2:.4f}), 64^2: "
          f"density L1 {l1:.2e}")
    assert np.isfinite(out).all() and abs(t2 - t) <= 1e-3 * t
    assert l1 <= 1e-3, l1


@pytest.mark.parametrize("interval", [2, 4])
def test_learned_form_four_quadrant(interval):
    """FP32 + the shipped selector with the robust variant on the
    four-quadrant problem at 128 x 128 for 300 steps, predicting every 2nd
    or 4th step: density L1 against the plain FP64 run within the
    spec bar."""
    from mallard_gb300.selector import Selector, default_weights_path
    path = default_weights_path()
    if not path.exists():
        pytest.skip("no shipped selector weights")
    m = tri_mesh(128, seed=7)
    U, W = four_quadrant(m)
    ref, _ = make_pair(m, variant="robust", precision="fp64")
    ref.set_state(U, W)
    ref.run(0.5, 300)
    Ur, _ = ref.get_state()
    ref.close()
    with Selector() as sel:
        sel.load(path)
        f32, _ = make_pair(m, variant="robust", precision="fp32")
        f32.attach_selector(sel, interval=interval)
        f32.set_state(U, W)
        f32.run(0.5, 300)
        Ug, _ = f32.get_state()
        st = f32.selector_stats()
        assert f32.status() == 0
        f32.close()
    l1 = _l1(m, Ug, Ur)
    frac = st["stencils_evaluated"] / st["stencils_full"]
    print(f"robust learned form, four-quadrant 128^2, 300 steps, interval {interval}: L1 {l1:.2e}, "
          f"stencils {frac:.3f}")
    assert st["error"] == 0 and np.isfinite(l1) and l1 <= 1e-3
    assert frac < 0.8


@pytest.mark.parametrize("shape", [0, 4, 7])
def test_batch_matches_single_case_runs(shape):
    """Random four-quadrant states (the ensemble's distribution) on two
    meshes, batched with the robust variant, against single-case runs."""
    from mallard_gb300.batch import Batch
    bcs = [{"name": z, "type": "extrapolation"} for z in ("right", "top", "left", "bottom")]
    ma = mg.Mesh.generate("cartesian_tri", 16, 16, 1.0, 1.0)
    mb = mg.Mesh.generate("cartesian_tri", 24, 24, 1.0, 1.0)
    r = np.random.default_rng(20261203)
    states = []
    for g, (m, n) in enumerate(((ma, 3), (mb, 2))):
        for k in range(n):
            q = np.column_stack([r.uniform(0.1, 2.0, 4), r.uniform(-1.5, 1.5, 4), r.uniform(-1.5, 1.5, 4),
                                 r.uniform(0.03, 2.0, 4)])
            U, W = four_quadrant(m, split=r.uniform(0.3, 0.7), states=[tuple(x) for x in q])
            states.append((g, k, U, W))
    steps = 40
    with Batch((ma, mb), [3, 2], boundaries=bcs, teno_variant="robust", **GAS) as b:
        b.set_launch_shape(shape)
        for g, k, U, W in states:
            b.set_state(g, k, U, W)
        b.run(0.5, steps)
        b.synchronize()
        flags, times = b.status()
        assert (flags == 0).all(), flags
        for i, (g, k, U, W) in enumerate(states):
            m = (ma, mb)[g]
            s, _ = make_pair(m, variant="robust", precision="fp32")
            s.set_state(U, W)
            t = s.run(0.5, steps)
            Us, _ = s.get_state()
            s.close()
            np.testing.assert_array_equal(b.get_state(g, k)[0], Us, err_msg=f"case {i}")
            assert times[i] == t
