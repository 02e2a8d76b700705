"""The learned stencil selector on the GPU, against the CPU oracle
(oracle/mlp.py): training gradients, tensor-core inference, harvested
features and labels, and the learned FP32 form against the plain FP64 run.
"""

import numpy as np
import pytest

import mallard_gb300 as mg
from mallard_gb300.selector import Selector, default_weights_path
from mallard_gb300.mesh import teno_tables
from cases import explosion, make_pair, perturbed
from oracle import mlp

pytestmark = pytest.mark.gpu


def _rows(n, seed):
    r = np.random.default_rng(seed)
    X = np.clip(r.normal(0, 0.5, (n, mlp.IN)), -1, 1).astype(np.float32)
    Y = r.integers(0, mlp.NCLS, (n, 4)).astype(np.uint8)
    return X, Y


def test_gradient_matches_oracle():
    with Selector(seed=11) as s:
        p = s.params
        X, Y = _rows(300, 1)
        g, loss = s.gradient(X, Y)
        lo, go = mlp.loss_and_grad(p.astype(np.float64), X, Y)
        assert abs(loss - lo) <= 1e-5 * abs(lo)
        scale = np.abs(go).max()
        err = np.abs(g - go).max() / scale
        print(f"selector gradient: max |g - g_oracle| / max|g_oracle| = {err:.2e}")
        assert err < 1e-4
        # every block of the packed layout is exercised
        for a, b in [(mlp.OFF_W1, mlp.OFF_B1), (mlp.OFF_B1, mlp.OFF_W2), (mlp.OFF_W2, mlp.OFF_B2),
                     (mlp.OFF_B2, mlp.OFF_W3), (mlp.OFF_W3, mlp.OFF_B3), (mlp.OFF_B3, mlp.N_PARAMS)]:
            assert np.abs(go[a:b]).max() > 0
            assert np.abs(g[a:b] - go[a:b]).max() <= 1e-4 * scale


def test_inference_matches_bf16_oracle():
    with Selector(seed=5) as s:
        r = np.random.default_rng(2)
        p = s.params
        p[mlp.OFF_B1:mlp.OFF_W2] = r.normal(0, 0.2, mlp.HID)
        p[mlp.OFF_B3:] = r.normal(0, 0.5, mlp.OUT)
        s.params = p
        # up to 60,000 rows: 469 row blocks, more CTAs than fit at once
        for n in (1, 127, 128, 1000, 60000):
            X, _ = _rows(n, 10 + n)
            L, P = s.infer(X, threshold=0.6)
            Lo = mlp.infer_bf16(p, X)
            err = np.abs(L - Lo).max()
            assert err < 2e-2 * max(1.0, np.abs(Lo).max()), (n, err)
            Po = mlp.predict(Lo, 0.6)
            # predictions agree wherever the oracle's margins are clear
            z = Lo.reshape(n, 4, 8)
            srt = np.sort(z, axis=2)
            clear = (srt[:, :, -1] - srt[:, :, -2]) > 0.05
            assert np.all((P & 0x7F)[clear] == (Po & 0x7F)[clear])


def test_training_learns_a_rule():
    r = np.random.default_rng(3)
    X = np.clip(r.normal(0, 0.5, (20000, mlp.IN)), -1, 1).astype(np.float32)
    A = r.normal(0, 1, (mlp.IN, 32))
    Y = (X @ A).reshape(-1, 4, 8).argmax(axis=2).astype(np.uint8)
    with Selector(seed=4) as s:
        s.add_samples(X, Y)
        assert len(s) == 20000
        Xr, Yr = s.samples(100, 5)
        np.testing.assert_array_equal(Xr, X[100:105])
        np.testing.assert_array_equal(Yr, Y[100:105])
        losses = s.train(epochs=12, batch=1024, lr=3e-3, seed=1)
        assert losses[-1] < 0.5 * losses[0], losses
        L, _ = s.infer(X[:4000], threshold=0.9)
        acc = (L.reshape(-1, 4, 8).argmax(2) == Y[:4000]).mean()
        print(f"synthetic rule: loss {losses[0]:.3f} -> {losses[-1]:.3f}, accuracy {acc:.3f}")
        assert acc > 0.85
        # deterministic: the same seed gives the same parameters
        p1 = s.params
    with Selector(seed=4) as s2:
        s2.add_samples(X, Y)
        s2.train(epochs=12, batch=1024, lr=3e-3, seed=1)
        np.testing.assert_array_equal(s2.params, p1)


def test_harvest_matches_oracle_features_and_masks():
    m = mg.Mesh.generate("cartesian_tri", 12, 12, 1.0, 1.0)
    s, _ = make_pair(m, variant="corrected", reorder=False)
    U, W = perturbed(m)
    s.set_state(U, W)
    _, masks = s.calc_face_values(U, masks=True)
    with Selector() as sel:
        n = sel.harvest(s, keep_central=1.0, seed=0)
        assert n == m.n_cells
        X, Y = sel.samples()
    t = teno_tables(m)
    Xo = mlp.features(U, t["offsets_stencils"], t["stencils"])
    np.testing.assert_allclose(X, Xo, rtol=0, atol=2e-6)
    np.testing.assert_array_equal(Y, mlp.class_of_mask(masks))


def _harvest_explosions(sel, n, seeds, steps=60, every=15):
    """Harvest seeded cylindrical explosions (random centre, radius and
    states) from FP64-fast runs, every few steps."""
    m = mg.Mesh.generate("cartesian_tri", n, n, 1.0, 1.0)
    rows = 0
    for sd in seeds:
        r = np.random.default_rng(sd)
        s, _ = make_pair(m, variant="corrected", precision="fp64_fast")
        U, W = explosion(m, center=r.uniform(0.3, 0.7, 2), radius=r.uniform(0.1, 0.25),
                         inside=(r.uniform(0.5, 2), r.uniform(0.5, 2)), outside=(r.uniform(0.1, 0.4), r.uniform(0.05, 0.3)))
        s.set_state(U, W)
        for k in range(steps // every):
            s.run(0.5, every)
            rows += sel.harvest(s, keep_central=0.3, seed=100 * sd + k)
        s.close()
    return rows


def test_learned_form_error_and_gain():
    with Selector(seed=9) as sel, Selector(seed=9) as untrained:
        rows = _harvest_explosions(sel, 48, seeds=[1, 2, 3, 4])
        losses = sel.train(epochs=10, batch=2048, lr=3e-3, seed=0)
        # a fresh problem on a permuted mesh: explosion off centre, 64 x 64
        m2 = mg.Mesh.generate("cartesian_tri", 64, 64, 1.0, 1.0)
        m2.permute_cells(20261203)
        U, W = explosion(m2, center=(0.45, 0.55), radius=0.18)
        ref, _ = make_pair(m2, variant="corrected", precision="fp64")
        ref.set_state(U, W)
        ref.run(0.5, 60)
        Ur, _ = ref.get_state()
        res = {}
        for name, selector in (("plain", None), ("untrained", untrained), ("trained", sel)):
            f32, _ = make_pair(m2, variant="corrected", precision="fp32")
            if selector is not None:
                f32.attach_selector(selector, threshold=0.9)
            f32.set_state(U, W)
            f32.run(0.5, 60)
            Ug, _ = f32.get_state()
            vol = m2.cell_volume
            l1 = np.sum(vol * np.abs(Ug[:, 0] - Ur[:, 0])) / np.sum(vol * np.abs(Ur[:, 0]))
            st = f32.selector_stats() if selector is not None else None
            res[name] = (l1, st)
    l1p = res["plain"][0]
    l1u, stu = res["untrained"]
    l1t, stt = res["trained"]
    frac_u = stu["stencils_evaluated"] / stu["stencils_full"]
    frac_t = stt["stencils_evaluated"] / stt["stencils_full"]
    print(f"selector: {rows} rows, loss {losses[0]:.3f} -> {losses[-1]:.3f}")
    print(f"learned form vs FP64 (explosion, 60 steps): L1 plain fp32 {l1p:.2e}, untrained {l1u:.2e} "
          f"(stencils {frac_u:.3f}), trained {l1t:.2e} (stencils {frac_t:.3f}, confident cells "
          f"{stt['confident_cells'] / stt['cells']:.3f})")
    assert stt["error"] == 0 and stu["error"] == 0
    # a small network trained in seconds: a loose error bound here; the
    # shipped network is held to 1e-3 below
    assert np.isfinite(l1t) and l1t <= 5e-3
    # the trained network skips work the untrained one cannot
    assert frac_t < 0.6 and frac_t < frac_u


@pytest.mark.parametrize("interval", [1, 2, 4])
@pytest.mark.parametrize("problem", ["explosion", "four_quadrant"])
def test_shipped_selector_error_and_work(problem, interval):
    """The trained weights shipped with the package, on problems they were not
    trained on, at the default central threshold 0.995 with one prediction per
    step: density L1 error against the plain FP64 run and the share of the
    full TENO work, held to the 1e-3 bar.  The explosion runs the corrected
    weighting for 80 steps; the four-quadrant problem runs the robust one
    (with which it stays finite to its end time) for 120 steps."""
    from mallard_gb300.selector import default_weights_path
    from cases import four_quadrant
    path = default_weights_path()
    if not path.exists():
        pytest.skip("no shipped selector weights")
    m = mg.Mesh.generate("cartesian_tri", 96, 96, 1.0, 1.0)
    m.permute_cells(7)
    if problem == "explosion":
        U, W = explosion(m, center=(0.52, 0.47), radius=0.22, inside=(1.2, 1.5), outside=(0.2, 0.15))
        steps, variant = 80, "corrected"
    else:
        U, W = four_quadrant(m)
        steps, variant = 120, "robust"
    ref, _ = make_pair(m, variant=variant, precision="fp64")
    ref.set_state(U, W)
    ref.run(0.5, steps)
    Ur, _ = ref.get_state()
    with Selector() as sel:
        sel.load(path)
        f32, _ = make_pair(m, variant=variant, precision="fp32")
        f32.attach_selector(sel, interval=interval)
        f32.set_state(U, W)
        f32.run(0.5, steps)
        Ug, _ = f32.get_state()
        st = f32.selector_stats()
    vol = m.cell_volume
    l1 = np.sum(vol * np.abs(Ug[:, 0] - Ur[:, 0])) / np.sum(vol * np.abs(Ur[:, 0]))
    frac = st["stencils_evaluated"] / st["stencils_full"]
    print(f"shipped selector on {problem}, interval {interval}: L1 {l1:.2e}, stencils {frac:.3f}, confident cells "
          f"{st['confident_cells'] / st['cells']:.3f}")
    assert st["error"] == 0
    assert np.isfinite(l1) and l1 <= 1e-3
    assert frac < 0.8


@pytest.mark.parametrize("n", [20, 160])
def test_in_solver_predictions_match_harvested_features(n):
    """The FP32 form's in-solver inference (features built from the FP32
    stage state inside the tcgen05 kernel) predicts exactly what the
    stand-alone inference predicts from the harvested features of the same
    state: same features, same BF16 operands, same logits, on a small mesh
    and on one of 51,200 cells (400 row blocks)."""
    m = mg.Mesh.generate("cartesian_tri", n, n, 1.0, 1.0)
    U, W = explosion(m, radius=0.25)
    with Selector() as sel:
        sel.load(default_weights_path())
        s, _ = make_pair(m, variant="corrected", precision="fp32", reorder=False)
        s.attach_selector(sel, threshold=0.98, directional_threshold=2.0)
        s.set_state(U, W)
        s.run(0.5, 1)   # predicts from the initial state
        P_in = s.selector_predictions(raw=True)
        s.close()
        h, _ = make_pair(m, variant="corrected", precision="fp64", reorder=False)
        h.set_state(U, W)
        sel.clear()
        assert sel.harvest(h, keep_central=1.0, seed=0) == m.n_cells
        X, _ = sel.samples()
        h.close()
        _, P = sel.infer(X, threshold=0.98, directional_threshold=2.0)
    np.testing.assert_array_equal(P_in, P)
