"""CPU checks of the selector oracle (oracle/mlp.py) that the GPU tests use:
its gradient against finite differences, BF16 rounding, the class <-> mask
map and the feature construction on a small mesh."""

import numpy as np

import mallard_gb300 as mg
from mallard_gb300.mesh import teno_tables
from oracle import mlp


def _params(seed):
    r = np.random.default_rng(seed)
    W1 = r.uniform(-1, 1, (mlp.IN, mlp.HID)) / np.sqrt(mlp.IN)
    W2 = r.uniform(-1, 1, (mlp.HID, mlp.HID)) / np.sqrt(mlp.HID)
    W3 = r.uniform(-1, 1, (mlp.HID, mlp.OUT)) / np.sqrt(mlp.HID)
    return mlp.pack(W1, r.normal(0, 0.1, mlp.HID), W2, r.normal(0, 0.1, mlp.HID), W3, r.normal(0, 0.1, mlp.OUT))


def test_gradient_finite_difference():
    r = np.random.default_rng(7)
    p = _params(3)
    X = r.normal(0, 0.7, (9, mlp.IN))
    Y = r.integers(0, mlp.NCLS, (9, 4))
    _, g = mlp.loss_and_grad(p, X, Y)
    idx = np.concatenate([r.choice(np.arange(mlp.OFF_B1), 12, replace=False),
                          np.arange(mlp.OFF_B1, mlp.OFF_B1 + 3), r.choice(np.arange(mlp.OFF_W2, mlp.OFF_B2), 8),
                          r.choice(np.arange(mlp.OFF_W3, mlp.OFF_B3), 8), np.arange(mlp.OFF_B3, mlp.OFF_B3 + 4)])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp.loss_and_grad(pp, X, Y)[0] - mlp.loss_and_grad(pm, X, Y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.001953125, 1.0029296875, -3.14159, 0.0], dtype=np.float32)
    b = mlp.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: nearest even is 1
    assert b[0] == 1.0 and b[1] == 1.0
    assert b[2] == np.float32(1.0078125)
    assert b[3] == 1.0 and b[4] == 1.0
    assert abs(b[5] - x[5]) <= abs(x[5]) * 2 ** -8 and b[6] == 0.0


def test_class_mask_roundtrip():
    masks = np.array([1, 2, 4, 6, 8, 10, 12, 14])
    c = mlp.class_of_mask(masks)
    assert list(c) == [0, 1, 2, 3, 4, 5, 6, 7]
    assert list(mlp.mask_of_class(c)) == list(masks)


def test_features_shape_and_ranges():
    m = mg.Mesh.generate("cartesian_tri", 6, 6, 1.0, 1.0)
    t = teno_tables(m)
    r = np.random.default_rng(1)
    U = np.column_stack([1 + 0.1 * r.random(m.n_cells), r.random(m.n_cells), r.random(m.n_cells),
                         2 + r.random(m.n_cells)])
    X = mlp.features(U, t["offsets_stencils"], t["stencils"])
    assert X.shape == (m.n_cells, mlp.IN)
    x = X.reshape(m.n_cells, 4, mlp.PER_VAR)
    assert np.all(np.abs(x[:, :, :19]) <= 1.0)
    assert np.all(np.ptp(np.concatenate([x[:, :, :19], np.zeros((m.n_cells, 4, 1))], 2), axis=2) <= 1.0 + 1e-6)
    assert np.all((x[:, :, 19] >= -1) & (x[:, :, 19] <= 1))
    # a cell on the boundary has a missing directional stencil: marker -1
    off = t["offsets_stencils"]
    empty = np.array([[off[4 * c + s + 1] == off[4 * c + s] for s in range(1, 4)] for c in range(m.n_cells)])
    assert empty.any()
    np.testing.assert_array_equal(x[:, :, 20:23][np.repeat(empty[:, None, :], 4, 1)], -1.0)
    assert np.all(x[:, :, 23] == 0)
    # a uniform state gives zero differences and the "no range" marker
    X0 = mlp.features(np.ones((m.n_cells, 4)), t["offsets_stencils"], t["stencils"]).reshape(m.n_cells, 4, mlp.PER_VAR)
    assert np.all(X0[:, :, :19] == 0) and np.all(X0[:, :, 19] == -1)
    # ranges up to 1e-5 (round-off noise of the FP32 form, denormals) count as zero
    Ut = np.ones((m.n_cells, 4))
    Ut[:, 1] = 1e-40 * r.random(m.n_cells)
    Ut[:, 2] = 1.0 + 2e-6 * r.random(m.n_cells)
    Xt = mlp.features(Ut, t["offsets_stencils"], t["stencils"]).reshape(m.n_cells, 4, mlp.PER_VAR)
    assert np.isfinite(Xt).all() and np.all(Xt[:, 1:3, 19] == -1) and np.all(Xt[:, 1:3, :19] == 0)
    assert np.all(Xt[:, 1:3, 20:23] <= 0)
