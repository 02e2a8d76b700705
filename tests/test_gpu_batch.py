"""The batched form against independent single-case runs of the same FP32
form: every case of a batch over two meshes must follow its own solver
(same arithmetic per cell; rows only relabelled), with its own time step."""

import numpy as np
import pytest

import mallard_gb300 as mg
from mallard_gb300.batch import Batch
from cases import GAS, explosion, make_pair, pulse

pytestmark = pytest.mark.gpu

BCS = [{"name": z, "type": "symmetry"} for z in ("right", "top", "left", "bottom")]


def _cases():
    ma = mg.Mesh.generate("cartesian_tri", 12, 12, 1.0, 1.0)
    mb = mg.Mesh.generate("cartesian_tri", 20, 20, 1.0, 1.0)
    mb.permute_cells(9)
    r = np.random.default_rng(3)
    states = []
    for g, (m, n) in enumerate(((ma, 3), (mb, 2))):
        for k in range(n):
            if (g + k) % 2:
                U, W = explosion(m, center=r.uniform(0.35, 0.65, 2), radius=r.uniform(0.15, 0.3),
                                 inside=(r.uniform(0.8, 1.5), r.uniform(0.8, 1.5)), outside=(0.3, 0.3))
            else:
                U, W = pulse(m, amp=r.uniform(0.05, 0.3))
            states.append((g, k, U, W))
    return (ma, mb), states


def _single(m, U, W, steps):
    s, _ = make_pair(m, variant="corrected", precision="fp32",
                     bcs={z: "symmetry" for z in ("right", "top", "left", "bottom")})
    s.set_state(U, W)
    t = s.run(0.5, steps)
    Ug, _ = s.get_state()
    s.close()
    return Ug, t


def test_batch_primitives_after_steps():
    """The batch's steps carry no FP64 primitives: get_state recovers them
    for the case asked for, from the conserved state it returns; before any
    step it returns the ones set_state was given."""
    meshes, states = _cases()
    with Batch(meshes, [3, 2], boundaries=BCS, **GAS) as b:
        for g, k, U, W in states:
            b.set_state(g, k, U, W)
        np.testing.assert_array_equal(b.get_state(0, 1)[1], states[1][3])
        b.run(0.5, 5)
        b.synchronize()
        for g, k, _, _ in states:
            Ub, Wb = b.get_state(g, k)
            np.testing.assert_array_equal(Wb, mg.primitives(Ub, **GAS))


@pytest.mark.parametrize("shape", [0, 4, 5, 7, 8])
def test_batch_matches_single_case_runs(shape):
    """Every case of a batch over two meshes against its own single-case run
    (direct shape 0, staged shapes 4 and 5, resident-table shapes 7 and 8)."""
    meshes, states = _cases()
    steps = 25
    with Batch(meshes, [3, 2], boundaries=BCS, **GAS) as b:
        b.set_launch_shape(shape)
        assert b.n_cases == 5
        for g, k, U, W in states:
            b.set_state(g, k, U, W)
        # state round trip before stepping
        U0, _ = b.get_state(1, 1)
        np.testing.assert_array_equal(U0, states[4][2])
        b.run(0.5, steps)
        b.synchronize()
        flags, times = b.status()
        assert (flags == 0).all()
        worst, identical = 0.0, []
        for i, (g, k, U, W) in enumerate(states):
            Ub, _ = b.get_state(g, k)
            Us, ts = _single(meshes[g], U, W, steps)
            assert abs(times[i] - ts) <= 1e-12 * ts, (i, times[i], ts)
            err = np.abs(Ub - Us).max() / np.abs(Us).max()
            worst = max(worst, err)
            identical.append(np.mean(Ub == Us))
        print(f"batch vs single-case runs: max rel diff {worst:.2e}, bit-identical fraction "
              f"{min(identical):.3f}..{max(identical):.3f}")
        assert worst <= 1e-6


def test_batch_autotune_and_independent_time_steps():
    meshes, states = _cases()
    with Batch(meshes, [3, 2], boundaries=BCS, **GAS) as b:
        for g, k, U, W in states:
            b.set_state(g, k, U, W)
        sh, bps, ms = b.autotune()
        assert 0 <= sh < 9 and bps in (0, 2, 4, 8)
        assert np.all(ms[:4] > 0) and np.all(ms[4:, 0] > 0) and np.all(ms[4:, 1:] == 0)
        for g, k, U, W in states:
            b.set_state(g, k, U, W)
        b.run(0.5, 5)
        flags, times = b.status()
        assert (flags == 0).all()
        # cases with different states and meshes take different time steps
        assert len(np.unique(np.round(times, 12))) == len(times)


def test_batch_rejects_other_forms():
    m = mg.Mesh.generate("cartesian_tri", 8, 8, 1.0, 1.0)
    import ctypes as C
    from mallard_gb300 import _native as N
    cfg = N.Config()
    N.lib().mgpu_config_defaults(C.byref(cfg))
    v = m.view()
    arr = (C.POINTER(N.MeshView) * 1)(C.pointer(v))
    h = C.c_void_p()
    one = np.ones(1, dtype=np.uint32)
    rc = N.lib().mgpu_batch_create(1, C.cast(arr, C.c_void_p), N.ptr(one), C.byref(cfg), C.byref(h))
    assert rc == 6  # MGPU_ERR_UNSUPPORTED
