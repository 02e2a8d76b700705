"""The reference's known-answer tests run on the GPU kernels (through the C ABI),
and checked bit-for-bit against the oracle."""

import numpy as np
import pytest

import mallard_gb300 as mg
from oracle import Oracle
from test_oracle_golden import _expected_flux, _riemann_inputs, riemann_cases

pytestmark = pytest.mark.gpu


def test_riemann_known_answers_gpu(golden):
    o = Oracle()
    for t in riemann_cases(golden):
        a = _riemann_inputs(t)
        F = mg.riemann_flux(t["riemann_solver"], **a)[0]
        for i, (val, tol) in _expected_flux(t).items():
            assert abs(F[i] - val) <= tol, (t["name"], i, F[i], val)
        np.testing.assert_array_equal(F, o.riemann_flux(t["riemann_solver"], **a), err_msg=t["name"])


@pytest.mark.parametrize("solver", ["Rusanov", "HLL", "HLLC"])
def test_riemann_random_states_bit_identical(solver):
    """Seeded random states covering every wave pattern, including the
    two-rarefaction and two-shock estimates (TRRS/TSRS branches)."""
    rng = np.random.default_rng(11)
    n = 4096
    ang = rng.uniform(0, 2 * np.pi, n)
    nrm = np.stack([np.cos(ang), np.sin(ang)], 1)
    rl, rr = rng.uniform(0.1, 2.0, n), rng.uniform(0.1, 2.0, n)
    pl, pr = 10 ** rng.uniform(-2, 1, n), 10 ** rng.uniform(-2, 1, n)
    ul, ur = rng.uniform(-2, 2, (n, 2)), rng.uniform(-2, 2, (n, 2))
    g = np.full(n, 1.4)
    hl = pl / ((g - 1) * rl) + pl / rl
    hr = pr / ((g - 1) * rr) + pr / rr
    F = mg.riemann_flux(solver, nrm, rl, ul, pl, g, hl, rr, ur, pr, g, hr)
    o = Oracle()
    ref = np.array([o.riemann_flux(solver, nrm[i], rl[i], ul[i], pl[i], g[i], hl[i], rr[i], ur[i], pr[i], g[i], hr[i])
                    for i in range(n)])
    exact = (F == ref).all(1).mean()
    # pow() in the two-rarefaction estimate (TRRS) may differ in its last bit
    # between the GPU and the host libm; every other branch is bit-identical.
    assert exact == 1.0 if solver == "Rusanov" else exact > 0.9, exact
    np.testing.assert_allclose(F, ref, rtol=1e-13, atol=1e-14)


def test_primitives_known_answer_gpu(golden):
    t = {x["name"]: x for x in golden["files"]["test/physics_test.cpp"]}["EulerPrimitivesFromConservatives"]
    s, v = t["scalars"], t["vectors"]
    R, _, cv = mg.gas_constants(s["gamma"], s["p_ref"], s["T_ref"], s["rho_ref"])
    u = v["u"]
    p, T = s["p"], s["T"]
    rho = p / (R * T)
    e = cv * T
    E = e + 0.5 * (u[0] * u[0] + u[1] * u[1])
    U = np.array([[rho, rho * u[0], rho * u[1], rho * E]] * 2)
    W = mg.primitives(U, s["gamma"], s["p_ref"], s["T_ref"], s["rho_ref"], s["p_min"], s["p_max"])
    for row in W:
        np.testing.assert_allclose(row, [u[0], u[1], p, T, e + p / rho], atol=golden["file_tolerances"]["test/physics_test.cpp"])
    np.testing.assert_array_equal(W, Oracle().primitives(U, s["gamma"], s["p_ref"], s["T_ref"], s["rho_ref"],
                                                          s["p_min"], s["p_max"]))


def test_primitives_random_bit_identical():
    rng = np.random.default_rng(3)
    n = 10000
    rho = rng.uniform(0.05, 3, n)
    U = np.stack([rho, rho * rng.uniform(-2, 2, n), rho * rng.uniform(-2, 2, n), rng.uniform(0.5, 10, n)], 1)
    for pmin in (-1e20, 1e-6):
        np.testing.assert_array_equal(mg.primitives(U, p_min=pmin), Oracle().primitives(U, 1.4, 101325.0, 298.15,
                                                                                        1.225, pmin, 1e20))


def test_fp64_probe_runs():
    g = mg.fp64_peak_gflops()
    assert g > 10.0


def test_integer_pipe_conversions():
    """f32_rn (FP64 -> FP32, nearest even, flush below FP32's normal range)
    and f64_of (FP32 -> FP64, exact) against numpy, over random magnitudes,
    rounding ties, subnormals, signed zeros, infinities and NaN."""
    import ctypes as C
    from mallard_gb300 import _native as N
    r = np.random.default_rng(11)
    x = np.concatenate([
        r.standard_normal(20000) * 10.0 ** r.uniform(-40, 40, 20000),
        r.uniform(-1, 1, 5000),
        # exact ties and neighbours of ties between two floats
        (np.float32(r.uniform(1, 2, 2000)).astype(np.float64) + np.float64(2.0 ** -24)),
        (np.float32(r.uniform(1, 2, 2000)).astype(np.float64) + np.float64(2.0 ** -24) * (1 + 2.0 ** -20)),
        [0.0, -0.0, np.inf, -np.inf, np.nan, 3.5e38, -3.5e38, 3.4028235677973366e38, 1.1754943508222875e-38,
         1.17549435e-38 * 0.5, 1e-300, -1e-300, 5e-324],
    ]).astype(np.float64)
    f = np.concatenate([
        r.standard_normal(20000).astype(np.float32) * np.float32(10.0) ** r.uniform(-37, 37, 20000).astype(np.float32),
        (r.integers(1, 1 << 23, 3000).astype(np.uint32)).view(np.float32),  # subnormals
        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.4e-45, -1.4e-45, 3.4028235e38], dtype=np.float32),
    ]).astype(np.float32)
    n = max(len(x), len(f))
    x = np.resize(x, n)
    f = np.resize(f, n)
    o32 = np.zeros(n, dtype=np.float32)
    o64 = np.zeros(n, dtype=np.float64)
    lib = N.lib()
    N.check(lib.mgpu_probe_conversions(0, N.ptr(x), N.ptr(o32), N.ptr(f), N.ptr(o64), C.c_uint64(n)))
    with np.errstate(over="ignore"):
        ref32 = x.astype(np.float32)
    tiny = np.abs(x) < np.float64(np.finfo(np.float32).tiny)
    ref32[tiny] = np.copysign(np.float32(0.0), x[tiny]).astype(np.float32)
    nan = np.isnan(x)
    assert np.isnan(o32[nan]).all()
    np.testing.assert_array_equal(o32[~nan].view(np.uint32), ref32[~nan].view(np.uint32))
    ref64 = f.astype(np.float64)
    fn = np.isnan(f)
    assert np.isnan(o64[fn]).all()
    np.testing.assert_array_equal(o64[~fn].view(np.uint64), ref64[~fn].view(np.uint64))
