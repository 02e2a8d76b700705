"""The CPU oracle against the reference's own known-answer tests.

Inputs and expected values come from tests/golden/reference_unit_vectors.json,
extracted from the reference's gtest sources by tests/golden/make_golden.py.
Tolerances are the reference tests' own (1e-6 absolute; exact where the
reference uses EXPECT_*_EQ).
"""

import numpy as np
import pytest

from oracle import Oracle


def _tests(golden, rel):
    return {t["name"]: t for t in golden["files"][rel]}


def _riemann_inputs(t):
    s, v = t["scalars"], t["vectors"]
    g = s["gamma"]
    rho_l, p_l, rho_r, p_r = s["rho_l"], s["p_l"], s["rho_r"], s["p_r"]
    # the test computes e and h from gamma (riemann_solver_test.cpp:33-36)
    e_r = p_r / ((g - 1.0) * rho_r)
    e_l = p_l / ((g - 1.0) * rho_l)
    h_l = e_l + p_l / rho_l
    h_r = e_r + p_r / rho_r
    return dict(n_unit=v["n_unit"], rho_l=rho_l, u_l=v["u_l"], p_l=p_l, gamma_l=g, h_l=h_l, rho_r=rho_r,
                u_r=v["u_r"], p_r=p_r, gamma_r=g, h_r=h_r)


def _expected_flux(t):
    out = {}
    for e in t["expects"]:
        lhs, val, tol = e["args"]
        idx = int(lhs.split("[")[1].rstrip("]"))
        out[idx] = (float(val), float(tol) if tol != "tol" else t["scalars"]["tol"])
    return out


def riemann_cases(golden):
    tests = golden["files"]["test/riemann_solver_test.cpp"]
    return [t for t in tests if t["riemann_solver"]]


def test_golden_fixture_shape(golden):
    names = {t["name"] for t in golden["files"]["test/riemann_solver_test.cpp"]}
    assert {"RusanovFlux", "RusanovFluxY", "RusanovFluxXY", "RusanovFluxZero", "HLLCFlux", "HLLCFluxY",
            "HLLCFluxXY", "HLLCFluxZero"} <= names
    assert len(golden["files"]["test/common_math_test.cpp"]) >= 40


def test_riemann_known_answers(golden):
    o = Oracle()
    cases = riemann_cases(golden)
    assert len(cases) == 8
    for t in cases:
        F = o.riemann_flux(t["riemann_solver"], **_riemann_inputs(t))
        for i, (val, tol) in _expected_flux(t).items():
            assert abs(F[i] - val) <= tol, (t["name"], i, F[i], val)


def test_physics_constants(golden):
    t = _tests(golden, "test/physics_test.cpp")["SetRCpCv"]
    s = t["scalars"]
    R, cp, cv = Oracle().gas_constants(s["gamma"], s["p_ref"], s["T_ref"], s["rho_ref"])
    tol = golden["file_tolerances"]["test/physics_test.cpp"]
    exp = {e["args"][0]: float(e["args"][1]) for e in t["expects"] if not e["args"][1].strip().isidentifier()}
    assert abs(R - exp["physics.get_h_R()"]) <= tol
    assert abs(cp - exp["physics.get_h_Cp()"]) <= tol
    assert abs(cv - exp["physics.get_h_Cv()"]) <= tol


def test_physics_primitives(golden):
    t = _tests(golden, "test/physics_test.cpp")["EulerPrimitivesFromConservatives"]
    s, v = t["scalars"], t["vectors"]
    o = Oracle()
    R, _, cv = o.gas_constants(s["gamma"], s["p_ref"], s["T_ref"], s["rho_ref"])
    u = v["u"]
    p, T = s["p"], s["T"]
    rho = p / (R * T)
    e = cv * T
    h = e + p / rho
    E = e + 0.5 * (u[0] * u[0] + u[1] * u[1])
    U = np.array([[rho, rho * u[0], rho * u[1], rho * E]] * 2)
    W = o.primitives(U, s["gamma"], s["p_ref"], s["T_ref"], s["rho_ref"], s["p_min"], s["p_max"])
    tol = golden["file_tolerances"]["test/physics_test.cpp"]
    for row in W:
        np.testing.assert_allclose(row, [u[0], u[1], p, T, h], atol=tol, rtol=0)


@pytest.mark.parametrize("name", ["FE", "RK4"])
def test_fe_rk4_consistency(golden, name):
    """time_integrator_test.cpp FE / RK4: a U-independent RHS advances U0 to 1.1 U0."""
    t = _tests(golden, "test/time_integrator_test.cpp")[name]
    assert t is not None
    n = golden["time_integrator_n_cells"]
    icpi = np.arange(n * 4, dtype=np.float64).reshape(n, 4)
    o = Oracle()
    U = (o.fe_const_rhs if name == "FE" else o.rk4_const_rhs)(icpi, icpi, 0.1)
    np.testing.assert_allclose(U, 1.1 * icpi, atol=golden["file_tolerances"]["test/time_integrator_test.cpp"])


def test_ssprk3_consistency(golden):
    """time_integrator_test.cpp SSPRK3: a U-independent RHS advances U0 to 1.1 U0."""
    t = _tests(golden, "test/time_integrator_test.cpp")["SSPRK3"]
    call = next(c for c in t["calls"] if c["fn"] == "integrator.take_step")
    dt = float(call["args"][0])
    n = golden["time_integrator_n_cells"]
    icpi = np.arange(n * 4, dtype=np.float64).reshape(n, 4)  # i_cell * 4 + i
    U = Oracle().ssprk3_const_rhs(icpi, icpi, dt)
    np.testing.assert_allclose(U, 1.1 * icpi, atol=golden["file_tolerances"]["test/time_integrator_test.cpp"])


@pytest.mark.parametrize("name", ["QRHouseholder3x3", "QRHouseholder3x4"])
def test_qr_known_answers(golden, name):
    t = _tests(golden, "test/common_math_test.cpp")[name]
    call = next(c for c in t["calls"] if c["fn"] == "QR_householder_noQ")
    m, n = int(call["args"][2]), int(call["args"][3])
    R = Oracle().qr_householder(t["vectors"]["A"], m, n)
    np.testing.assert_allclose(R, t["vectors"]["expected_R"], atol=t["scalars"]["tol"], rtol=0)


def _subst_cases(golden, fn):
    tests = golden["files"]["test/common_math_test.cpp"]
    return [t["name"] for t in tests if any(c["fn"] == fn for c in t["calls"])]


def test_substitutions_known_answers(golden):
    o = Oracle()
    tests = _tests(golden, "test/common_math_test.cpp")
    checked = 0
    for fn, kind in (("forward_substitution", "L"), ("back_substitution", "U")):
        for name in _subst_cases(golden, fn):
            t = tests[name]
            call = next(c for c in t["calls"] if c["fn"] == fn)
            a = call["args"]
            m, n, p = int(a[3]), int(a[4]), int(a[5])
            tL, tB = a[6] == "true", a[7] == "true"
            B = t["vectors"].get("B", t["vectors"].get("b"))
            f = o.forward_substitution if fn == "forward_substitution" else o.back_substitution
            X = f(t["vectors"][kind], B, m, n, p, tL, tB)
            exp = t["vectors"].get("expected_X", t["vectors"].get("expected_x"))
            np.testing.assert_allclose(X, exp, atol=t["scalars"]["tol"], rtol=0, err_msg=name)
            checked += 1
    assert checked == 10


def test_triangle_known_answers(golden):
    o = Oracle()
    tests = _tests(golden, "test/common_math_test.cpp")
    for name in ("TriangleArea2", "TriangleArea2NegativeCoordinates", "TriangleArea2ZeroArea"):
        t = tests[name]
        v = t["vectors"]
        assert o.triangle_area(v["v0"], v["v1"], v["v2"]) == t["scalars"]["expected_area"]
    # TriangleJJinvTranslate / Unit declare their vertices as std::vector
    for name, verts in (("TriangleJJinvTranslate", ([1.0, 1.0], [2.0, 1.0], [1.0, 2.0])),
                        ("TriangleJJinvUnit", ([0.0, 0.0], [1.0, 0.0], [0.0, 1.0]))):
        t = tests[name]
        v = t["vectors"]
        got = [v.get("v0"), v.get("v1"), v.get("v2")]
        verts = [g if g is not None else d for g, d in zip(got, verts)]
        J, Ji = o.triangle_jac(*verts)
        assert list(J) == v["expected_J"]
        assert list(Ji) == v["expected_J_inv"]
