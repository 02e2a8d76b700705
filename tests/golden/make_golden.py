"""Extract the reference's known-answer vectors into a JSON fixture.

Reads the reference's own gtest sources as text (nothing is compiled or run)
and records, for every TEST block of the files below, the literal inputs it
declares and the values it expects:

    test/riemann_solver_test.cpp    Rusanov / HLLC fluxes for Sod states
    test/physics_test.cpp           R, cp, cv and primitive recovery
    test/time_integrator_test.cpp   FE / RK4 / SSPRK3 with a constant RHS
    test/common_math_test.cpp       QR, substitutions, triangle J and area

Usage (in a container that has the reference checkout):

    python tests/golden/make_golden.py /path/to/Mallard  > tests/golden/reference_unit_vectors.json

The JSON is committed; the tests never read the reference tree.
"""

import json
import math
import re
import sys
from pathlib import Path

FILES = [
    "test/riemann_solver_test.cpp",
    "test/physics_test.cpp",
    "test/time_integrator_test.cpp",
    "test/common_math_test.cpp",
]

_TEST_RE = re.compile(r"^TEST\((\w+),\s*(\w+)\)\s*\{", re.M)


def _eval_number(expr):
    """Evaluate a C++ numeric literal expression (casts and sqrt allowed)."""
    e = expr.strip()
    e = re.sub(r"\(rtype\)", "", e)
    e = re.sub(r"static_cast<rtype>\(([^)]*)\)", r"(\1)", e)
    e = e.replace("Kokkos::sqrt", "sqrt").replace("std::sqrt", "sqrt")
    e = re.sub(r"(\d)[fF]\b", r"\1", e)
    if not re.fullmatch(r"[0-9eE+\-*/(). sqrt]*", e):
        raise ValueError(expr)
    return float(eval(e, {"__builtins__": {}}, {"sqrt": math.sqrt}))


def _split_top(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return out


def _blocks(text):
    starts = [(m.start(), m.group(1), m.group(2)) for m in _TEST_RE.finditer(text)]
    for i, (pos, suite, name) in enumerate(starts):
        end = starts[i + 1][0] if i + 1 < len(starts) else len(text)
        yield suite, name, text[pos:end]


def _parse_block(body):
    body = re.sub(r"//[^\n]*", "", body)
    scalars, vectors, expects, calls = {}, {}, [], []
    for m in re.finditer(r"(?:const\s+)?(?:rtype|double)\s+(\w+)\s*=\s*([^;]+);", body):
        try:
            scalars[m.group(1)] = _eval_number(m.group(2))
        except (ValueError, SyntaxError):
            scalars[m.group(1)] = m.group(2).strip()
    for m in re.finditer(r"(?:std::vector<rtype>|NVector)\s+(\w+)\s*=\s*\{([^}]*)\};", body, re.S):
        vals = [v for v in _split_top(m.group(2)) if v.strip()]
        vectors[m.group(1)] = [_eval_number(v) for v in vals]
    for m in re.finditer(r"(?:std::vector<rtype>)\s+(\w+)\((\d+)\);", body):
        vectors.setdefault(m.group(1), [0.0] * int(m.group(2)))
    for m in re.finditer(r"EXPECT_(NEAR|RTYPE_EQ|DOUBLE_EQ|EQ)\(([^;]*)\);", body):
        args = [a.strip() for a in _split_top(m.group(2))]
        expects.append({"kind": m.group(1), "args": args})
    for m in re.finditer(r"\b(\w+(?:\.\w+)?)\(([^;{}]*)\);", body):
        fn = m.group(1)
        if fn.startswith("EXPECT") or fn in ("for", "if"):
            continue
        calls.append({"fn": fn, "args": [a.strip() for a in _split_top(m.group(2))]})
    m = re.search(r"^\s*(Rusanov|HLLC|HLL)\s+riemann_solver;", body, re.M)
    solver = m.group(1) if m else None
    m = re.search(r"^\s*(FE|RK4|SSPRK3)\s+integrator;", body, re.M)
    integrator = m.group(1) if m else None
    return {
        "scalars": scalars,
        "vectors": vectors,
        "expects": expects,
        "calls": calls,
        "riemann_solver": solver,
        "integrator": integrator,
    }


def main(root):
    root = Path(root)
    out = {"source": "reference gtest sources, read as text", "files": {}}
    for rel in FILES:
        text = (root / rel).read_text()
        tests = []
        for suite, name, body in _blocks(text):
            rec = {"suite": suite, "name": name}
            rec.update(_parse_block(body))
            tests.append(rec)
        out["files"][rel] = tests
    # Constants the physics and integrator tests declare at file scope.
    tol = {}
    for rel in FILES:
        m = re.search(r"const\s+rtype\s+TOL\s*=\s*([^;]+);", (root / rel).read_text())
        if m:
            tol[rel] = _eval_number(m.group(1))
    out["file_tolerances"] = tol
    m = re.search(r"const\s+int\s+N_CELLS\s*=\s*(\d+);", (root / "test/time_integrator_test.cpp").read_text())
    out["time_integrator_n_cells"] = int(m.group(1)) if m else None
    json.dump(out, sys.stdout, indent=1, sort_keys=True)
    sys.stdout.write("\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout> > "
                 "tests/golden/reference_unit_vectors.json")
    main(sys.argv[1])
