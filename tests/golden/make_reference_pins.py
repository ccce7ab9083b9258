"""Extract the known-answer values of MAST's own unit tests into
reference_pins.json (the fixture tests/test_oracle_pins.py reads).

Reads, as text, from the MAST source tree whose root is the one required
argument (python make_reference_pins.py <mast-source-root>):
  tests/material/mast_isotropic_material.cpp        hand-computed C matrices
  tests/element/structural/2D/mast_structural_element_2d.h   default E, nu, h, k
  tests/element/structural/2D/quad4/
      mast_quad4_linear_structural_extension_internal_jacobian.cpp
                                                     element coords, the fixed
                                                     displacement vector and the
                                                     transform_element sections
  tests/test_helpers.cpp                             FD step of the 6th-order stencil
Only numbers are extracted; nothing of the reference is executed.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
if len(sys.argv) != 2:
    sys.exit("usage: python make_reference_pins.py <mast-source-root>")
REF = sys.argv[1]


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def test_case(src, name):
    i = src.index('TEST_CASE("%s"' % name)
    j = src.find("TEST_CASE(", i + 10)
    return src[i:j if j > 0 else len(src)]


def matrix_truth(block, var="K_mat_true", nth=0):
    """Collect `var(i,j) = <expr>;` assignments of the nth truth matrix in block."""
    starts = [m.start() for m in re.finditer(r"RealMatrixX %s = RealMatrixX::Zero\((\d+),(\d+)\)" % var, block)]
    s = starts[nth]
    e = starts[nth + 1] if nth + 1 < len(starts) else len(block)
    sub = block[s:e]
    dims = re.search(r"Zero\((\d+),(\d+)\)", sub)
    n, m = int(dims.group(1)), int(dims.group(2))
    M = [[0.0] * m for _ in range(n)]
    for line in sub.splitlines():
        lhs = re.findall(r"%s\((\d+),(\d+)\)" % var, line)
        if not lhs or "=" not in line:
            continue
        expr = line.split("=")[-1].strip().rstrip(";")
        expr = expr.replace("/2.", "/2.0")
        val = float(eval(expr, {"__builtins__": {}}))
        for (i, j) in lhs:
            M[int(i)][int(j)] = val
    return M


def main():
    mat = read("tests/material/mast_isotropic_material.cpp")
    c2 = test_case(mat, "constant_isotropic_structural_material_2d")
    c3 = test_case(mat, "constant_isotropic_structural_material_3d")
    pins = {
        "source": "MAST tests (read as text by tests/golden/make_reference_pins.py)",
        "material": {
            "E": float(re.search(r'Parameter E\("E_param", ([0-9.e+-]+)\)', c3).group(1)),
            "nu": float(re.search(r'Parameter nu\("nu_param", ([0-9.e+-]+)\)', c3).group(1)),
            "C3d_true": matrix_truth(c3),
            "C2d_plane_stress_true": matrix_truth(c2, nth=0),
            "C2d_plane_strain_true": matrix_truth(c2, nth=1),
            "where": {"3d": "tests/material/mast_isotropic_material.cpp:611-708",
                      "2d": "tests/material/mast_isotropic_material.cpp:272-445"},
        },
    }
    fix = read("tests/element/structural/2D/mast_structural_element_2d.h")
    getp = lambda nm: float(re.search(r"\b%s\(\"[A-Za-z_]+\",\s*([0-9.e+-]+)\)" % nm, fix).group(1))
    quad = read("tests/element/structural/2D/quad4/"
                "mast_quad4_linear_structural_extension_internal_jacobian.cpp")
    coords = re.search(r"coords <<([^;]*);", quad).group(1)
    coords = [float(x) for x in coords.replace("\n", " ").split(",")]
    sol = re.search(r"elem_sol <<([^;]*);", quad).group(1)
    sol = [float(x) for x in sol.replace("\n", " ").split(",")]
    sections = []
    for m in re.finditer(r'SECTION\("(.*?)"\)\s*\{(.*?)\n    \}', quad, flags=re.S):
        name, body = m.group(1).replace('\\"', ''), m.group(2)
        t = re.search(r"transform_element\(test_elem\.mesh,\s*coords,\s*([^;]*)\);", body)
        if not t:
            continue
        args = [float(x) for x in t.group(1).replace("\n", " ").split(",")]
        args += [0.0] * (10 - len(args))
        sections.append({"name": name, "args": args,
                         "expect_same_volume": "REQUIRE_FALSE" not in body.split("update_residual")[0]})
    helpers = read("tests/test_helpers.cpp")
    delta = float(re.search(r"Real delta = ([0-9.e+-]+);", helpers).group(1))
    pins["quad4_membrane"] = {
        "E": getp("E"), "nu": getp("nu"), "thickness": getp("thickness"), "k": getp(r"k"),
        "coords_3x4": coords, "elem_sol_24": sol, "fd_delta": delta,
        "margin_factor": 1.490116119384766e-08,
        "transforms": sections,
        "where": "tests/element/structural/2D/quad4/"
                 "mast_quad4_linear_structural_extension_internal_jacobian.cpp:45-367",
    }
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(pins, f, indent=1)
    print("wrote reference_pins.json with %d transform sections" % len(sections))


if __name__ == "__main__":
    main()
