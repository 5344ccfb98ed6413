"""Regenerates ``reference_known_answers.json`` from the reference's own files.

Reads (as text, nothing is compiled or run):
  * examples/patch-solver/README.md:17-25   -- 5-point leaf solve errors, N = 8 ... 1024
  * test/test_matrix.cpp:155-192            -- dgesv known answers
  * test/test_matrix.cpp:270-300            -- blockPermute known answer
  * test/test_finite_volume_grid.cpp:30-49  -- cell-centre coordinates

Usage: python tests/golden/make_golden.py /path/to/reference-checkout
"""
import json
import re
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py /path/to/reference-checkout")
REF = Path(sys.argv[1])
OUT = Path(__file__).with_name("reference_known_answers.json")


def numbers(text):
    return [float(t) for t in re.findall(r"-?\d+(?:\.\d+)?(?:e[-+]?\d+)?", text)]


def block(text, start_pat, end_pat="});"):
    i = text.index(start_pat)
    j = text.index(end_pat, i)
    return text[i + len(start_pat):j]


def main():
    readme = (REF / "examples/patch-solver/README.md").read_text()
    errs = {}
    for m in re.finditer(r"N =\s*(\d+), Error = ([0-9.e+-]+)", readme):
        errs[int(m.group(1))] = float(m.group(2))
    order = float(re.search(r"Convergence Order = ([0-9.]+)", readme).group(1))

    tm = (REF / "test/test_matrix.cpp").read_text()
    ls = tm[tm.index("TEST(Matrix, linear_solve)"):]
    A = numbers(block(ls, "Matrix<double> A(3, 3, {"))
    b = numbers(block(ls, "Vector<double> b = {", "};"))
    x = numbers(block(ls, "Vector<double> x_expected = {", "};"))
    B = numbers(block(ls, "Matrix<double> B(3, 4, {"))
    X = numbers(block(ls, "Matrix<double> X_expected(3, 4, {"))

    bp = tm[tm.index("TEST(Matrix, block_permute)"):]
    m1 = numbers(block(bp, "Matrix<double> m1(4, 6, {"))
    pr = [int(v) for v in numbers(block(bp, "Vector<int> pi_rows = {", "};"))]
    pc = [int(v) for v in numbers(block(bp, "Vector<int> pi_cols = {", "};"))]
    R = [int(v) for v in numbers(block(bp, "Vector<int> R = {", "};"))]
    Cb = [int(v) for v in numbers(block(bp, "Vector<int> C = {", "};"))]
    m2 = numbers(block(bp, "Matrix<double> m2_expected(4, 6, {"))

    tg = (REF / "test/test_finite_volume_grid.cpp").read_text()
    pts = tg[tg.index("TEST(FiniteVolumeGrid, points)"):]
    xp = numbers(block(pts, "std::vector<double> expected_xpoints = {", "};"))
    yp = numbers(block(pts, "std::vector<double> expected_ypoints = {", "};"))

    data = {
        "source": "EllipticForest reference files (see make_golden.py)",
        "patch_solver_readme": {"domain": [-1, 1, -1, 1], "u": "sin(x)+sin(y)", "f": "-u",
                                "inf_errors": {str(k): v for k, v in sorted(errs.items())},
                                "order": order},
        "matrix_linear_solve": {"A": A, "b": b, "x": x, "B": B, "X": X, "tol_vec": 1e-15, "tol_mat": 1e-14},
        "matrix_block_permute": {"m1": m1, "shape": [4, 6], "pi_rows": pr, "pi_cols": pc, "R": R, "C": Cb,
                                 "expected": m2},
        "grid_points": {"nx": 4, "x": [0, 1], "ny": 4, "y": [1, 3], "xpoints": xp, "ypoints": yp, "tol": 1e-16},
    }
    OUT.write_text(json.dumps(data, indent=1) + "\n")
    print(OUT)


if __name__ == "__main__":
    main()
