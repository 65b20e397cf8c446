"""Extract the reference's known-answer tests for the SPD path into JSON fixtures.

Reads the Rust test sources of linfa-linalg 0.2.1 (the reference tree, default
/root/reference, or the path given as argv[1]) as TEXT, pulls out the
`array![...]` literals of each known-answer test by their `let` names, and
writes tests/golden/reference_kats.json.  Nothing is executed from the
reference.  Re-run this script to regenerate the fixture; the committed JSON
is what the tests read (the reference tree is not available everywhere the
tests run).

Cases and their sources:
  cholesky.rs  decompose      src/cholesky.rs:208-216
  cholesky.rs  bad_matrix     src/cholesky.rs:218-245
  cholesky.rs  solvec         src/cholesky.rs:247-259
  cholesky.rs  invc           src/cholesky.rs:261-266
  cholesky.rs  corner_cases   src/cholesky.rs:268-277
  tests        cholesky_f32   tests/cholesky.rs:87-95
  triangular   square/masks   src/triangular.rs:198-246
  triangular   solve          src/triangular.rs:248-262
  triangular   solve corners  src/triangular.rs:264-277
  triangular   solve_error    src/triangular.rs:279-298
  tests        known_failure  tests/triangular.rs:49-180
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _read(ref, rel):
    with open(os.path.join(ref, rel)) as f:
        return f.read().split("\n")


def _literal(lines, first, last, name):
    """Return the `let <name> = array![...]` literal inside lines[first-1:last] (1-based)."""
    text = "\n".join(lines[first - 1:last])
    m = re.search(r"let\s+(?:mut\s+)?" + re.escape(name) + r"\s*=\s*array!\s*\[", text)
    if not m:
        raise KeyError(f"{name} not found in lines {first}-{last}")
    i = m.end() - 1
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "[":
            depth += 1
        elif text[j] == "]":
            depth -= 1
            if depth == 0:
                return _to_json(text[i:j + 1])
    raise ValueError("unbalanced literal")


def _literal_inline(lines, lineno, start_pat):
    """Array literal that follows `start_pat` on a single source line."""
    line = lines[lineno - 1]
    k = line.index(start_pat) + len(start_pat) - 1
    depth = 0
    for j in range(k, len(line)):
        if line[j] == "[":
            depth += 1
        elif line[j] == "]":
            depth -= 1
            if depth == 0:
                return _to_json(line[k:j + 1])
    raise ValueError("unbalanced literal")


def _to_json(lit):
    lit = re.sub(r"(\d)(f32|f64)", r"\1", lit)           # 25f32 -> 25
    lit = re.sub(r"(\d)\.(?!\d)", r"\1.0", lit)           # 25. -> 25.0
    lit = re.sub(r",(\s*)\]", r"\1]", lit)                # trailing commas
    return json.loads(lit)


def main(ref):
    chol = _read(ref, "src/cholesky.rs")
    tri = _read(ref, "src/triangular.rs")
    tchol = _read(ref, "tests/cholesky.rs")
    ttri = _read(ref, "tests/triangular.rs")
    cases = []

    arr = _literal(chol, 208, 216, "arr")
    cases.append({"name": "decompose", "source": "src/cholesky.rs:208-216", "kind": "cholesky",
                  "dtype": "f64", "a": arr, "lower": _literal(chol, 208, 216, "lower"),
                  "eps": 1e-7})
    cases.append({"name": "bad_matrix_not_square", "source": "src/cholesky.rs:220-228",
                  "kind": "error", "dtype": "f64", "a": _literal(chol, 218, 245, "row"),
                  "b_shape": [2, 3], "error": {"code": 1, "rows": 2, "cols": 3}})
    cases.append({"name": "bad_matrix_non_pd", "source": "src/cholesky.rs:230-238",
                  "kind": "error", "dtype": "f64", "a": _literal(chol, 218, 245, "non_pd"),
                  "b_shape": [2, 3], "error": {"code": 2}})
    cases.append({"name": "bad_matrix_zeros", "source": "src/cholesky.rs:240-244",
                  "kind": "error_cholesky_only", "dtype": "f64",
                  "a": _literal(chol, 218, 245, "zeros"), "error": {"code": 2}})
    cases.append({"name": "solvec", "source": "src/cholesky.rs:247-259", "kind": "solvec",
                  "dtype": "f64", "a": _literal(chol, 247, 259, "arr"),
                  "x": _literal(chol, 247, 259, "x"), "eps": 1e-7})
    # assert_abs_diff_eq! without epsilon uses f64::EPSILON (approx 0.5 default)
    cases.append({"name": "invc", "source": "src/cholesky.rs:261-266", "kind": "invc",
                  "dtype": "f64", "a": _literal(chol, 261, 266, "arr"),
                  "eps": 2.220446049250313e-16})
    cases.append({"name": "corner_cases_one", "source": "src/cholesky.rs:274-276",
                  "kind": "cholesky_exact", "dtype": "f64", "a": _literal(chol, 268, 277, "one"),
                  "lower": _literal(chol, 268, 277, "one"), "inv": _literal(chol, 268, 277, "one")})
    cases.append({"name": "corner_cases_empty", "source": "src/cholesky.rs:270-272",
                  "kind": "empty", "dtype": "f64"})
    cases.append({"name": "cholesky_f32", "source": "tests/cholesky.rs:87-95", "kind": "cholesky",
                  "dtype": "f32", "a": _literal(tchol, 87, 95, "arr"),
                  "lower": _literal(tchol, 87, 95, "lower"), "eps": 1e-7})

    sq = _literal(tri, 231, 246, "square")
    cases.append({"name": "triangular_square", "source": "src/triangular.rs:231-246",
                  "kind": "mask", "dtype": "f64", "a": sq,
                  "upper": _literal_inline(tri, 238, "array!["),
                  "lower": _literal_inline(tri, 245, "array![")})
    cases.append({"name": "triangular_non_square_row", "source": "src/triangular.rs:212-220",
                  "kind": "mask_error", "dtype": "f64", "a": _literal(tri, 212, 229, "row"),
                  "uplo": "lower", "error": {"code": 1, "rows": 2, "cols": 3}})
    cases.append({"name": "triangular_non_square_col", "source": "src/triangular.rs:222-228",
                  "kind": "mask_error", "dtype": "f64", "a": _literal(tri, 212, 229, "col"),
                  "uplo": "upper", "error": {"code": 1, "rows": 3, "cols": 2}})
    cases.append({"name": "solve_triangular_lower", "source": "src/triangular.rs:248-255",
                  "kind": "trsm", "dtype": "f64", "uplo": "lower",
                  "a": _literal(tri, 248, 262, "lower"), "x": _literal(tri, 248, 262, "expected"),
                  "eps": 1e-7})
    cases.append({"name": "solve_triangular_upper", "source": "src/triangular.rs:257-261",
                  "kind": "trsm", "dtype": "f64", "uplo": "upper",
                  "a": _literal(tri, 248, 262, "upper"), "x": _literal(tri, 248, 262, "expected"),
                  "eps": 1e-7})
    cases.append({"name": "solve_corner_diag_zero", "source": "src/triangular.rs:274-276",
                  "kind": "trsm_nocrash", "dtype": "f64", "uplo": "lower",
                  "a": _literal(tri, 264, 277, "diag_zero"), "b": [[0.0, 0.0], [0.0, 0.0]]})
    cases.append({"name": "solve_error_not_square", "source": "src/triangular.rs:281-287",
                  "kind": "trsm_error", "dtype": "f64", "uplo": "lower",
                  "a": _literal(tri, 279, 298, "non_square"),
                  "b": _literal(tri, 279, 298, "non_square"), "error": {"code": 1, "rows": 1, "cols": 2}})
    cases.append({"name": "solve_error_wrong_rows", "source": "src/triangular.rs:289-297",
                  "kind": "trsm_error", "dtype": "f64", "uplo": "upper",
                  "a": _literal(tri, 279, 298, "square"),
                  "b": _literal_inline(tri, 292, "&array!["),
                  "error": {"code": 3, "expected": 2, "actual": 1}})
    cases.append({"name": "known_failure", "source": "tests/triangular.rs:49-180",
                  "kind": "trsm", "dtype": "f64", "uplo": "upper",
                  "a": _literal(ttri, 49, 180, "a"), "x": _literal(ttri, 49, 180, "x"),
                  "eps": 1e-4})

    out = os.path.join(HERE, "reference_kats.json")
    with open(out, "w") as f:
        json.dump({"reference": "rust-ml/linfa-linalg 0.2.1",
                   "generator": "tests/golden/make_golden.py", "cases": cases}, f, indent=1)
    print(f"wrote {len(cases)} cases to {out}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
