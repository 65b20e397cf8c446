"""Pins the CPU oracle to the reference before anything is compared with it.

1. Every known-answer test of the reference's SPD path (extracted verbatim
   into tests/golden/reference_kats.json) passes through the oracle with the
   reference's own assertion and tolerance.
2. The reference's property tests (tests/cholesky.rs:69-85,
   tests/triangular.rs:33-47) pass on seeded draws of the same strategies.
3. Results do not depend on the memory layout of the views (the restatement
   is index-based, like the reference).
4. Large-n cross-check against LAPACK (scipy): the oracle's factor and solve
   meet the normwise bounds ||LL^T - A||/||A|| <= 10 n eps and backward error
   <= 10 n eps.
"""
import numpy as np
import pytest

import cases
from oracle import oracle as ora

EPS64 = np.finfo(np.float64).eps


def arr(x, dtype="f64"):
    return np.array(x, dtype=np.float64 if dtype == "f64" else np.float32)


def test_build_flags():
    assert ora.build_info() == "ieee-ffp-contract-off"


def test_kat_decompose_and_f32():
    for name in ("decompose", "cholesky_f32"):
        c = cases.kat(name)
        a = arr(c["a"], c["dtype"])
        orig = a.copy()
        st = ora.cholesky_inplace(a)
        assert st == {"code": 0}
        np.testing.assert_allclose(a, arr(c["lower"], c["dtype"]), rtol=0, atol=c["eps"])
        np.testing.assert_allclose(a.astype(np.float64) @ a.T.astype(np.float64), orig,
                                   rtol=0, atol=c["eps"])
        # the factor of this KAT is exact in both precisions
        assert np.array_equal(a, arr(c["lower"], c["dtype"]))


def test_kat_errors():
    c = cases.kat("bad_matrix_not_square")
    a = arr(c["a"])
    assert ora.cholesky_inplace(a.copy()) == c["error"]
    assert ora.solvec_inplace(a.copy(), np.zeros(c["b_shape"])) == c["error"]
    for name in ("bad_matrix_non_pd",):
        c = cases.kat(name)
        a = arr(c["a"])
        assert ora.cholesky_inplace(a.copy())["code"] == 2
        assert ora.solvec_inplace(a.copy(), np.zeros(c["b_shape"]))["code"] == 2
    c = cases.kat("bad_matrix_zeros")
    assert ora.cholesky_inplace(arr(c["a"]))["code"] == 2


def test_kat_solvec():
    c = cases.kat("solvec")
    a, x = arr(c["a"]), arr(c["x"])
    b = a @ x
    st = ora.solvec_inplace(a.copy(), b)
    assert st["code"] == 0
    np.testing.assert_allclose(b, x, rtol=0, atol=c["eps"])


def test_kat_invc():
    c = cases.kat("invc")
    a = arr(c["a"])
    st, inv = ora.invc_inplace(a.copy())
    assert st["code"] == 0
    # assert_abs_diff_eq!(arr.dot(&inv), eye) with the default epsilon (f64::EPSILON)
    np.testing.assert_allclose(a @ inv, np.eye(3), rtol=0, atol=c["eps"])


def test_kat_corner_cases():
    e = np.zeros((0, 0))
    assert ora.cholesky_inplace(e)["code"] == 0
    st, inv = ora.invc_inplace(np.zeros((0, 0)))
    assert st["code"] == 0 and inv.shape == (0, 0)
    c = cases.kat("corner_cases_one")
    one = arr(c["a"])
    assert ora.cholesky_inplace(one)["code"] == 0 and one.tolist() == c["lower"]
    st, inv = ora.invc_inplace(arr(c["a"]))
    assert st["code"] == 0 and inv.tolist() == c["inv"]


def test_kat_triangular_masks():
    c = cases.kat("triangular_square")
    a = arr(c["a"])
    assert not ora.is_triangular(a, "lower") and not ora.is_triangular(a, "upper")
    up = a.copy()
    assert ora.triangular_inplace(up, "upper")["code"] == 0
    assert up.tolist() == c["upper"]
    assert ora.is_triangular(up, "upper") and not ora.is_triangular(up, "lower")
    lo = a.copy()
    assert ora.triangular_inplace(lo, "lower")["code"] == 0
    assert lo.tolist() == c["lower"]
    assert ora.is_triangular(lo, "lower") and not ora.is_triangular(lo, "upper")
    for name in ("triangular_non_square_row", "triangular_non_square_col"):
        c = cases.kat(name)
        a = arr(c["a"])
        assert not ora.is_triangular(a, "lower") and not ora.is_triangular(a, "upper")
        assert ora.triangular_inplace(a, c["uplo"]) == c["error"]
    e = np.zeros((0, 0))
    assert ora.is_triangular(e, "lower") and ora.is_triangular(e, "upper")


def test_kat_solve_triangular():
    for name in ("solve_triangular_lower", "solve_triangular_upper", "known_failure"):
        c = cases.kat(name)
        a, x = arr(c["a"]), arr(c["x"])
        assert ora.is_triangular(a, c["uplo"])
        b = a @ x
        assert ora.solve_triangular_inplace(a, b, c["uplo"])["code"] == 0
        np.testing.assert_allclose(b, x, rtol=0, atol=c["eps"])


def test_kat_solve_corners_and_errors():
    e = np.zeros((0, 0))
    assert ora.solve_triangular_inplace(e, e.copy(), "upper")["code"] == 0
    one = np.ones((1, 1))
    b = one.copy()
    assert ora.solve_triangular_inplace(one, b, "upper")["code"] == 0 and b[0, 0] == 1.0
    c = cases.kat("solve_corner_diag_zero")
    b = arr(c["b"])
    with np.errstate(all="ignore"):
        assert ora.solve_triangular_inplace(arr(c["a"]), b, c["uplo"])["code"] == 0
    for name in ("solve_error_not_square", "solve_error_wrong_rows"):
        c = cases.kat(name)
        assert ora.solve_triangular_inplace(arr(c["a"]), arr(c["b"]), c["uplo"]) == c["error"]


@pytest.mark.parametrize("seed", range(4))
def test_property_cholesky_solvec_invc(seed):
    """run_cholesky_test / run_solvec_test / run_invc_test (tests/cholesky.rs:21-67)."""
    rng = np.random.default_rng(1000 + seed)
    for _ in range(150):
        a = cases.hpd(rng)
        orig = np.array(a)
        chol = np.array(a)
        assert ora.cholesky_inplace(chol)["code"] == 0
        np.testing.assert_allclose(chol @ chol.T, orig, rtol=0, atol=1e-7 * max(1, np.abs(orig).max() / 1e4))
        assert ora.is_triangular(chol, "lower")
        dirty = np.array(orig)
        assert ora.cholesky_inplace_dirty(dirty)["code"] == 0
        assert np.array_equal(np.tril(dirty), chol)
        assert np.array_equal(np.triu(dirty, 1), np.triu(orig, 1))  # upper untouched
        x = cases.system(rng, a)
        b = orig @ x
        aa = np.array(orig)
        assert ora.solvec_inplace(aa, b)["code"] == 0
        np.testing.assert_allclose(b, x, rtol=0, atol=1e-5)
        assert np.array_equal(np.tril(aa), chol)  # solvec leaves the dirty factor
        st, inv = ora.invc_inplace(np.array(orig))
        assert st["code"] == 0
        np.testing.assert_allclose(orig @ inv, np.eye(orig.shape[0]), rtol=0, atol=1e-7)


@pytest.mark.parametrize("uplo", ["lower", "upper"])
def test_property_solve_triangular(uplo):
    """run_solve_triangular_test (tests/triangular.rs:22-31), 1e-4."""
    rng = np.random.default_rng(7 if uplo == "lower" else 8)
    for _ in range(300):
        a = cases.tri(rng, uplo)
        x = cases.system(rng, a)
        b = np.array(a) @ np.array(x)
        assert ora.solve_triangular_inplace(a, b, uplo)["code"] == 0
        np.testing.assert_allclose(b, x, rtol=0, atol=1e-4)


def test_layout_invariance_bitwise():
    """Same logical matrix in four memory layouts -> bit-identical factor and solve."""
    rng = np.random.default_rng(3)
    for n in (1, 2, 7, 33):
        m = cases.spd_gram(rng, n)
        bx = rng.standard_normal((n, 3))
        ref_a = m.copy()
        ref_b = bx.copy()
        assert ora.solvec_inplace(ref_a, ref_b)["code"] == 0
        for lay in range(4):
            store = np.array(m, order="F" if lay & 1 else "C")
            if lay & 2:
                store = np.array(store[::-1, ::-1], order="C")[::-1, ::-1]
            bb = np.array(bx, order="F" if lay & 1 else "C")
            assert ora.solvec_inplace(store, bb)["code"] == 0
            assert np.array_equal(np.tril(store), np.tril(ref_a))
            assert np.array_equal(bb, ref_b)


def test_not_positive_definite_state_matches_reference_semantics():
    """On failure at row j, rows < j are factored, row j's strict lower part is
    written and rows > j are untouched (src/cholesky.rs:54-74 returns early)."""
    rng = np.random.default_rng(5)
    n = 12
    a = cases.spd_gram(rng, n)
    a[7, 7] = -1.0
    orig = a.copy()
    st = ora.cholesky_inplace_dirty(a)
    assert st == {"code": 2, "index": 7}
    assert np.array_equal(a[8:], orig[8:])
    assert a[7, 7] == orig[7, 7]
    ref = orig.copy()
    ora.cholesky_inplace_dirty(ref[:7, :7])
    assert np.array_equal(np.tril(a[:7, :7]), np.tril(ref[:7, :7]))


def test_nan_does_not_error():
    """`d <= 0` is false for NaN: NaN input propagates without an error."""
    a = np.array([[np.nan, 0.0], [0.0, 1.0]])
    assert ora.cholesky_inplace(a)["code"] == 0
    assert np.isnan(a[0, 0])


@pytest.mark.parametrize("n", [64, 200, 400])
def test_against_lapack(n):
    sl = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(n)
    a = cases.spd_gram(rng, n)
    l = a.copy()
    assert ora.cholesky_inplace(l)["code"] == 0
    ref = sl.cholesky(a, lower=True)
    bound = 10 * n * EPS64
    assert np.linalg.norm(l @ l.T - a) / np.linalg.norm(a) <= bound
    assert np.linalg.norm(l - ref) / np.linalg.norm(ref) <= bound * 10
    b = rng.standard_normal((n, 4))
    x = b.copy()
    assert ora.solvec_inplace(a.copy(), x)["code"] == 0
    r = b - a @ x
    be = np.abs(r).max() / (np.abs(a).sum(1).max() * np.abs(x).max() + np.abs(b).max())
    assert be <= bound
