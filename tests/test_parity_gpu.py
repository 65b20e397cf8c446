"""GPU parity: the CUDA library against the oracle, through the C ABI.

EXACT mode keeps the reference's operation order, so its results must be
bit-identical to the oracle's (factor, solution, inverse, failure index and
the partially-written matrix left by a failure).  FAST mode must meet the
tolerance the target states for the FP64 path: ||L L^T - A|| / ||A|| and the
normwise backward error each <= 10 n eps, and raise NotPositiveDefinite on
the same inputs.  f32 uses eps32.
"""
import numpy as np
import pytest

import cases
from oracle import oracle as ora

pytestmark = pytest.mark.gpu

EPS = {np.float64: np.finfo(np.float64).eps, np.float32: np.finfo(np.float32).eps}


@pytest.fixture
def exact(gpu_lla):
    prev = gpu_lla.set_algorithm(gpu_lla.ALGO_EXACT)
    yield gpu_lla
    gpu_lla.set_algorithm(prev)


@pytest.fixture
def fast(gpu_lla):
    prev = gpu_lla.set_algorithm(gpu_lla.ALGO_FAST)
    yield gpu_lla
    gpu_lla.set_algorithm(prev)


def same_bits(x, y):
    """Bitwise equality of two arrays' logical contents (any memory layout)."""
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    return x.shape == y.shape and x.dtype == y.dtype and \
        np.array_equal(x.view(np.uint8), y.view(np.uint8))


# ---- known-answer tests of the reference, through the GPU -------------------

def test_kats(exact):
    lla = exact
    for name in ("decompose", "cholesky_f32"):
        c = cases.kat(name)
        dt = np.float64 if c["dtype"] == "f64" else np.float32
        a = np.array(c["a"], dtype=dt)
        chol = lla.cholesky(a)
        assert np.array_equal(chol, np.array(c["lower"], dtype=dt))
    c = cases.kat("solvec")
    a, x = np.array(c["a"]), np.array(c["x"])
    out = lla.solvec(a.copy(), a @ x)
    np.testing.assert_allclose(out, x, rtol=0, atol=c["eps"])
    c = cases.kat("invc")
    a = np.array(c["a"])
    np.testing.assert_allclose(a @ lla.invc(a), np.eye(3), rtol=0, atol=c["eps"])
    one = np.array(cases.kat("corner_cases_one")["a"])
    assert lla.cholesky(one).tolist() == [[1.0]] and lla.invc(one).tolist() == [[1.0]]
    with pytest.raises(lla.NotPositiveDefinite):
        lla.cholesky(np.array(cases.kat("bad_matrix_non_pd")["a"]))
    with pytest.raises(lla.NotPositiveDefinite):
        lla.solvec(np.array(cases.kat("bad_matrix_non_pd")["a"]), np.zeros((2, 3)))
    with pytest.raises(lla.NotPositiveDefinite):
        lla.cholesky(np.array(cases.kat("bad_matrix_zeros")["a"]))
    for name in ("solve_triangular_lower", "solve_triangular_upper", "known_failure"):
        c = cases.kat(name)
        a, x = np.array(c["a"]), np.array(c["x"])
        out = lla.solve_triangular(a, a @ x, c["uplo"])
        np.testing.assert_allclose(out, x, rtol=0, atol=c["eps"])
        ref = a @ x
        ora.solve_triangular_inplace(a, ref, c["uplo"])
        assert same_bits(out, ref)
    c = cases.kat("solve_corner_diag_zero")
    with np.errstate(all="ignore"):
        out = lla.solve_triangular(np.array(c["a"]), np.array(c["b"]), c["uplo"])
        ref = np.array(c["b"])
        ora.solve_triangular_inplace(np.array(c["a"]), ref, c["uplo"])
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    c = cases.kat("triangular_square")
    sq = np.array(c["a"], dtype=np.float64)  # the reference's mask tests use integers
    assert lla.into_triangular(sq.copy(), "upper").tolist() == c["upper"]
    assert lla.into_triangular(sq.copy(), "lower").tolist() == c["lower"]
    assert not lla.is_triangular(sq, "upper") and not lla.is_triangular(sq, "lower")
    assert lla.is_triangular(np.array(c["upper"], dtype=np.float64), "upper")
    assert lla.is_triangular(np.array(c["lower"], dtype=np.float64), "lower")


# ---- property tests, bit-identical to the oracle ----------------------------

@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_cholesky_solvec_invc_bitwise(exact, dtype):
    """run_cholesky_test / run_solvec_test / run_invc_test strategies
    (tests/cholesky.rs:21-85) on strided views."""
    lla = exact
    rng = np.random.default_rng(11 if dtype == np.float64 else 12)
    for _ in range(60):
        a = cases.hpd(rng, dtype)
        for dirty in (True, False):
            g = cases.relayout(np.array(a), rng)
            r = np.array(a)
            st = ora.cholesky_inplace_dirty(r) if dirty else ora.cholesky_inplace(r)
            if st["code"] != 0:  # f32 inputs can be indefinite after rounding
                with pytest.raises(lla.NotPositiveDefinite):
                    (lla.cholesky_inplace_dirty if dirty else lla.cholesky_inplace)(g)
                assert same_bits(g, r)
                continue
            (lla.cholesky_inplace_dirty if dirty else lla.cholesky_inplace)(g)
            assert same_bits(g, r)
        x = cases.system(rng, a, dtype)
        b = (np.array(a, dtype=np.float64) @ np.array(x, dtype=np.float64)).astype(dtype)
        ag, bg = cases.relayout(np.array(a), rng), cases.relayout(b.copy(), rng)
        ar, br = np.array(a), b.copy()
        st = ora.solvec_inplace(ar, br)
        if st["code"] == 0:
            lla.solvec_inplace(ag, bg)
            assert same_bits(ag, ar) and same_bits(bg, br)
            inv_g = lla.invc(np.array(a))
            st, inv_r = ora.invc_inplace(np.array(a))
            assert st["code"] == 0 and same_bits(inv_g, inv_r)


@pytest.mark.parametrize("uplo", ["lower", "upper"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_solve_triangular_bitwise(exact, uplo, dtype):
    """run_solve_triangular_test strategy (tests/triangular.rs:9-47)."""
    lla = exact
    rng = np.random.default_rng(21 + (uplo == "upper") + 2 * (dtype == np.float32))
    for _ in range(80):
        a = cases.tri(rng, uplo, dtype)
        x = cases.system(rng, a, dtype)
        b = (np.array(a, np.float64) @ np.array(x, np.float64)).astype(dtype)
        bg, br = cases.relayout(b.copy(), rng), b.copy()
        lla.solve_triangular_inplace(a, bg, uplo)
        assert ora.solve_triangular_inplace(a, br, uplo)["code"] == 0
        assert same_bits(bg, br)
        if dtype == np.float64:
            np.testing.assert_allclose(bg, x, rtol=0, atol=1e-4)
        # custom diagonal (the diag_fn of solve_triangular_system)
        d = np.abs(np.diag(np.array(a))) + 0.5
        bg, br = b.copy(), b.copy()
        lla.solve_triangular_inplace(a, bg, uplo, diag=d)
        ora.solve_triangular_inplace(a, br, uplo, diag=d)
        assert same_bits(bg, br)


def test_masks_and_predicate(gpu_lla):
    lla = gpu_lla
    rng = np.random.default_rng(5)
    for _ in range(20):
        a = cases.square(rng)
        for uplo in ("lower", "upper"):
            g, r = cases.relayout(np.array(a), rng), np.array(a)
            lla.triangular_inplace(g, uplo)
            ora.triangular_inplace(r, uplo)
            assert same_bits(g, r)
            assert lla.is_triangular(g, uplo) and ora.is_triangular(r, uplo)
            other = "upper" if uplo == "lower" else "lower"
            assert lla.is_triangular(g, other) == ora.is_triangular(r, other)


def test_device_masks_and_predicate(gpu_lla):
    """triangular_inplace / is_triangular on device-resident column-major
    matrices (lla_?triangular_device, lla_?is_triangular_device) against the
    oracle: the same entries zeroed, the same verdicts, -0.0 counts as zero and
    NaN does not, a non-square matrix is NotSquare / not triangular."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(55)
    for it in range(12):
        n = int(rng.integers(1, 300)) if it else 1
        dt = np.float64 if it % 2 == 0 else np.float32
        a = rng.uniform(-100, 100, (n, n)).astype(dt)
        for uplo in ("lower", "upper"):
            g = torch.tensor(a, device="cuda").T.contiguous().T  # column-major
            r = a.copy()
            lla.triangular_device(g, uplo)
            ora.triangular_inplace(r, uplo)
            assert same_bits(g.cpu().numpy(), r)
            other = "upper" if uplo == "lower" else "lower"
            assert int(lla.is_triangular_device(g, uplo).item()) == int(ora.is_triangular(r, uplo)) == 1
            want = ora.is_triangular(r, other)
            assert int(lla.is_triangular_device(g, other).item()) == int(want)
    # -0.0 is zero, NaN is not
    z = np.tril(rng.standard_normal((40, 40)))
    z[3, 20] = -0.0
    assert int(lla.is_triangular_device(torch.tensor(z, device="cuda").T.contiguous().T, "lower").item()) == 1
    z[3, 20] = np.nan
    assert int(lla.is_triangular_device(torch.tensor(z, device="cuda").T.contiguous().T, "lower").item()) == 0
    assert ora.is_triangular(z, "lower") is False or ora.is_triangular(z, "lower") == 0
    # non-square: NotSquare for the mask, "not triangular" for the predicate
    ns = torch.zeros(5, 7, dtype=torch.float64, device="cuda").T.contiguous().T
    with pytest.raises(lla.NotSquare):
        lla.triangular_device(ns, "lower")
    assert int(lla.is_triangular_device(ns, "lower").item()) == 0


@pytest.mark.parametrize("n", [33, 64, 100, 257, 512, 1000])
def test_larger_n_bitwise(exact, n):
    """Multi-panel sizes (panels of 32, trailing tiles of 64, solve blocks of 32)."""
    lla = exact
    rng = np.random.default_rng(n)
    a = cases.spd_gram(rng, n)
    b = rng.standard_normal((n, 3))
    ag, bg, ar, br = a.copy(), b.copy(), a.copy(), b.copy()
    lla.solvec_inplace(ag, bg)
    assert ora.solvec_inplace(ar, br)["code"] == 0
    assert same_bits(ag, ar) and same_bits(bg, br)


def test_single_matrix_workload_n512(exact):
    """A = G G^T / 512 + I, one RHS; Cholesky, cholesky-solve, and
    solve_triangular lower and upper against the resulting L."""
    lla = exact
    rng = np.random.default_rng(2024)
    n = 512
    a = cases.spd_gram(rng, n)
    b = rng.standard_normal((n, 1))
    L = lla.cholesky(a)
    Lr = a.copy()
    ora.cholesky_inplace(Lr)
    assert same_bits(L, Lr)
    x = lla.solvec(a.copy(), b)
    xr = b.copy()
    ora.solvec_inplace(a.copy(), xr)
    assert same_bits(x, xr)
    for uplo, T in (("lower", L), ("upper", np.ascontiguousarray(L.T))):
        y = lla.solve_triangular(T, b, uplo)
        yr = b.copy()
        ora.solve_triangular_inplace(T, yr, uplo)
        assert same_bits(y, yr)
    r = b - a @ x
    assert np.abs(r).max() / (np.abs(a).sum(1).max() * np.abs(x).max()) <= 10 * n * EPS[np.float64]


@pytest.mark.parametrize("algo", ["exact", "fast"])
def test_not_positive_definite_same_row_and_state(gpu_lla, algo):
    """The failure is raised at the same row, and the view is left exactly as
    the reference leaves it (rows before the failing one factored)."""
    lla = gpu_lla
    prev = lla.set_algorithm(lla.ALGO_EXACT if algo == "exact" else lla.ALGO_FAST)
    try:
        rng = np.random.default_rng(9)
        for n, bad in ((12, 7), (100, 40), (300, 250), (700, 33)):
            a = cases.spd_gram(rng, n)
            a[bad, bad] = -abs(a[bad, bad])
            g, r = a.copy(), a.copy()
            with pytest.raises(lla.NotPositiveDefinite) as e:
                lla.cholesky_inplace(g)
            st = ora.cholesky_inplace(r)
            assert st == {"code": 2, "index": e.value.index}
            assert same_bits(g, r)
            # solvec: same error, b untouched
            g, bb = a.copy(), np.ones((n, 2))
            with pytest.raises(lla.NotPositiveDefinite):
                lla.solvec_inplace(g, bb)
            assert same_bits(g, r) and np.all(bb == 1.0)
        # rank-deficient PSD (borderline): the verdict matches the reference's
        g0 = rng.standard_normal((60, 59))
        a = g0 @ g0.T
        g, r = a.copy(), a.copy()
        st = ora.cholesky_inplace_dirty(r)
        if st["code"] == 0:
            lla.cholesky_inplace_dirty(g)
        else:
            with pytest.raises(lla.NotPositiveDefinite) as e:
                lla.cholesky_inplace_dirty(g)
            assert e.value.index == st["index"]
        assert same_bits(g, r)
    finally:
        lla.set_algorithm(prev)


def test_wrong_rows_after_factor(gpu_lla):
    """solvec factors `self` before checking b (src/cholesky.rs:140-141)."""
    lla = gpu_lla
    a = cases.spd_gram(np.random.default_rng(1), 5)
    g = a.copy()
    with pytest.raises(lla.WrongRows) as e:
        lla.solvec_inplace(g, np.zeros((4, 2)))
    assert (e.value.expected, e.value.actual) == (5, 4)
    r = a.copy()
    ora.cholesky_inplace_dirty(r)
    assert same_bits(g, r)


def test_nan_propagates_without_error(gpu_lla):
    lla = gpu_lla
    a = np.array([[np.nan, 0.0], [0.0, 1.0]])
    out = lla.cholesky(a)  # `d <= 0` is false for NaN (src/cholesky.rs:69)
    ref = a.copy()
    assert ora.cholesky_inplace(ref)["code"] == 0
    assert np.isnan(out[0, 0]) and np.isnan(out[1, 1])
    assert same_bits(np.isnan(out), np.isnan(ref))


# ---- FAST mode: tolerance of the FP64 path ----------------------------------

@pytest.mark.parametrize("n", [64, 300, 1024, 2100])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fast_within_tolerance(fast, n, dtype):
    lla = fast
    eps = EPS[dtype]
    rng = np.random.default_rng(100 + n)
    a64 = cases.spd_gram(rng, n)
    a = a64.astype(dtype)
    L = lla.cholesky(a).astype(np.float64)
    a_d = a.astype(np.float64)
    assert np.linalg.norm(L @ L.T - a_d) / np.linalg.norm(a_d) <= 10 * n * eps
    b = rng.standard_normal((n, 4)).astype(dtype)
    x = lla.solvec(a.copy(), b).astype(np.float64)
    r = b.astype(np.float64) - a_d @ x
    be = np.abs(r).max() / (np.abs(a_d).sum(1).max() * np.abs(x).max() + np.abs(b).max())
    assert be <= 10 * n * eps
    if n <= 1024:
        lr = a.copy()
        ora.cholesky_inplace(lr)
        assert np.abs(L - lr).max() <= 10 * n * eps * np.abs(lr).max() * 10


@pytest.mark.parametrize("n", [300, 1100, 2500])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fast_invc_potri_panels(fast, n, dtype):
    """FAST-mode InverseC: column panels of L^-1 solved only below their first
    row, the upper part mirrored (symmetric by construction); accuracy of the
    FP64 path: ||A inv - I|| within kappa * n * eps."""
    lla = fast
    eps = EPS[dtype]
    rng = np.random.default_rng(200 + n)
    a = cases.spd_gram(rng, n).astype(dtype)
    inv = lla.invc(a.copy())
    assert np.array_equal(inv, inv.T)
    a_d, inv_d = a.astype(np.float64), inv.astype(np.float64)
    kappa = np.linalg.cond(a_d)
    resid = np.abs(a_d @ inv_d - np.eye(n)).max()
    assert resid <= 10 * n * eps * kappa, (resid, kappa)
    ref = np.linalg.inv(a_d)
    assert np.abs(inv_d - ref).max() <= 10 * n * eps * kappa * np.abs(ref).max()


def test_device_api_matches_host_api(gpu_lla):
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(77)
    n, m = 300, 5
    a = cases.spd_gram(rng, n)
    b = rng.standard_normal((n, m))
    A = torch.tensor(a, device="cuda").T.contiguous().T  # column-major
    info = lla.potrf_device(A, algo=lla.ALGO_EXACT)
    B = torch.tensor(b, device="cuda").T.contiguous().T
    lla.trsm_device(A, B, trans=0, algo=lla.ALGO_EXACT)
    lla.trsm_device(A, B, trans=1, algo=lla.ALGO_EXACT)
    torch.cuda.synchronize()
    assert int(info.item()) == -1
    ar, br = a.copy(), b.copy()
    ora.solvec_inplace(ar, br)
    assert same_bits(np.tril(A.cpu().numpy()), np.tril(ar))
    assert same_bits(B.cpu().numpy(), br)
    # FAST device path: tolerance
    A2 = torch.tensor(a, device="cuda").T.contiguous().T
    info = lla.potrf_device(A2, algo=lla.ALGO_FAST)
    torch.cuda.synchronize()
    L = np.tril(A2.cpu().numpy())
    assert int(info.item()) == -1
    assert np.linalg.norm(L @ L.T - a) / np.linalg.norm(a) <= 10 * n * EPS[np.float64]
