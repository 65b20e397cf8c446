"""GPU tests of LOBPCG's Cholesky-QR callers of the path
(src/lobpcg/algorithm.rs:63-96): orthonormalize and apply_constraints.

The Gram matrix is summed on the device in fixed row chunks (the reference's
ndarray product has its own order), so L matches the restated path to
rounding; given L, the substitution is the reference's own order, so U is
bit-identical to the oracle's solve with the same L."""
import numpy as np
import pytest

from oracle import oracle as ora

pytestmark = pytest.mark.gpu


def test_orthonormalize_reference_case(gpu_lla):
    """The reference's test_orthonormalize (algorithm.rs:486-503): a random 10 x 10
    matrix times 10; U U^T = I and |R| of a QR equals |L^T| (there to 1e-2)."""
    lla = gpu_lla
    rng = np.random.default_rng(486)
    m = rng.random((10, 10)) * 10.0
    u, l = lla.orthonormalize(m)
    assert np.abs(u @ u.T - np.eye(10)).max() <= 1e-10
    r = np.linalg.qr(m)[1]
    assert np.abs(np.abs(r) - np.abs(l.T)).max() <= 1e-9 * np.abs(r).max()
    assert np.all(np.triu(l, 1) == 0)  # cholesky_into zeroes the upper part


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n,k", [(1, 1), (37, 5), (5000, 24), (20000, 64), (3000, 130)])
def test_orthonormalize_against_oracle(gpu_lla, dtype, n, k):
    lla = gpu_lla
    rng = np.random.default_rng(n + k)
    v = (rng.standard_normal((n, k)) * 10.0 ** rng.uniform(-1, 1, k)).astype(dtype)
    if n < k:
        pytest.skip("rank-deficient")
    u, l = lla.orthonormalize(v)
    eps = np.finfo(dtype).eps
    tol = 50 * k * eps
    # L L^T = V^T V to rounding of the Gram matrix
    g = v.astype(np.float64).T @ v.astype(np.float64)
    assert np.abs(l.astype(np.float64) @ l.T.astype(np.float64) - g).max() <= tol * np.abs(g).max()
    # given L, U is the reference's substitution bit for bit
    st, u_ora, _ = ora.orthonormalize(v)
    assert st["code"] == 0
    vt = np.array(v.T, order="C")
    assert ora.solve_triangular_inplace(np.array(l, order="C"), vt, "lower")["code"] == 0
    assert np.array_equal(u, vt.T)
    # orthonormal columns, U L^T = V
    assert np.abs(u.T.astype(np.float64) @ u.astype(np.float64) - np.eye(k)).max() <= 1e3 * k * eps
    back = u.astype(np.float64) @ l.T.astype(np.float64)
    assert np.abs(back - v).max() <= 1e2 * k * eps * np.abs(v).max()
    # and agrees with the restated path (numpy Gram) to rounding
    assert np.abs(u - u_ora).max() <= 1e3 * k * eps


def test_orthonormalize_strided_views_and_errors(gpu_lla):
    lla = gpu_lla
    rng = np.random.default_rng(7)
    big = rng.standard_normal((400, 30))
    v = big[::2, 3:20:2]  # strided, 200 x 9
    u, l = lla.orthonormalize(v)
    st, u_ora, l_ora = ora.orthonormalize(np.array(v))
    assert np.abs(u - u_ora).max() <= 1e-12
    assert np.abs(l - l_ora).max() <= 1e-12 * np.abs(l_ora).max()
    # a zero column makes V^T V singular: the Cholesky reports its row
    z = rng.standard_normal((50, 6))
    z[:, 3] = 0.0
    with pytest.raises(lla.NotPositiveDefinite) as exc:
        lla.orthonormalize(z)
    assert ora.orthonormalize(z)[0]["code"] == 2
    assert exc.value.index == ora.orthonormalize(z)[0]["index"]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_apply_constraints(gpu_lla, dtype):
    """V loses its component in span(Y): Y^T V_new = 0, and V_new matches the
    reference formula V - Y (L_yy^-1 (Y^T V)) with L_yy L_yy^T = Y^T Y."""
    lla = gpu_lla
    rng = np.random.default_rng(63)
    n, ky, k = 3000, 7, 11
    y = rng.standard_normal((n, ky)).astype(dtype)
    v = rng.standard_normal((n, k)).astype(dtype)
    lyy = np.array(y.T @ y, dtype=dtype)
    lla.cholesky_inplace(lyy)
    v0 = v.astype(np.float64)
    lla.apply_constraints(v, lyy, y)
    eps = np.finfo(dtype).eps
    yd, ld = y.astype(np.float64), lyy.astype(np.float64)
    u = np.linalg.solve(ld, yd.T @ v0)
    ref = v0 - yd @ u
    assert np.abs(v - ref).max() <= 1e3 * eps * np.abs(v0).max()
    # the constraint the reference establishes when lyy factors Y^T Y (Y orthogonal
    # after the LOBPCG normalisation): here, the projection residual of a full solve
    with pytest.raises(lla.WrongRows):
        lla.apply_constraints(v, np.eye(ky + 1, dtype=dtype), y)
