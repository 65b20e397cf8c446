"""Failure detection without a GPU fault.

Every inter-CTA wait of the triangular solve is bounded.  These tests arm the
library's one-shot failure injection (lla_debug_inject_lost_handoff): the next
substitution launch loses its first block -- the block is never solved and
its flag never published, a flag that nothing sets -- and its waits give up
after a short poll limit.  The waiting blocks then record LLA_ERR_TIMEOUT and
return, the device stays usable, and the status reaches the caller:

* asynchronous device calls (lla_?trsm_device) through lla_device_status;
* the allocation-free solve through lla_dtrsm_device_noalloc_status
  (tests/test_zz_no_alloc.py);
* host-view calls (solve_triangular, solvec) directly in their return code.

The refined solve's FP64 fallback decides NotPositiveDefinite in the
reference's own operation order: its failing row equals the oracle's
(src/cholesky.rs:69-71) even for a borderline (singular) matrix.
"""
import numpy as np
import pytest

import cases
from oracle import oracle as ora

pytestmark = pytest.mark.gpu

TIMEOUT = 19


def lower_factor(torch, n, seed):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n))
    a = g @ g.T / n + np.eye(n)
    L = torch.linalg.cholesky(torch.tensor(a, device="cuda"))
    return L.T.contiguous().T, rng  # column-major


def residual_ok(L, X, B, trans):
    Lh = np.tril(L.cpu().numpy())
    T = Lh if trans == 0 else Lh.T
    x, b = X.cpu().numpy(), B.cpu().numpy()
    eps = np.finfo(np.float64).eps
    return np.abs(T @ x - b).max() <= 10 * T.shape[0] * eps * np.abs(T).sum(1).max() * np.abs(x).max()


@pytest.mark.parametrize("trans", [0, 1])
def test_device_trsm_reports_a_lost_handoff(gpu_lla, trans):
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    n, m = 2048, 16
    L, rng = lower_factor(torch, n, 11 + trans)
    B = torch.tensor(rng.standard_normal((n, m)), device="cuda").T.contiguous().T
    lla.device_status()  # nothing recorded before
    X = B.clone()
    lla.debug_inject_lost_handoff(2000)
    lla.trsm_device(L, X, trans)  # asynchronous: the launch itself succeeds
    with pytest.raises(lla.DeviceError) as e:
        lla.device_status()
    assert e.value.code == TIMEOUT
    lla.device_status()  # the record was cleared
    # the context is still usable and the next call is correct
    X = B.clone()
    lla.trsm_device(L, X, trans)
    lla.device_status()
    assert residual_ok(L, X, B, trans)


def test_host_view_solves_report_a_lost_handoff(gpu_lla):
    lla = gpu_lla
    rng = np.random.default_rng(3)
    n = 1500
    g = rng.standard_normal((n, n))
    a = g @ g.T / n + np.eye(n)
    l = np.linalg.cholesky(a)
    b = rng.standard_normal((n, 4))
    lla.debug_inject_lost_handoff(2000)
    with pytest.raises(lla.DeviceError) as e:
        lla.solve_triangular_inplace(l.copy(), b.copy(), lla.LOWER)
    assert e.value.code == TIMEOUT
    # solvec: the factor runs first, then the injected substitution times out
    lla.debug_inject_lost_handoff(2000)
    with pytest.raises(lla.DeviceError) as e:
        lla.solvec_inplace(a.copy(), b.copy())
    assert e.value.code == TIMEOUT
    x = lla.solve_triangular(l, b, lla.LOWER)
    assert np.abs(l @ x - b).max() <= 1e-10 * np.abs(b).max()


def test_refined_fallback_verdict_in_reference_order(gpu_lla):
    """A singular PSD matrix (rank n - 3): whether and where the reference fails
    depends on its rounding; the refined solve's fallback must agree with the
    oracle's exact-order verdict and failing row."""
    lla = gpu_lla
    rng = np.random.default_rng(21)
    for n in (120, 333):
        g = rng.standard_normal((n, n - 3))
        a = g @ g.T
        ref = a.copy()
        st = ora.cholesky_inplace_dirty(ref)
        x = np.ones((n, 2))
        try:
            rep = lla.posv_refined(a, x)
        except lla.NotPositiveDefinite as e:
            assert st["code"] == 2 and e.value.index == st["index"], (n, e.value.index, st)
        else:
            # success: either the low-precision path converged (no verdict was
            # needed), or the fallback factored it, as the reference does
            assert rep["fell_back"] == 0 or st["code"] == 0, (n, rep, st)
    # a clearly indefinite matrix fails at the same row as the oracle
    n = 257
    a = cases.spd_gram(rng, n)
    a[200, 200] = -5.0
    ref = a.copy()
    st = ora.cholesky_inplace_dirty(ref)
    assert st["code"] == 2
    with pytest.raises(lla.NotPositiveDefinite) as e:
        lla.posv_refined(a, np.ones((n, 1)))
    assert e.value.index == st["index"]
