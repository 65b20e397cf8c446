"""The allocation-free triangular solve, lla_dtrsm_device_noalloc.

It serves callers that must not allocate device memory (code running inside
another allocator's callback, hosts that own every device allocation, loops
where an allocation would synchronise the device).  Its scratch is a fixed
array inside the library, so this test checks, through the C ABI, that it
returns the same solutions as the allocating entry point lla_dtrsm_device --
bit for bit in exact order, within 10 n eps in fast mode -- on two calls in a
row (the second call starts from the scratch the first one left behind), and
that a problem beyond the array's limit is rejected before any device work.
This file is collected last so that a stop-at-first-failure run has already
run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOO_LARGE = 23


def _fn(lib, name):
    f = getattr(lib, name)
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_noalloc_trsm_matches_allocating_entry(gpu_lla):
    torch = pytest.importorskip("torch")
    lib = ctypes.CDLL(gpu_lla.LIB_PATH)
    ref_fn, noalloc_fn = _fn(lib, "lla_dtrsm_device"), _fn(lib, "lla_dtrsm_device_noalloc")
    rng = np.random.default_rng(404)
    n, m = 700, 13
    g = rng.standard_normal((n, n))
    a = g @ g.T / n + np.eye(n)
    L = torch.linalg.cholesky(torch.tensor(a, device="cuda"))
    Lc = L.T.contiguous().T  # column-major, ld = n
    B = torch.tensor(rng.standard_normal((n, m)), device="cuda").T.contiguous().T
    stream = torch.cuda.current_stream().cuda_stream
    eps = np.finfo(np.float64).eps
    for algo in (1, 2):  # exact order, then fast
        for trans in (0, 1):
            for call in range(2):  # two calls in a row
                X_ref, X_new = B.clone(), B.clone()
                assert ref_fn(Lc.data_ptr(), n, n, trans, X_ref.data_ptr(), m, n, algo,
                              stream, None) == 0
                assert noalloc_fn(Lc.data_ptr(), n, n, trans, X_new.data_ptr(), m, n, algo,
                                  stream, None) == 0
                torch.cuda.synchronize()
                xr, xn = X_ref.cpu().numpy(), X_new.cpu().numpy()
                if algo == 1:
                    assert np.array_equal(xr, xn), (trans, call)
                else:
                    assert np.abs(xr - xn).max() <= 10 * n * eps * np.abs(xr).max(), (trans, call)
                # and it solves the system
                Lnp = np.tril(L.cpu().numpy())
                T = Lnp if trans == 0 else Lnp.T
                r = T @ xn - B.cpu().numpy()
                assert np.abs(r).max() <= 10 * n * eps * (np.abs(T).sum(1).max() * np.abs(xn).max())


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_lla):
    torch = pytest.importorskip("torch")
    lib = ctypes.CDLL(gpu_lla.LIB_PATH)
    fn = _fn(lib, "lla_dtrsm_device_noalloc")
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    # 32 * 65537 rows -> 65537 row blocks > 65536 flags: rejected on the host, nothing launched
    n = 32 * 65537
    assert fn(dummy.data_ptr(), n, n, 0, dummy.data_ptr(), 1, n, 1, None, None) == TOO_LARGE
    assert fn(dummy.data_ptr(), 1024, 1024, 0, dummy.data_ptr(), 8 * 2049, 1024, 1, None,
              None) == TOO_LARGE


def test_noalloc_uses_every_flag(gpu_lla):
    """Exactly 65,536 flags (32 row blocks x 2,048 RHS chunks of 8): accepted,
    and the last flag, next to the array's status words, is used correctly."""
    torch = pytest.importorskip("torch")
    lib = ctypes.CDLL(gpu_lla.LIB_PATH)
    ref_fn, noalloc_fn = _fn(lib, "lla_dtrsm_device"), _fn(lib, "lla_dtrsm_device_noalloc")
    rng = np.random.default_rng(65536)
    n, m = 1024, 8 * 2048
    g = rng.standard_normal((n, n))
    L = torch.linalg.cholesky(torch.tensor(g @ g.T / n + np.eye(n), device="cuda"))
    Lc = L.T.contiguous().T
    B = torch.randn(m, n, dtype=torch.float64, device="cuda").T  # column-major, ld = n
    stream = torch.cuda.current_stream().cuda_stream
    X_ref, X_new = B.clone(), B.clone()
    assert ref_fn(Lc.data_ptr(), n, n, 0, X_ref.data_ptr(), m, n, 1, stream, None) == 0
    assert noalloc_fn(Lc.data_ptr(), n, n, 0, X_new.data_ptr(), m, n, 1, stream, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(X_ref, X_new)
    st = lib.lla_dtrsm_device_noalloc_status
    st.argtypes, st.restype = [ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int
    assert st(stream, None) == 0


def test_noalloc_reports_a_lost_handoff(gpu_lla):
    """A bounded wait that gives up (the injected lost hand-off: a flag that
    nothing sets) is reported by lla_dtrsm_device_noalloc_status, which also
    clears it; the next call is correct again."""
    torch = pytest.importorskip("torch")
    lib = ctypes.CDLL(gpu_lla.LIB_PATH)
    fn = _fn(lib, "lla_dtrsm_device_noalloc")
    st = lib.lla_dtrsm_device_noalloc_status
    st.argtypes, st.restype = [ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int
    rng = np.random.default_rng(19)
    n, m = 2048, 8
    g = rng.standard_normal((n, n))
    L = torch.linalg.cholesky(torch.tensor(g @ g.T / n + np.eye(n), device="cuda"))
    Lc = L.T.contiguous().T
    B = torch.tensor(rng.standard_normal((n, m)), device="cuda").T.contiguous().T
    stream = torch.cuda.current_stream().cuda_stream
    assert st(stream, None) == 0
    gpu_lla.debug_inject_lost_handoff(2000)
    X = B.clone()
    assert fn(Lc.data_ptr(), n, n, 0, X.data_ptr(), m, n, 2, stream, None) == 0
    assert st(stream, None) == 19  # LLA_ERR_TIMEOUT
    assert st(stream, None) == 0
    X = B.clone()
    assert fn(Lc.data_ptr(), n, n, 0, X.data_ptr(), m, n, 2, stream, None) == 0
    assert st(stream, None) == 0
    r = np.tril(L.cpu().numpy()) @ X.cpu().numpy() - B.cpu().numpy()
    assert np.abs(r).max() <= 1e-10 * np.abs(B.cpu().numpy()).max()
