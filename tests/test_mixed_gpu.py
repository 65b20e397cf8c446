"""GPU tests of the mixed-precision refined solve (low-precision Cholesky of
the equilibrated matrix + FP64 refinement + plain FP64 fallback).

Every converged result must reach the target normwise backward error
(1e-13 by default) measured here independently in FP64, and agree with the
plain FP64 solution to the forward error the conditioning allows.  Failures
are decided by the FP64 path: a non-SPD input raises NotPositiveDefinite.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

UPDATES = ["fp32", "fp16x3", "bf16x6", "bf16x3"]


def qdq(rng, n, kappa, diag_scale=0.0):
    """A = D Q diag(s) Q^T D, Q from QR of a Gaussian, s log-uniform in [1, kappa],
    D = diag(10^U(-diag_scale, diag_scale))."""
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.exp(rng.uniform(0, np.log(kappa), n))
    s[0], s[-1] = 1.0, kappa
    a = (q * s) @ q.T
    a = (a + a.T) / 2
    if diag_scale:
        d = 10.0 ** rng.uniform(-diag_scale, diag_scale, n)
        a = a * d[:, None] * d[None, :]
    return a


def backward_error(a, x, b):
    r = b - a @ x
    return (np.abs(r).max(0) / (np.abs(a).sum(1).max() * np.abs(x).max(0) + np.abs(b).max(0))).max()


@pytest.mark.parametrize("update", UPDATES)
@pytest.mark.parametrize("n,kappa", [(100, 1e2), (512, 1e6), (1000, 1e4), (1537, 1e6)])
def test_refined_reaches_fp64_accuracy(gpu_lla, update, n, kappa):
    lla = gpu_lla
    rng = np.random.default_rng(n)
    a = qdq(rng, n, kappa)
    b = rng.standard_normal((n, 7))
    x = b.copy()
    rep = lla.posv_refined(a, x, update=update)
    assert rep["converged"] == 1 and rep["fell_back"] == 0, rep
    assert rep["backward_error"] <= 1e-13
    be = backward_error(a, x, b)
    assert be <= 2e-13, be
    xr = np.linalg.solve(a, b)
    fe = np.abs(x - xr).max() / np.abs(xr).max()
    assert fe <= 10 * kappa * max(rep["backward_error"], 1e-15), fe  # forward <~ kappa * backward


@pytest.mark.parametrize("n,m", [(777, 1), (777, 20), (777, 64), (777, 97), (2111, 37), (4160, 64)])
def test_refined_many_right_hand_sides(gpu_lla, n, m):
    """Several 16-column chunks in the FP32 substitutions, ragged n; n >= 1024
    (16 block rows) brings in the helper items that sum the first half of a late
    block row's coupling terms."""
    lla = gpu_lla
    rng = np.random.default_rng(m + n)
    a = qdq(rng, n, 1e5)
    b = rng.standard_normal((n, m))
    x = b.copy()
    rep = lla.posv_refined(a, x, update="bf16x6")
    assert rep["converged"] == 1 and rep["fell_back"] == 0, rep
    assert backward_error(a, x, b) <= 2e-13


def test_equilibration_handles_badly_scaled_diagonal(gpu_lla):
    lla = gpu_lla
    rng = np.random.default_rng(3)
    n = 700
    a = qdq(rng, n, 1e4, diag_scale=3.0)
    b = rng.standard_normal((n, 4))
    x = b.copy()
    rep = lla.posv_refined(a, x)
    assert rep["backward_error"] <= 1e-13
    assert backward_error(a, x, b) <= 2e-13


def test_strided_views_and_lower_triangle_only(gpu_lla):
    """Only the lower triangle is read (as in the reference's solvec)."""
    lla = gpu_lla
    rng = np.random.default_rng(4)
    n = 300
    a = cases.spd_gram(rng, n)
    garbage = a.copy()
    garbage[np.triu_indices(n, 1)] = 1e9
    b = rng.standard_normal((n, 3))
    x = cases.relayout(b.copy(), rng)
    lla.posv_refined(cases.relayout(garbage, rng), x)
    assert backward_error(a, x, b) <= 2e-13


def test_not_positive_definite_decided_by_fp64_path(gpu_lla):
    lla = gpu_lla
    rng = np.random.default_rng(6)
    n = 200
    a = cases.spd_gram(rng, n)
    a[50, 50] = -1.0
    with pytest.raises(lla.NotPositiveDefinite) as e:
        lla.posv_refined(a, np.ones((n, 2)))
    assert e.value.index == 50


def test_ill_conditioned_falls_back_or_converges(gpu_lla):
    lla = gpu_lla
    rng = np.random.default_rng(8)
    n = 400
    a = qdq(rng, n, 1e12)
    b = rng.standard_normal((n, 2))
    x = b.copy()
    rep = lla.posv_refined(a, x)
    assert rep["converged"] == 1 or rep["fell_back"] == 1
    assert backward_error(a, x, b) <= 1e-13
    x2 = b.copy()
    with pytest.raises(lla.DeviceError) as e:
        lla.posv_refined(a, x2, fallback=False, max_iters=2)
    assert e.value.code == lla.ERR_NOT_CONVERGED


def test_device_form_matches_host_form(gpu_lla):
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(10)
    n, m = 640, 5
    a = qdq(rng, n, 1e5)
    b = rng.standard_normal((n, m))
    A = torch.tensor(a, device="cuda").T.contiguous().T
    B = torch.tensor(b, device="cuda").T.contiguous().T
    X = torch.empty_like(B.T.contiguous()).T
    rep = lla.posv_refined_device(A, B, X)
    x = b.copy()
    rep2 = lla.posv_refined(a, x)
    assert rep["iterations"] == rep2["iterations"]
    assert np.array_equal(X.cpu().numpy(), x)


@pytest.mark.parametrize("order", ["C", "F"])
def test_pinned_host_input_read_in_place(gpu_lla, order):
    """A in page-locked host memory is read in place by the import kernel (no
    staging copy); the result is bit-identical to the pageable-memory path."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(12)
    n, m = 700, 3
    a = qdq(rng, n, 1e4)
    b = rng.standard_normal((n, m))
    ap = torch.empty((n, n), dtype=torch.float64, pin_memory=True).numpy()
    if order == "F":
        ap = ap.T  # a column-major view of the pinned buffer
    ap[...] = a
    x1, x2 = b.copy(), b.copy()
    r1 = lla.posv_refined(ap, x1)
    r2 = lla.posv_refined(np.array(a, order=order), x2)
    assert r1["converged"] == 1 and r1["iterations"] == r2["iterations"]
    assert np.array_equal(x1, x2)
    assert np.array_equal(ap, a)  # A is only read


# accuracy of the low-precision factorisation alone: ||L L^T - A|| / ||A||
# bounds per update form (FP32 panels; the split forms are FP32-accurate)
FACTOR_TOL = {"fp32": 2e-6, "fp16x3": 4e-6, "bf16x6": 4e-6, "bf16x3": 3e-5, "fp16": 3e-3,
              "bf16": 3e-2}


@pytest.mark.parametrize("update", list(FACTOR_TOL))
@pytest.mark.parametrize("n", [128, 200, 385, 1024])
def test_lowp_factor_accuracy(gpu_lla, update, n):
    """Checks the tensor-core trailing update (and the FP32 diagonal/panel
    kernels) directly: partial tiles, several panels, every term form."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(1000 + n)
    a = cases.spd_gram(rng, n)
    d = 1.0 / np.sqrt(np.diag(a))
    a = a * d[:, None] * d[None, :]  # unit diagonal, as after equilibration
    A = torch.tensor(a, dtype=torch.float32, device="cuda").T.contiguous().T
    info = lla.spotrf_mixed_device(A, update=update)
    torch.cuda.synchronize()
    assert int(info.item()) == -1
    L = np.tril(A.cpu().numpy().astype(np.float64))
    rel = np.linalg.norm(L @ L.T - a) / np.linalg.norm(a)
    assert rel <= FACTOR_TOL[update], rel


@pytest.mark.parametrize("n,m", [(200, 3), (1000, 64), (4099, 17)])
def test_exact_slice_residual_matches_fp64(gpu_lla, n, m):
    """The tensor-core exact-slice residual against an extended-precision
    reference: both it and the FP64 residual must be within ~FP64 rounding of
    the exact B - A X (relative to |A| |x|, the scale of the cancellation)."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(n)
    a = qdq(rng, n, 1e6) * 10.0 ** rng.uniform(-3, 3)
    x = rng.standard_normal((n, m)) * 10.0 ** rng.uniform(-2, 2, m)
    b = a @ x + 1e-9 * rng.standard_normal((n, m))  # residual ~1e-9: heavy cancellation
    A = torch.tensor(a, device="cuda").T.contiguous().T
    X = torch.tensor(x, device="cuda").T.contiguous().T
    B = torch.tensor(b, device="cuda").T.contiguous().T
    R1 = torch.empty_like(B.T.contiguous()).T
    R2 = torch.empty_like(B.T.contiguous()).T
    lla.residual_device(A, X, B, R1, "fp64")
    lla.residual_device(A, X, B, R2, "slices")
    torch.cuda.synchronize()
    # extended-precision reference with numpy longdouble where available
    ref = (b.astype(np.longdouble) - a.astype(np.longdouble) @ x.astype(np.longdouble)).astype(np.float64)
    scale = (np.abs(a) @ np.abs(x))
    e1 = (np.abs(R1.cpu().numpy() - ref) / scale).max()
    e2 = (np.abs(R2.cpu().numpy() - ref) / scale).max()
    assert e1 <= 1e-14, e1
    assert e2 <= 1e-14, e2


def test_refined_with_exact_slice_residual(gpu_lla):
    lla = gpu_lla
    rng = np.random.default_rng(31)
    n = 1500
    a = qdq(rng, n, 1e6)
    b = rng.standard_normal((n, 8))
    x1, x2 = b.copy(), b.copy()
    r1 = lla.posv_refined(a, x1)
    r2 = lla.posv_refined(a, x2, residual="slices")
    assert r2["converged"] == 1 and r2["fell_back"] == 0
    assert backward_error(a, x2, b) <= 2e-13
    assert abs(r1["iterations"] - r2["iterations"]) <= 1


def device_qdq(torch, n, kappa, seed, diag_scale=0.0):
    """A = D Q diag(s) Q^T D built on the device in FP64 (Q from the QR of a
    seeded Gaussian, s log-uniform in [1, kappa], D = diag(10^U(-d, d)))."""
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    G = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    Q, _ = torch.linalg.qr(G)
    del G
    s = torch.exp(torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * np.log(kappa))
    s[0], s[-1] = 1.0, kappa
    A = (Q * s) @ Q.T
    del Q
    A = (A + A.T) * 0.5
    if diag_scale:
        d = 10.0 ** ((torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1) * diag_scale)
        A = A * d[:, None] * d[None, :]
    B = torch.randn(n, 64, dtype=torch.float64, device="cuda", generator=g)
    return A, B


def device_backward_error(torch, A, X, B):
    R = B - A @ X
    return float((R.abs().amax(0) / (A.abs().sum(1).amax() * X.abs().amax(0) + B.abs().amax(0))).max())


@pytest.mark.parametrize("residual", ["slices", "fp64"])
def test_precision_sweep_size_kappa_1e8_diag_scaled(gpu_lla, residual):
    """The precision-sweep configuration at its own size: n = 8192, 16 RHS,
    kappa = 1e8, diagonal scaled by 10^U(-3, 3); the bf16x6 form must reach the
    1e-13 backward error without falling back (equilibration removes D)."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    n, m = 8192, 16
    A, B = device_qdq(torch, n, 1e8, 8192, diag_scale=3.0)
    B = B[:, :m].T.contiguous().T
    X = torch.empty_like(B.T.contiguous()).T
    rep = lla.posv_refined_device(A.T, B, X, update="bf16x6", residual=residual)
    torch.cuda.synchronize()
    assert rep["converged"] == 1 and rep["fell_back"] == 0, rep
    be = device_backward_error(torch, A, X, B)
    assert be <= 1e-13, (be, rep)


def test_headline_size_n16384_kappa_1e6(gpu_lla):
    """The headline configuration under the test suite: n = 16384, 64 RHS,
    kappa = 1e6, bf16x6 updates with the exact-slice residual, checked by an
    independent FP64 product; and it agrees with the plain FP64 path's solution
    to the forward error the conditioning allows."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    n = 16384
    A, B = device_qdq(torch, n, 1e6, 16384)
    B = B.T.contiguous().T
    X = torch.empty_like(B.T.contiguous()).T
    rep = lla.posv_refined_device(A.T, B, X, update="bf16x6", residual="slices")
    torch.cuda.synchronize()
    assert rep["converged"] == 1 and rep["fell_back"] == 0, rep
    be = device_backward_error(torch, A, X, B)
    assert be <= 1e-13, (be, rep)
    W = A.clone()
    info = lla.potrf_device(W.T, algo=lla.ALGO_FAST)
    Xp = B.clone()
    lla.trsm_device(W.T, Xp, 0)
    lla.trsm_device(W.T, Xp, 1)
    lla.device_status()
    assert int(info.item()) == -1
    fe = float((X - Xp).abs().max() / Xp.abs().max())
    assert fe <= 1e6 * 1e-13 * 10, fe


@pytest.mark.parametrize("update", ["bf16x6", "bf16x3", "fp16x3"])
@pytest.mark.parametrize("kchunk,epilogue", [(64, 1), (32, 1), (32, 2)])
def test_update_kchunk_forms(gpu_lla, update, kchunk, epilogue):
    """The tensor-core update with 64-wide K-chunks (128-byte swizzle) and with
    32-wide K-chunks (64-byte swizzle, twice the stages), with the register
    epilogue (1) and the TMA-staged one (2): all converge to the FP64 target."""
    lla = gpu_lla
    rng = np.random.default_rng(3 + kchunk + epilogue)
    n = 1537
    a = qdq(rng, n, 1e6)
    b = rng.standard_normal((n, 9))
    x = b.copy()
    rep = lla.posv_refined(a, x, update=update, update_kchunk=kchunk, update_epilogue=epilogue)
    assert rep["converged"] == 1 and rep["fell_back"] == 0, rep
    assert backward_error(a, x, b) <= 2e-13


@pytest.mark.parametrize("n", [300, 1030])
def test_lowp_factor_leaves_upper_triangle(gpu_lla, n):
    """The in-place low-precision factorisation writes the lower triangle only:
    the TMA-staged epilogue (leading dimension a multiple of 4: n = 300) stores
    whole tiles and must write the upper part of diagonal tiles back unchanged;
    the register epilogue (n = 1030) never touches it."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(n)
    a = cases.spd_gram(rng, n)
    d = 1.0 / np.sqrt(np.diag(a))
    a = (a * d[:, None] * d[None, :]).astype(np.float32)
    junk = rng.standard_normal((n, n)).astype(np.float32)
    a_in = np.tril(a) + np.triu(junk, 1)
    A = torch.tensor(a_in, device="cuda").T.contiguous().T
    info = lla.spotrf_mixed_device(A, update="fp16x3")  # a two-term form: TMA-staged when n % 4 == 0
    torch.cuda.synchronize()
    assert int(info.item()) == -1
    out = A.cpu().numpy()
    assert np.array_equal(np.triu(out, 1), np.triu(junk, 1))
    L = np.tril(out.astype(np.float64))
    assert np.linalg.norm(L @ L.T - a) / np.linalg.norm(a) <= 4e-6


@pytest.mark.parametrize("n,m", [(100, 3), (191, 5), (777, 20), (2111, 37), (4160, 64), (8193, 17)])
def test_chain_substitution_matches_lookback(gpu_lla, n, m):
    """The chain form of the FP32 substitutions against the look-back form on
    the same factor: the first solve's backward error (set by the
    substitutions' accuracy) agrees within a factor of two, both converge to
    the FP64 target without fallback, with the same iteration count +-1.
    Sizes cover one to three block rows (no helper work), ragged last blocks,
    several column chunks and positions with several helper groups."""
    lla = gpu_lla
    rng = np.random.default_rng(n + m)
    a = qdq(rng, n, 1e5)
    b = rng.standard_normal((n, m))
    reps = {}
    for form in ("lookback", "chain"):
        x = b.copy()
        reps[form] = lla.posv_refined(a, x, residual="slices", substitution=form)
        assert reps[form]["converged"] == 1 and reps[form]["fell_back"] == 0, (form, reps[form])
        assert backward_error(a, x, b) <= 2e-13, form
    e0c, e0l = reps["chain"]["backward_error0"], reps["lookback"]["backward_error0"]
    assert 0.5 * e0l <= e0c <= 2.0 * e0l, (e0c, e0l)
    assert abs(reps["chain"]["iterations"] - reps["lookback"]["iterations"]) <= 1


def test_refine_autotune_records_and_reuses(gpu_lla, tmp_path, monkeypatch):
    """The per-shape autotuner times the refined solve's schedule candidates on
    the caller's system, records the winner under the shape key, and a later
    solve with default options runs that schedule (the report says which)."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    monkeypatch.setenv("LLA_AUTOTUNE_CACHE", str(tmp_path / "tune.txt"))
    rng = np.random.default_rng(77)
    n, m = 1537, 9
    a = qdq(rng, n, 1e5)
    b = rng.standard_normal((n, m))
    A = torch.tensor(a, device="cuda").T.contiguous().T
    B = torch.tensor(b, device="cuda").T.contiguous().T
    X = torch.empty_like(B.T.contiguous()).T
    chosen, ms = lla.refine_autotune(A, B, X, residual="slices")
    assert ms > 0 and chosen["update_kchunk"] in (32, 64) and chosen["update_epilogue"] in (1, 2)
    assert chosen["substitution"] in (1, 2)
    assert "r:n11:m4:u6:s1" in (tmp_path / "tune.txt").read_text()
    rep = lla.posv_refined_device(A, B, X, residual="slices")
    want = (chosen["update_kchunk"] << 8) | (chosen["update_epilogue"] << 4) | chosen["substitution"]
    assert rep["schedule"] == want and rep["converged"] == 1
    assert backward_error(a, X.cpu().numpy(), b) <= 2e-13


def test_concurrent_solves_on_two_streams_match_alone(gpu_lla):
    """Two refined solves from two host threads (each its own stream and
    workspace) overlap on the device: the persistent update kernels then share
    the SMs and claim their tiles from their own counters.  Each result is
    bit-identical to the same solve run alone."""
    import threading
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(31)
    systems = []
    for n in (2200, 1700):
        a = qdq(rng, n, 1e5)
        b = rng.standard_normal((n, 3))
        A = torch.tensor(a, device="cuda").T.contiguous().T
        B = torch.tensor(b, device="cuda").T.contiguous().T
        systems.append((A, B))
    alone = []
    for A, B in systems:
        X = torch.empty_like(B.T.contiguous()).T
        lla.posv_refined_device(A, B, X)
        torch.cuda.synchronize()
        alone.append(X.cpu().numpy())
    outs = [None, None]

    def run(i):
        A, B = systems[i]
        st = torch.cuda.Stream()
        X = torch.empty_like(B.T.contiguous()).T
        for _ in range(3):  # several rounds so that the solves do overlap
            with torch.cuda.stream(st):
                lla.posv_refined_device(A, B, X, stream=st)
        st.synchronize()
        outs[i] = X.cpu().numpy()

    th = [threading.Thread(target=run, args=(i,)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i in range(2):
        assert np.array_equal(outs[i], alone[i])
