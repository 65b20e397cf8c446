"""GPU tests of the batched path: many independent SPD systems of uneven
order in one persistent launch (and its CUDA-graph replay).

Each system must be solved to the accuracy of the per-matrix FP64 path
(normwise backward error <= 10 n eps of its element type), failures must be
reported per system at the row the reference would report, and the graph
replay must reproduce the direct launch bit for bit (each system is solved by
exactly one CTA with a fixed operation order)."""
import numpy as np
import pytest

from oracle import oracle as ora

pytestmark = pytest.mark.gpu


def make_batch(rng, count, dtype, nmax=256):
    n = np.exp(rng.uniform(np.log(16), np.log(nmax), count)).astype(np.int32)
    n[: 8] = [1, 2, 31, 32, 33, 64, 255, 256][: min(8, count)]
    n = np.minimum(n, nmax)
    m = rng.integers(1, 9, count).astype(np.int32)
    As, Bs = [], []
    for i in range(count):
        g = rng.standard_normal((n[i], n[i]))
        As.append((g @ g.T / n[i] + 0.1 * np.eye(n[i])).astype(dtype))
        Bs.append(rng.standard_normal((n[i], m[i])).astype(dtype))
    return n, m, As, Bs


def backward_error(a, x, b):
    a, x, b = (np.asarray(v, np.float64) for v in (a, x, b))
    r = b - a @ x
    return (np.abs(r).max(0) / (np.abs(a).sum(1).max() * np.abs(x).max(0) + np.abs(b).max(0))).max()


def run(lla, plan, As, Bs, graph=False):
    torch = pytest.importorskip("torch")
    ap, bp = plan.pack(As, Bs)
    dA = torch.from_numpy(ap).cuda()
    dB = torch.from_numpy(bp).cuda()
    info = torch.full((plan.count,), -7, dtype=torch.int32, device="cuda")
    (plan.solve_graph if graph else plan.solve)(dA, dB, info)
    torch.cuda.synchronize()
    return plan.unpack_x(dB.cpu().numpy()), info.cpu().numpy(), dA.cpu().numpy()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batch_matches_fp64_accuracy(gpu_lla, dtype):
    lla = gpu_lla
    rng = np.random.default_rng(77)
    n, m, As, Bs = make_batch(rng, 300, dtype)
    plan = lla.BatchPlan(n, m, "f64" if dtype == np.float64 else "f32")
    X, info, _ = run(lla, plan, As, Bs)
    assert np.all(info == -1)
    eps = np.finfo(dtype).eps
    prev = lla.set_algorithm(lla.ALGO_FAST)
    try:
        for i in range(plan.count):
            be = backward_error(As[i], X[i], Bs[i])
            assert be <= 10 * n[i] * eps, (i, n[i], be)
            # the per-matrix FP64 (FAST) path on the same system reaches the same class
            if i % 25 == 0:
                xi = lla.solvec(As[i].copy(), Bs[i])
                assert backward_error(As[i], xi, Bs[i]) <= 10 * n[i] * eps
    finally:
        lla.set_algorithm(prev)


def test_batch_graph_replay_is_bit_identical(gpu_lla):
    lla = gpu_lla
    rng = np.random.default_rng(78)
    n, m, As, Bs = make_batch(rng, 200, np.float64)
    plan = lla.BatchPlan(n, m, "f64")
    X1, info1, L1 = run(lla, plan, As, Bs)
    X2, info2, L2 = run(lla, plan, As, Bs, graph=True)
    X3, info3, L3 = run(lla, plan, As, Bs, graph=True)  # replay of the instantiated graph
    assert np.array_equal(info1, info2) and np.array_equal(info1, info3)
    assert np.array_equal(L1, L2) and np.array_equal(L1, L3)
    for a, b, c in zip(X1, X2, X3):
        assert np.array_equal(a, b) and np.array_equal(a, c)


def test_batch_reports_failures_per_system(gpu_lla):
    lla = gpu_lla
    rng = np.random.default_rng(79)
    n, m, As, Bs = make_batch(rng, 40, np.float64)
    bad = {3: 0, 10: 5, 17: None}
    for i, r in bad.items():
        if r is None:
            r = n[i] - 1
        r = min(r, n[i] - 1)
        As[i][r, r] = -1.0
        bad[i] = r
    plan = lla.BatchPlan(n, m, "f64")
    X, info, _ = run(lla, plan, As, Bs)
    for i in range(plan.count):
        if i in bad:
            ref = As[i].copy()
            st = ora.cholesky_inplace_dirty(ref)
            assert st["code"] == 2 and info[i] == st["index"], (i, info[i], st)
        else:
            assert info[i] == -1
            assert backward_error(As[i], X[i], Bs[i]) <= 10 * n[i] * np.finfo(np.float64).eps


def test_batch_rejects_oversized_systems(gpu_lla):
    lla = gpu_lla
    with pytest.raises(lla.DeviceError) as e:
        lla.BatchPlan([300], [1])
    assert e.value.code == 23
    with pytest.raises(lla.DeviceError):
        lla.BatchPlan([10], [9])


def test_batch_autotune_keeps_results(gpu_lla, tmp_path, monkeypatch):
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("LLA_AUTOTUNE_CACHE", str(tmp_path / "tune.txt"))
    lla = gpu_lla
    rng = np.random.default_rng(80)
    n, m, As, Bs = make_batch(rng, 64, np.float64)
    plan = lla.BatchPlan(n, m, "f64")
    ap, bp = plan.pack(As, Bs)
    dA, dB = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    info = torch.empty(plan.count, dtype=torch.int32, device="cuda")
    ms = plan.autotune(dA, dB, info)
    assert ms > 0
    # the pools still hold the inputs
    assert np.array_equal(dA.cpu().numpy(), ap) and np.array_equal(dB.cpu().numpy(), bp)
    assert (tmp_path / "tune.txt").read_text().strip()


@pytest.mark.parametrize("dtype", ["f64", "f32", "f64-refined"])
def test_batch_configuration_10000_systems(gpu_lla, dtype):
    """The batched configuration at its own size: 10,000 systems, n log-uniform
    in [16, 256], A = G G^T / n + 0.1 I, 1..8 RHS, one graph replay; EVERY
    system within the per-matrix FP64 class (backward error <= 10 n eps)."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    count = 10000
    rng = np.random.default_rng(10000)
    n = np.clip(np.exp(rng.uniform(np.log(16), np.log(256), count)).round(), 16, 256).astype(np.int32)
    m = rng.integers(1, 9, count).astype(np.int32)
    dt = torch.float32 if dtype == "f32" else torch.float64
    plan = lla.BatchPlan(n, m, dtype[:3])
    if dtype == "f64-refined":
        plan.set_refined(True)
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    A0 = torch.zeros(plan.a_elems, dtype=dt, device="cuda")
    B0 = torch.zeros(plan.b_elems, dtype=dt, device="cuda")
    As, Bs = [], []
    for i in range(count):
        G = torch.randn(int(n[i]), int(n[i]), dtype=torch.float64, device="cuda", generator=g)
        a = (G @ G.T / int(n[i]) + 0.1 * torch.eye(int(n[i]), dtype=torch.float64, device="cuda")).to(dt)
        b = torch.randn(int(n[i]), int(m[i]), dtype=torch.float64, device="cuda", generator=g).to(dt)
        As.append(a)
        Bs.append(b)
        A0[plan.a_off[i]:plan.a_off[i] + n[i] * n[i]] = a.T.reshape(-1)
        B0[plan.b_off[i]:plan.b_off[i] + n[i] * m[i]] = b.T.reshape(-1)
    info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    plan.solve_graph(A0, B0, info)
    torch.cuda.synchronize()
    assert int((info != -1).sum()) == 0
    eps = float(torch.finfo(dt).eps)
    worst = []
    for i in range(count):
        x = B0[plan.b_off[i]:plan.b_off[i] + n[i] * m[i]].reshape(int(m[i]), int(n[i])).T.double()
        a, b = As[i].double(), Bs[i].double()
        r = b - a @ x
        be = (r.abs().amax(0) / (a.abs().sum(1).amax() * x.abs().amax(0) + b.abs().amax(0))).amax()
        worst.append(be / (float(n[i]) * eps))
    w = float(torch.stack(worst).max())
    assert w <= 10.0, w


def test_batch_refined_mode(gpu_lla):
    """f64 systems through an FP32 factorisation with per-system FP64
    refinement: every system at the per-matrix FP64 class (backward error
    <= 10 n eps), A left untouched (read only), the graph replay identical to
    the direct launch, and a non-SPD system reported at the row the plain FP64
    batched solve reports (its fallback is that routine)."""
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(808)
    n, m, As, Bs = make_batch(rng, 300, np.float64)
    bad = [5, 77, 150]
    for i in bad:
        As[i] = As[i].copy()
        As[i][min(3, n[i] - 1), min(3, n[i] - 1)] = -1.0
    plan = lla.BatchPlan(n, m, "f64")
    plan.set_refined(True)
    X, info, a_after = run(lla, plan, As, Bs)
    ap, _ = plan.pack(As, Bs)
    assert np.array_equal(a_after, ap)  # A is read only in this mode
    eps = np.finfo(np.float64).eps
    for i in range(plan.count):
        if i in bad:
            continue
        assert info[i] == -1, (i, info[i])
        be = backward_error(As[i], X[i], Bs[i])
        assert be <= 10 * n[i] * eps, (i, n[i], be)
    X2, info2, _ = run(lla, plan, As, Bs, graph=True)
    assert np.array_equal(info, info2) and all(np.array_equal(X[i], X2[i]) for i in range(plan.count))
    plain = lla.BatchPlan(n, m, "f64")
    _, info_p, _ = run(lla, plain, As, Bs)
    for i in bad:
        assert info[i] == info_p[i] and info[i] >= 0, (i, info[i], info_p[i])
    with pytest.raises(lla.DeviceError):
        lla.BatchPlan(n[:4], m[:4], "f32").set_refined(True)
