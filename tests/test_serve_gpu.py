"""GPU tests of the serving loop: requests of different order, precision and
kind submitted while others run, admitted against an HBM budget, small ones
batched, large ones overlapped on several streams, factors kept for repeat
right-hand sides.

Each result must meet its request's tolerance (normwise backward error
measured here in FP64 from the inputs), and must equal -- within that
tolerance -- the result of the same request served alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def qdq(rng, n, kappa):
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.exp(rng.uniform(0, np.log(kappa), n))
    a = (q * s) @ q.T
    return (a + a.T) / 2


def col(torch, x, dtype):
    return torch.tensor(np.asarray(x), dtype=dtype, device="cuda").T.contiguous().T


def backward_error(a, x, b):
    a, x, b = (np.asarray(v, np.float64) for v in (a, x, b))
    r = b - a @ x
    return (np.abs(r).max(0) / (np.abs(a).sum(1).max() * np.abs(x).max(0) + np.abs(b).max(0))).max()


def make_requests(rng):
    reqs = []  # (kind, a, b, dtype, tol, keep)
    sizes = [40, 100, 256, 300, 700, 1200, 64, 200, 2048, 90]
    for i, n in enumerate(sizes):
        a = qdq(rng, n, 10 ** rng.uniform(1, 5))
        b = rng.standard_normal((n, int(rng.integers(1, 9))))
        f32 = i % 2 == 1
        reqs.append(("solve", a, b, np.float32 if f32 else np.float64, 1e-6 if f32 else 1e-13,
                     i == 4))
    n = 500
    l = np.linalg.cholesky(qdq(rng, n, 1e3))
    reqs.append(("trsm", l, rng.standard_normal((n, 3)), np.float64, 1e-13, False))
    return reqs


def serve(lla, torch, reqs, slots=4, budget=40e9, one_at_a_time=False):
    srv = lla.Server(hbm_budget_bytes=budget, slots=slots, batch_window_us=300.0)
    outs, res, handles = {}, {}, {}
    try:
        for tag, (kind, a, b, dt, tol, keep) in enumerate(reqs):
            tdt = torch.float64 if dt == np.float64 else torch.float32
            A, B = col(torch, a, tdt), col(torch, b, tdt)
            k = lla.REQ_TRSM if kind == "trsm" else lla.REQ_SOLVE
            srv.submit(k, A, B, tol=tol, keep_factor=keep, tag=tag)
            outs[tag] = B
            if one_at_a_time:
                srv.drain()
        srv.drain()
        torch.cuda.synchronize()
        for r in srv.poll():
            res[r["user_tag"]] = r
            if r["factor_handle"] > 0 and reqs[r["user_tag"]][5]:
                handles[r["user_tag"]] = r["factor_handle"]
        # repeat right-hand sides on the kept factors
        extra = {}
        for tag, h in handles.items():
            a = reqs[tag][1]
            b2 = np.random.default_rng(tag).standard_normal((a.shape[0], 2))
            A, B = col(torch, a, torch.float64), col(torch, b2, torch.float64)
            srv.submit(lla.REQ_RESOLVE, A, B, handle=h, tag=1000 + tag)
            extra[1000 + tag] = (a, b2, B)
        srv.drain()
        for r in srv.poll():
            res[r["user_tag"]] = r
        stats = srv.stats()
        for h in handles.values():
            srv.release(h)
    finally:
        srv.close()
    xs = {t: B.cpu().numpy().astype(np.float64) for t, B in outs.items()}
    return xs, res, extra, stats


def test_mixed_stream_meets_tolerances(gpu_lla):
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(2026)
    reqs = make_requests(rng)
    xs, res, extra, stats = serve(lla, torch, reqs)
    assert stats["completed"] == len(reqs) + len(extra)
    for tag, (kind, a, b, dt, tol, keep) in enumerate(reqs):
        r = res[tag]
        assert r["status"] == 0, r
        a_eff = a.astype(dt).astype(np.float64)
        b_eff = b.astype(dt).astype(np.float64)
        if kind == "trsm":
            be = backward_error(np.tril(a_eff), xs[tag], b_eff)
        else:
            be = backward_error(a_eff, xs[tag], b_eff)
        # f32 results are rounded to f32 on output
        assert be <= (tol if dt == np.float64 else 4 * tol), (tag, kind, a.shape[0], be, r)
        assert r["t_done_us"] >= r["t_start_us"] >= r["t_admit_us"] >= r["t_submit_us"]
    for tag, (a, b2, B) in extra.items():
        assert res[tag]["status"] == 0 and res[tag]["path"] == "kept_factor"
        assert backward_error(a, B.cpu().numpy(), b2) <= 1e-13
    paths = {res[t]["path"] for t in range(len(reqs))}
    assert "batched" in paths and "mixed" in paths


def test_same_result_alone_and_in_the_mix(gpu_lla):
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(7)
    reqs = make_requests(rng)
    x_mix, r_mix, _, _ = serve(lla, torch, reqs, slots=4)
    x_alone, r_alone, _, _ = serve(lla, torch, reqs, slots=1, one_at_a_time=True)
    for tag, (kind, a, b, dt, tol, keep) in enumerate(reqs):
        diff = np.abs(x_mix[tag] - x_alone[tag]).max() / max(np.abs(x_alone[tag]).max(), 1e-300)
        if r_mix[tag]["path"] in ("batched", "fp64") or kind == "trsm":
            assert diff == 0.0, (tag, r_mix[tag]["path"], diff)  # same kernels, same order
        else:
            kappa_bound = 1e5 * max(tol, 1e-13) * 10
            assert diff <= kappa_bound, (tag, diff)


def test_admission_respects_the_budget(gpu_lla):
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(11)
    reqs = [("solve", qdq(rng, n, 1e3), rng.standard_normal((n, 2)), np.float64, 1e-13, False)
            for n in (800, 900, 1000, 700, 600)]
    budget = 40e6  # a few of these at a time at most
    xs, res, _, stats = serve(lla, torch, reqs, slots=4, budget=budget)
    assert stats["bytes_peak"] <= budget
    for tag, (kind, a, b, dt, tol, keep) in enumerate(reqs):
        assert res[tag]["status"] == 0
        assert backward_error(a, xs[tag], b) <= 1e-13
    srv = lla.Server(hbm_budget_bytes=1e6)
    try:
        big = col(torch, np.eye(2000), torch.float64)
        with pytest.raises(lla.DeviceError) as e:
            srv.submit(lla.REQ_SOLVE, big, col(torch, np.ones((2000, 1)), torch.float64))
        assert e.value.code == lla.ERR_BUSY
    finally:
        srv.close()


def test_not_positive_definite_request(gpu_lla):
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    a = np.eye(400)
    a[10, 10] = -1
    small = np.eye(50)
    small[3, 3] = -2
    srv = lla.Server()
    try:
        A, B = col(torch, a, torch.float64), col(torch, np.ones((400, 1)), torch.float64)
        As, Bs = col(torch, small, torch.float64), col(torch, np.ones((50, 1)), torch.float64)
        srv.submit(lla.REQ_SOLVE, A, B, tag=1)
        srv.submit(lla.REQ_SOLVE, As, Bs, tag=2)
        srv.drain()
        res = {r["user_tag"]: r for r in srv.poll()}
        assert res[1]["status"] == lla.NOT_POSITIVE_DEFINITE
        assert res[2]["status"] == lla.NOT_POSITIVE_DEFINITE
    finally:
        srv.close()


def test_device_loop_serves_requests_as_they_arrive(gpu_lla):
    """Small requests go to the device-resident loop as soon as they are
    admitted.  Requests submitted while the loop runs join it; a pause longer
    than its idle limit lets its CTAs return, and the next request relaunches
    it.  Each result is bit-identical to the batched kernel's solve of the same
    system (the same per-CTA arithmetic), for f64 and f32."""
    import time
    torch = pytest.importorskip("torch")
    lla = gpu_lla
    rng = np.random.default_rng(99)
    systems = []
    for i in range(40):
        n = int(rng.integers(16, 257))
        m = int(rng.integers(1, 9))
        dt = np.float64 if i % 3 else np.float32
        g = rng.standard_normal((n, n))
        systems.append(((g @ g.T / n + 0.1 * np.eye(n)).astype(dt), rng.standard_normal((n, m)).astype(dt)))
    srv = lla.Server(batch_window_us=500.0, device_ctas=8)
    outs = {}
    try:
        for tag, (a, b) in enumerate(systems):
            tdt = torch.float64 if a.dtype == np.float64 else torch.float32
            A, B = col(torch, a, tdt), col(torch, b, tdt)
            torch.cuda.synchronize()
            srv.submit(lla.REQ_SOLVE, A, B, tag=tag)
            outs[tag] = B
            if tag in (9, 19, 29):
                time.sleep(0.02)  # longer than the idle limit: the loop's CTAs return
        srv.drain()
        res = {r["user_tag"]: r for r in srv.poll()}
        stats = srv.stats()
    finally:
        srv.close()
    assert stats["device_loop_launches"] >= 2, stats
    for dt in (np.float64, np.float32):
        idx = [i for i, (a, _) in enumerate(systems) if a.dtype == dt]
        plan = lla.BatchPlan(np.array([systems[i][0].shape[0] for i in idx], np.int32),
                             np.array([systems[i][1].shape[1] for i in idx], np.int32),
                             "f64" if dt == np.float64 else "f32")
        ap, bp = plan.pack([systems[i][0] for i in idx], [systems[i][1] for i in idx])
        dA, dB = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
        info = torch.full((plan.count,), -7, dtype=torch.int32, device="cuda")
        plan.solve(dA, dB, info)
        torch.cuda.synchronize()
        xb = plan.unpack_x(dB.cpu().numpy())
        for k, i in enumerate(idx):
            r = res[i]
            assert r["status"] == 0 and r["path"] == "batched", r
            x = outs[i].cpu().numpy()
            assert np.array_equal(x, xb[k]), (i, np.abs(x - xb[k]).max())
            a, b = systems[i]
            assert backward_error(a, x, b) <= 10 * a.shape[0] * np.finfo(dt).eps
