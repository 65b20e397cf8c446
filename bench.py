"""Benchmark: SPD solves/s of the single large f64 system, n = 16384 with 64
right-hand sides, A = Q diag(s) Q^T (Q from the QR of a seeded Gaussian,
s log-uniform in [1, 1e6], kappa = 1e6), B ~ N(0, 1), on one GB300.

A "step" is one complete solve of that system with the inputs resident in
HBM: copy A into the working buffer, factor, and solve (plus refinement for
the mixed-precision form).  Every solution is checked to reach normwise
backward error <= 1e-13 before a number is reported.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores (the C
restatement of linfa-linalg's solvec in oracle/, the reference itself being a
Rust crate that cannot be built here) on bounded samples of the same workload
and scales them to the n = 16384 system by the flop model.

Under torchrun (N > 1) each rank solves its own copy of the system (a single
factorisation does not shard: replicas only); `value` is the solves of all
ranks divided by the slowest rank's time.
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT, NRHS_DEFAULT, KAPPA_DEFAULT, SEED = 16384, 64, 1e6, 20240611
BE_TARGET = 1e-13
METRIC = "SPD solves/s at backward error <= 1e-13 (n=16384, 64 RHS, kappa=1e6)"


def max_over_ranks(dist, ms, device):
    """The slowest rank's time for the timed region (ranks are replicas, each solving
    its own system), then a barrier so that no rank starts the next phase early."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def job_rate(world, steps, ms):
    """Solves per second of the whole job: every rank solved `steps` systems within ms."""
    return world * steps / (ms / 1e3)


def mixed_update_bytes(n, nb=128):
    """FP32 trailing-matrix bytes (read + write of the lower part) of the tensor-core
    updates of one low-precision factorisation, and their launch count: panels in
    pairs, a narrow update of the next 128-column block, then one update of the rest."""
    tot, launches, p = 0.0, 0, 0
    while p < n:
        b = min(nb, n - p)
        rest = n - p - b
        if rest <= 0:
            break
        if rest > nb:
            rows = n - p - nb
            tot += (rows * nb - nb * (nb - 1) / 2) * 8
            rows = n - p - 2 * nb
            tot += rows * (rows + 1) / 2 * 8
            launches += 2
            p += 2 * nb
        else:
            rows = n - p - nb
            tot += rows * (rows + 1) / 2 * 8
            launches += 1
            p += nb
    return tot, launches


def flops_solve(n, m):
    """Cholesky n^3/3 + two triangular solves 2 n^2 m."""
    return n ** 3 / 3.0 + 2.0 * n * n * m


# ---------------------------------------------------------------------------
# reference arm / CPU baseline (oracle; test infrastructure, never the product)

def _cpu_sample(args):
    n, m, seed = args
    from oracle import oracle as ora
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n))
    a = g @ g.T / n + np.eye(n)
    b = rng.standard_normal((n, m))
    t0 = time.perf_counter()
    st = ora.solvec_inplace(a, b)
    dt = time.perf_counter() - t0
    assert st["code"] == 0
    return dt


class OneCore:
    """Pins the calling process to one host core (the reference is
    single-threaded) and restores its affinity afterwards."""

    def __enter__(self):
        self.prev = None
        if hasattr(os, "sched_getaffinity"):
            self.prev = os.sched_getaffinity(0)
            os.sched_setaffinity(0, {min(self.prev)})
        return self

    def __exit__(self, *a):
        if self.prev is not None:
            os.sched_setaffinity(0, self.prev)


def cpu_rate(n_sample, m, seed=1):
    """The oracle's single-core solve of an n_sample system with m right-hand
    sides, timed directly; returns (seconds, solves/s of the n = 16384 system
    extrapolated from it by the flop model n^3/3 + 2 n^2 m)."""
    with OneCore():
        dt = _cpu_sample((n_sample, m, seed))
    scale = flops_solve(n_sample, m) / flops_solve(N_DEFAULT, NRHS_DEFAULT)
    return dt, scale / dt


def run_cpu_sweep(args):
    """The oracle (one core) timed directly at n = 512 .. 4096, 64 RHS (and the
    n=512, 1-RHS single-matrix workload): the CPU side of the scaling table."""
    from oracle import oracle as ora
    ora.lib()
    rows = []
    with OneCore():
        for n, m in [(512, 1), (512, 64), (1024, 64), (2048, 64), (4096, 64)]:
            dt = _cpu_sample((n, m, 7))
            rows.append({"n": n, "nrhs": m, "seconds": dt, "solves_per_s": 1.0 / dt,
                         "gflops": flops_solve(n, m) / dt / 1e9})
    # n^3 fit of the largest timed size, for the sizes not timed directly
    big = rows[-1]
    extrap = {str(n): big["seconds"] * flops_solve(n, NRHS_DEFAULT) / flops_solve(big["n"], 64)
              for n in (8192, 16384)}
    print(json.dumps({"workload": "cpu-sweep", "impl": "oracle (1 core, -O2 -ffp-contract=off)",
                      "cores": 1, "rows": rows, "extrapolated_seconds_by_flops": extrap,
                      "cpu": platform.processor() or platform.machine()}))


def run_reference(args):
    """The reference's CPU algorithm (the oracle: a loop-for-loop C restatement
    of linfa-linalg's solvec, single-threaded like the reference), pinned to one
    host core.  Each timed step is one complete solve of an n = 4096, 64-RHS
    SPD system, the largest sample that keeps the run within a few minutes; the
    n = 16384 rate is extrapolated from it by the flop model and marked so."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as ora
    ora.lib()  # builds the oracle if needed
    n_s, m = args.ref_sample_n, NRHS_DEFAULT
    for i in range(args.warmup):  # the C code has no JIT; a short solve pages it in
        _cpu_sample((min(n_s, 1024), m, 100 + i))
    secs = [cpu_rate(n_s, m, seed=1 + i)[0] for i in range(args.steps)]
    sec = statistics.median(secs)
    scale = flops_solve(n_s, m) / flops_solve(N_DEFAULT, NRHS_DEFAULT)
    value = scale / sec
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sec, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "extrapolated": True,
        "config": {"workload": f"single SPD solve n={N_DEFAULT} nrhs={NRHS_DEFAULT} kappa=1e6",
                   "sample": f"one solvec of n={n_s} nrhs={m} per step (A = G G^T/n + I), 1 core; "
                             f"warm-up steps at n={min(n_s, 1024)}"},
        "measured": {"n": n_s, "nrhs": m, "seconds_median": sec, "seconds": secs,
                     "solves_per_s": 1.0 / sec, "gflops": flops_solve(n_s, m) / sec / 1e9},
        "extrapolation": f"solves/s at n={N_DEFAULT}, m={NRHS_DEFAULT} = measured rate at n={n_s} x "
                         f"(n^3/3 + 2 n^2 m at n={n_s}) / (the same at n={N_DEFAULT}) = x{scale:.3e}",
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": 1, "kind": "port",
                         "extrapolated": True,
                         "sample": f"oracle solvec n={n_s} m={m} on 1 pinned core, median of "
                                   f"{args.steps}; n^3 fit to n={N_DEFAULT}",
                         "cpu": platform.processor() or platform.machine(),
                         "host_cores": os.cpu_count()},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# GPU arm

class Clocks:
    """nvidia-smi sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        rows = []
        with open(self.f.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def make_system(torch, n, m, kappa, seed, device):
    """A = Q diag(s) Q^T, Q from QR of a seeded Gaussian, s log-uniform in
    [1, kappa]; B ~ N(0,1).  Built in FP64 on the device."""
    # torch loads its CUDA linear-algebra library lazily by name; under a
    # profiler that rewrites the loader environment that lookup can fail, so
    # load it by path first.
    import ctypes
    lib = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
    if os.path.exists(lib):
        ctypes.CDLL(lib, mode=ctypes.RTLD_GLOBAL)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    G = torch.randn(n, n, dtype=torch.float64, device=device, generator=g)
    Q, _ = torch.linalg.qr(G)
    del G
    u = torch.rand(n, dtype=torch.float64, device=device, generator=g)
    s = torch.exp(u * np.log(kappa))
    s[0], s[-1] = 1.0, kappa
    A = (Q * s) @ Q.T
    del Q
    A = (A + A.T) * 0.5
    B = torch.randn(n, m, dtype=torch.float64, device=device, generator=g)
    return A, B


def backward_error(torch, A, X, B):
    R = B - A @ X
    num = R.abs().amax(dim=0)
    den = A.abs().sum(dim=1).amax() * X.abs().amax(dim=0) + B.abs().amax(dim=0)
    return float((num / den).max())


def roofline_of(kern, prof, args, n, m, hbm, bf16, fp64_peak, ffma_peak, peak_note, ms_step):
    """Roofline of one kernel of the headline solve from its live CUDA-event time
    and its ALGORITHMIC work per launch (the flops and bytes the operation needs,
    not what the implementation executes).  The bound is the roofline whose floor
    (work / peak) is the larger for that work; `frac` = that floor / the measured
    time.  Executed-work figures (term products on the tensor pipe) are reported
    beside it, never as `frac`."""
    k_ms, k_n, k_work = prof[kern]
    sec = k_ms * 1e-3
    out = {"kernel": kern, "launches": k_n, "avg_launch_ms": k_ms / max(k_n, 1),
           "share_of_step": k_ms / ms_step, "peak_source": peak_note}
    if kern == "mixed_update":
        # per solve: n^3/3 flops (one product per term, the algorithmic update) against
        # the FP32 trailing matrix's read + write, m(m+1)/2 * 8 bytes per K = 256 pass
        # of the panel-pair schedule: 64 flop/B, below the ridge (bf16 peak / HBM, about
        # 280 flop/B), so HBM bounds the algorithmic work
        upd_bytes, upd_launches = mixed_update_bytes(n)
        solves = k_n / upd_launches
        flops, byts = k_work, upd_bytes * solves
        products = {"bf16": 1, "fp16": 1, "bf16x3": 3, "fp16x3": 3, "bf16x6": 6}.get(args.update, 1)
        out.update({"tensor_pipe_tflops": products * flops / sec / 1e12,
                    "tensor_pipe_frac": products * flops / sec / 1e12 / bf16,
                    "tensor_products": products,
                    "note": "frac: algorithmic bytes (FP32 trailing matrix read + write of the pair schedule) "
                            "over the measured copy bandwidth; flop_frac: n^3/3 flops over the bf16 burst; "
                            "tensor_pipe_frac: executed term products over the bf16 burst"})
        fpeak, funit = bf16, "TFLOP/s (bf16 tensor)"
    elif kern == "mixed_trsm":
        # FP32 substitutions: n^2 m flops per launch against the lower triangle of the
        # FP32 factor (2 n^2 bytes) and B (read + write, 8 n m): m/2 flop/B, above the
        # FFMA ridge (FFMA peak / HBM, about 11 flop/B), so FP32 FFMA bounds them
        nsub = max(1, k_n - 2 * args.steps)  # minus the per-factor inverse and coupling kernels
        flops, byts = k_work, nsub * (2.0 * n * n + 16.0 * n * m)
        fpeak, funit = ffma_peak, "TFLOP/s (FP32 FMA, measured live)"
        out["note"] = "substitution launches only; flops n^2 m per launch"
    elif kern == "residual":
        # R = B - A X in FP64 accuracy: 2 n^2 m flops, the lower triangle of A (4 n^2 bytes)
        flops, byts = k_work, k_n * (4.0 * n * n + 24.0 * n * m)
        if args.residual == "slices":
            fpeak, funit = bf16, "TFLOP/s (bf16 tensor; FP64-equivalent flops)"
            out.update({"tensor_pipe_tflops": 36 * flops / sec / 1e12,
                        "tensor_pipe_frac": 36 * flops / sec / 1e12 / bf16})
        else:
            fpeak, funit = fp64_peak, "TFLOP/s (FP64 tensor pipe, measured live)"
    else:
        flops, byts = k_work, None
        fpeak, funit = ffma_peak, "TFLOP/s (FP32 FMA, measured live)"
    t_flop = flops / (fpeak * 1e12) if fpeak and fpeak > 0 else 0.0
    t_byte = byts / (hbm * 1e9) if byts else 0.0
    if t_byte >= t_flop and byts:
        out.update({"bound": "hbm", "achieved": byts / sec / 1e9, "peak": hbm, "unit": "GB/s",
                    "frac": t_byte / sec, "algorithmic_bytes_per_launch": byts / k_n})
    else:
        out.update({"bound": "tensor" if "tensor" in funit else "fp32-fma", "achieved": flops / sec / 1e12,
                    "peak": fpeak, "unit": funit.split(" (")[0], "peak_kind": funit, "frac": t_flop / sec})
        if byts:
            out["algorithmic_bytes_per_launch"] = byts / k_n
    out["flop_frac"] = flops / sec / 1e12 / fpeak if fpeak and fpeak > 0 else None
    out["flop_peak_kind"] = funit
    if byts:
        out["hbm_frac"] = byts / sec / 1e9 / hbm
    # DRAM traffic of one ncu-captured launch, scaled to this workload's launches
    tpath = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    key = "residual_slices" if kern == "residual" and args.residual == "slices" else kern
    t = json.load(open(tpath)).get(key) if os.path.exists(tpath) else None
    out["traffic"], out["traffic_source"] = None, None
    if t and "algorithmic_bytes" in t and out.get("algorithmic_bytes_per_launch"):
        ratio = t["dram_bytes"] / t["algorithmic_bytes"]
        out["traffic"] = ratio * out["algorithmic_bytes_per_launch"]
        out["traffic_source"] = f"{t['source']} (DRAM/algorithmic = {ratio:.2f})"
    elif t and "n_captured" in t:
        out["traffic"] = t["dram_bytes"] * (n / t["n_captured"]) ** t["exponent"]
        out["traffic_source"] = f"{t['source']}, scaled from n={t['n_captured']} by (n/{t['n_captured']})^{t['exponent']}"
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--nrhs", type=int, default=NRHS_DEFAULT)
    ap.add_argument("--ref-sample-n", type=int, default=4096)
    ap.add_argument("--cpu-sample-n", type=int, default=4096)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer C-ABI leg")
    ap.add_argument("--update", default="bf16x6",
                    help="trailing-update form of the mixed path: fp32|bf16|bf16x3|bf16x6|fp16|fp16x3")
    ap.add_argument("--plain-steps", type=int, default=2, help="timed steps of the plain FP64 leg")
    ap.add_argument("--substitution", default="auto", choices=["auto", "chain", "lookback"],
                    help="form of the refinement's FP32 substitutions")
    ap.add_argument("--residual", default="slices", choices=["fp64", "slices"],
                    help="refinement residual of the headline: FP64 MMA pipe, or exact BF16 slices")
    ap.add_argument("--no-alt", action="store_true", help="skip timing the other residual method")
    ap.add_argument("--workload", default="single",
                    choices=["single", "batch", "serve", "sweep", "cpu-sweep"],
                    help="single: the n=16384 system (the headline); batch: 10,000 uneven small systems")
    ap.add_argument("--batch-count", type=int, default=10000)
    ap.add_argument("--batch-dtype", default="f64", choices=["f64", "f32"])
    ap.add_argument("--batch-refined", action="store_true",
                    help="f64 batch through an FP32 factor with per-system FP64 refinement")
    ap.add_argument("--serve-requests", type=int, default=400)
    ap.add_argument("--serve-rates", default="100,200,400,800", help="Poisson arrival rates (requests/s)")
    ap.add_argument("--serve-rate", type=float, default=200.0,
                    help="arrival rate of the serving leg of the default run (requests/s)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched leg of the default run")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg of the default run")
    args = ap.parse_args()
    if args.workload == "cpu-sweep":
        run_cpu_sweep(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "serve":
        run_serve(args)
        return
    if args.workload == "sweep":
        run_sweep(args)
        return

    import torch
    import __graft_entry__
    lla = __graft_entry__.load_package()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    n, m = args.n, args.nrhs

    # CPU baseline first (before any GPU work), bounded sample, 1 core
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as ora
        ora.lib()
        dt, rate = cpu_rate(args.cpu_sample_n, m)
        cpu = {"value": rate, "unit": "solves/s", "cores": 1, "kind": "port", "extrapolated": True,
               "sample": f"oracle solvec n={args.cpu_sample_n} m={m} on 1 pinned core took {dt:.2f} s; "
                         f"scaled by (n^3/3+2n^2m) to n={n}"}

    A0, B0 = make_system(torch, n, m, KAPPA_DEFAULT, SEED + rank, dev)
    A0c = A0.T  # A is symmetric: its row-major buffer is also its column-major buffer
    B0c = B0.T.contiguous().T  # column-major (n, m)
    W = torch.empty_like(A0)
    X = torch.empty_like(B0c.T).T  # column-major (n, m)
    Xm = torch.empty_like(B0c.T).T
    info = torch.empty(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()

    def plain_step():
        W.copy_(A0)
        lla.potrf_device(W.T, algo=lla.ALGO_FAST, info=info, stream=stream)
        X.copy_(B0c)
        lla.trsm_device(W.T, X, 0, algo=lla.ALGO_FAST, stream=stream)
        lla.trsm_device(W.T, X, 1, algo=lla.ALGO_FAST, stream=stream)

    reports = []

    def mixed_step(residual=args.residual):
        reports.append(lla.posv_refined_device(A0c, B0c, Xm, stream=stream, update=args.update,
                                               residual=residual, substitution=args.substitution))

    # the refined solve's schedule for this shape, from the per-shape autotuner (recorded in the
    # autotune cache; the timed solves below take it up with their default options)
    schedule = None
    if args.substitution == "auto":
        chosen, tune_ms = lla.refine_autotune(A0c, B0c, Xm, stream=stream, update=args.update,
                                              residual=args.residual)
        schedule = dict(chosen, autotune_best_ms=tune_ms)
    # correctness gates (outside the timed regions)
    plain_step()
    torch.cuda.synchronize()
    assert int(info.item()) == -1, "plain FP64 factorisation failed"
    be_plain = backward_error(torch, A0, X, B0)
    assert be_plain <= BE_TARGET, be_plain
    mixed_step()
    torch.cuda.synchronize()
    be_mixed = backward_error(torch, A0, Xm, B0)
    assert be_mixed <= BE_TARGET, (be_mixed, reports[-1])
    fwd_vs_fp64 = float((Xm - X).abs().max() / X.abs().max())

    def timed(step, k, w, profile=False):
        for _ in range(w):
            step()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        l0 = lla.kernel_launches()
        if profile:
            lla.profile_start()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(k + 1)]
        with Clocks(local) as clk:
            ev[0].record(stream)
            for i in range(k):
                step()
                ev[i + 1].record(stream)  # per-solve latency (the steps run back to back)
            torch.cuda.synchronize()
        prof = lla.profile_stop() if profile else None
        launches = lla.kernel_launches() - l0
        ms = ev[0].elapsed_time(ev[k])
        timed.per_step = [ev[i].elapsed_time(ev[i + 1]) for i in range(k)]
        ms = max_over_ranks(dist, ms, dev)
        return ms, launches, prof, clk.summary()

    k_plain = max(1, min(args.steps, args.plain_steps))
    ms_plain, _, prof_plain, _ = timed(plain_step, k_plain, min(args.warmup, 3), profile=True)
    plain_sps = job_rate(world, k_plain, ms_plain)
    reports.clear()
    ms_mixed, launches, prof, clocks = timed(mixed_step, args.steps, args.warmup, profile=True)
    lat = sorted(timed.per_step)
    latency = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
               "max_ms": lat[-1], "samples": len(lat),
               "note": "per-solve CUDA-event durations of the timed steps (device-resident A, B)"}
    timed_reports = reports[-args.steps:]
    mixed_sps = job_rate(world, args.steps, ms_mixed)
    assert all(r["backward_error"] <= BE_TARGET for r in timed_reports), timed_reports
    # the other residual method, timed the same way (reported beside the headline)
    alt = None
    if not args.no_alt:
        other = "slices" if args.residual == "fp64" else "fp64"
        reports.clear()
        ms_alt, _, prof_alt, _ = timed(lambda: mixed_step(other), args.steps, 1, profile=True)
        torch.cuda.synchronize()
        be_alt = backward_error(torch, A0, Xm, B0)
        assert be_alt <= BE_TARGET and all(r["backward_error"] <= BE_TARGET for r in reports), be_alt
        alt = {"residual": other, "value": job_rate(world, args.steps, ms_alt), "unit": "solves/s",
               "ms_per_step": ms_alt / args.steps, "iterations": reports[-1]["iterations"],
               "backward_error": be_alt,
               "kernels": {k: {"ms": v[0] / args.steps, "launches": v[1] // args.steps}
                           for k, v in prof_alt.items()}}

    # roofline of the dominant kernel of the headline (mixed) step: algorithmic units per
    # launch from the kernel's own accounting, live CUDA-event durations
    fp64_peak = lla.measure_peak_tflops(0)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    bf16 = peaks.get("bf16_tflops", 1900.0)
    peak_note = "MEASURED_PEAKS.json" if peaks else "fallback (6.8 TB/s, 1.9 PF/s)"
    ffma_peak = lla.measure_peak_tflops(2)
    dom = max(prof, key=lambda k: prof[k][0])
    roofline = roofline_of(dom, prof, args, n, m, hbm, bf16, fp64_peak, ffma_peak, peak_note, ms_mixed)
    roofline_others = {k: roofline_of(k, prof, args, n, m, hbm, bf16, fp64_peak, ffma_peak, peak_note, ms_mixed)
                       for k in ("mixed_update", "mixed_trsm", "residual", "mixed_diag", "mixed_panel")
                       if k in prof and k != dom}

    # end to end through the C ABI with host (pinned) buffers: lla_dposv_refined reads A
    # and overwrites B with X
    e2e = None
    if rank == 0 and not args.no_e2e:
        Ah = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
        Bh = torch.empty((n, m), dtype=torch.float64, pin_memory=True)
        Ah.copy_(A0.cpu())
        B0_cpu = B0.cpu()
        tot, k_e2e = 0.0, max(1, args.steps)
        for it in range(k_e2e + 1):
            Bh.copy_(B0_cpu)
            t0 = time.perf_counter()
            lla.posv_refined(Ah.numpy(), Bh.numpy(), update=args.update, residual=args.residual,
                             substitution=args.substitution)
            dt = time.perf_counter() - t0
            if it > 0:
                tot += dt
        be = backward_error(torch, A0, Bh.to(dev), B0)
        assert be <= BE_TARGET, be
        e2e = {"value": k_e2e / tot, "unit": "solves/s",
               "h2d_bytes_per_step": (n * n + n * m) * 8, "d2h_bytes_per_step": n * m * 8,
               "path": "lla_dposv_refined: pinned host row-major A (read) and B (overwritten by X)"}

    # the batched and serving configurations, measured in the same run (rank 0)
    batch = serve = None
    if rank == 0 and not args.no_batch:
        kb, wb = max(3, min(args.steps, 10)), max(3, args.warmup)
        batch = {dtn: measure_batch(torch, lla, dev, args.batch_count, dtn, kb, wb,
                                    cpu_sample=0 if args.no_cpu else 200)
                 for dtn in ("f64", "f32")}
        batch["f64_refined"] = measure_batch(torch, lla, dev, args.batch_count, "f64", kb, wb, refined=True)
    if rank == 0 and not args.no_serve:
        rng = np.random.default_rng(SEED)
        pool, tri = serve_pools(torch, dev, rng)
        serve = measure_serve(torch, lla, dev, pool, tri, rng, args.serve_rate, args.serve_requests)
        del pool, tri

    if rank == 0:
        rep = timed_reports[-1]
        out = {
            "metric": METRIC, "value": mixed_sps, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_mixed / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Q diag(s) Q^T, built on the device)",
            "config": {"workload": f"single SPD solve n={n} nrhs={m} kappa=1e6",
                       "path": f"mixed: equilibrated low-precision Cholesky ({args.update} trailing "
                               f"updates) + FP64 refinement ({args.residual} residual), FP64 fallback",
                       "l2": "inputs larger than L2 (A = %.2f GB)" % (n * n * 8 / 1e9),
                       "refine_schedule": schedule,
                       "parallelism": "replicas" if world > 1 else "single"},
            "backward_error": max(r["backward_error"] for r in timed_reports),
            "latency": latency,
            "refinement": {"iterations": rep["iterations"], "backward_error0": rep["backward_error0"],
                           "fell_back": sum(r["fell_back"] for r in timed_reports),
                           "ms_factor": rep["ms_factor"], "ms_refine": rep["ms_refine"],
                           "forward_error_vs_fp64": fwd_vs_fp64},
            "plain_fp64": {"value": plain_sps, "unit": "solves/s", "steps": k_plain,
                           "ms_per_step": ms_plain / k_plain, "backward_error": be_plain,
                           "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in prof_plain.items()}},
            "mixed_over_plain": mixed_sps / plain_sps,
            "other_residual": alt,
            "gflops": flops_solve(n, m) * mixed_sps / 1e9,
            "roofline": roofline, "roofline_other_kernels": roofline_others,
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": launches,
            "kernels": {k: {"ms": v[0], "launches": v[1], "work": v[2]} for k, v in prof.items()},
            "batch": batch, "serve": serve,
        }
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def make_batch(torch, count, seed, device, dtype):
    """n log-uniform in [16, 256], A = G G^T / n + 0.1 I (G from a per-system
    seed), 1..8 right-hand sides uniform."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(16), np.log(256), count)).round().astype(np.int32)
    n = np.clip(n, 16, 256)
    m = rng.integers(1, 9, count).astype(np.int32)
    g = torch.Generator(device=device)
    As, Bs = [], []
    for i in range(count):
        g.manual_seed(seed * 100003 + i)
        G = torch.randn(int(n[i]), int(n[i]), dtype=torch.float64, device=device, generator=g)
        As.append((G @ G.T / int(n[i]) + 0.1 * torch.eye(int(n[i]), dtype=torch.float64,
                                                          device=device)).to(dtype))
        Bs.append(torch.randn(int(n[i]), int(m[i]), dtype=torch.float64, device=device,
                              generator=g).to(dtype))
    return n, m, As, Bs


def batch_backward_errors(torch, plan, n, m, As, Bs, dX, dt):
    """Normwise backward error / (n eps) of EVERY system of the batch, computed
    here in FP64 from the caller's copies of A_i and B_i."""
    eps = float(torch.finfo(dt).eps)
    vals = []
    for i in range(len(n)):
        x = dX[plan.b_off[i]:plan.b_off[i] + n[i] * m[i]].reshape(int(m[i]), int(n[i])).T.double()
        a, b = As[i].double(), Bs[i].double()
        r = b - a @ x
        be = (r.abs().amax(0) / (a.abs().sum(1).amax() * x.abs().amax(0) + b.abs().amax(0))).amax()
        vals.append(be / (float(n[i]) * eps))
    return float(torch.stack(vals).max())


def measure_batch(torch, lla, dev, count, dtname, steps, warmup, cpu_sample=0, refined=False):
    """The batched configuration: `count` systems, n log-uniform in [16, 256],
    A = G G^T / n + 0.1 I, 1..8 RHS; one persistent launch replayed from a CUDA
    graph per step (pools restored outside the events; pools > L2).  refined:
    f64 systems through an FP32 factorisation with per-system FP64 refinement."""
    dt = torch.float64 if dtname == "f64" else torch.float32
    n, m, As, Bs = make_batch(torch, count, SEED, dev, dt)
    plan = lla.BatchPlan(n, m, dtname)
    if refined:
        plan.set_refined(True)
    A0 = torch.zeros(plan.a_elems, dtype=dt, device=dev)
    B0 = torch.zeros(plan.b_elems, dtype=dt, device=dev)
    for i in range(count):
        A0[plan.a_off[i]:plan.a_off[i] + n[i] * n[i]] = As[i].T.reshape(-1)
        B0[plan.b_off[i]:plan.b_off[i] + n[i] * m[i]] = Bs[i].T.reshape(-1)
    dA, dB = A0.clone(), B0.clone()
    info = torch.empty(count, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    tune_ms = plan.autotune(dA, dB, info, stream=stream)
    # correctness: every system against the per-matrix FP64 class, 10 n eps
    dA.copy_(A0)
    dB.copy_(B0)
    plan.solve_graph(dA, dB, info, stream=stream)
    torch.cuda.synchronize()
    assert int((info != -1).sum()) == 0
    worst = batch_backward_errors(torch, plan, n, m, As, Bs, dB, dt)
    assert worst <= 10.0, worst
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total = 0.0
    l0 = lla.kernel_launches()
    lla.profile_start()
    with Clocks(dev.index or 0) as clk:
        for it in range(warmup + steps):
            dA.copy_(A0)
            dB.copy_(B0)
            e0.record(stream)
            plan.solve_graph(dA, dB, info, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            if it >= warmup:
                total += e0.elapsed_time(e1)
    prof = lla.profile_stop()
    launches = lla.kernel_launches() - l0
    ms = total / steps
    # the timed replays' results are checked too (the last one)
    assert int((info != -1).sum()) == 0
    worst_timed = batch_backward_errors(torch, plan, n, m, As, Bs, dB, dt)
    assert worst_timed <= 10.0, worst_timed
    flops = plan.shape()["flops"]
    peak = lla.measure_peak_tflops(0 if dt == torch.float64 else 2)
    achieved = flops / (ms * 1e-3) / 1e12
    cpu = None
    if cpu_sample:
        from oracle import oracle as ora
        idx = np.random.default_rng(1).choice(count, size=min(count, cpu_sample), replace=False)
        fl = 0.0
        with OneCore():
            t0 = time.perf_counter()
            for i in idx:
                a = As[i].cpu().numpy().astype(np.float64 if dt == torch.float64 else np.float32)
                b = Bs[i].cpu().numpy().astype(a.dtype)
                ora.solvec_inplace(a, b)
                fl += n[i] ** 3 / 3.0 + 2.0 * n[i] ** 2 * m[i]
            tcpu = time.perf_counter() - t0
        cpu = {"value": (fl / tcpu) / flops * count, "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"oracle solvec on {len(idx)} random systems of the batch (1 pinned core), "
                         f"scaled by flops to the whole batch"}
    return {
        "metric": f"batched SPD solves/s ({count} uneven systems, n 16-256, 1-8 RHS, {dtname}"
                  f"{', FP32 factor + FP64 refinement per system' if refined else ''})",
        "path": "FP32 factorisation + per-system FP64 refinement (plain FP64 fallback)" if refined
                else f"plain {dtname} factorisation",
        "value": count / (ms * 1e-3), "unit": "solves/s", "ms_per_step": ms, "steps": steps,
        "warmup": warmup, "dtype": dtname,
        "config": {"workload": f"batch count={count} n=16..256 log-uniform m=1..8 {dtname}",
                   "launch": "one persistent kernel replayed from a CUDA graph",
                   "shape": plan.shape(), "autotune_ms": tune_ms,
                   "l2": "pools %.2f GB (> L2)" % (plan.a_elems * (8 if dt == torch.float64 else 4) / 1e9)},
        "backward_error_over_n_eps": max(worst, worst_timed),
        "checked": f"all {count} systems, FP64 residual of the caller's copies",
        "roofline": {"kernel": "batch", "bound": "fp64-tensor" if dt == torch.float64 else "fp32-fma",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak > 0 else None,
                     "peak_source": "measured live (FP64 tensor pipe / FFMA loop on all SMs)"},
        "cpu_baseline": cpu, "clocks": clk.summary(),
        "gpu_launches": launches * steps // (warmup + steps),
        "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in prof.items()},
    }


def run_batch(args):
    import torch
    import __graft_entry__
    lla = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    out = measure_batch(torch, lla, dev, args.batch_count, args.batch_dtype, args.steps, args.warmup,
                        cpu_sample=0 if args.no_cpu else 300, refined=args.batch_refined)
    out.update({"n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "data": "synthetic (seeded G G^T/n + 0.1 I)"})
    print(json.dumps(out))


def run_sweep(args):
    """Precision sweep: n=8192, 16 RHS, A = D Q diag(s) Q^T D with kappa(Q diag(s) Q^T) in
    {1e2, 1e4, 1e6, 1e8} (log-uniform spectra) and D = diag(10^U(-3,3)); every update form;
    reports iterations to converge, backward error, fallback and time."""
    import torch
    import __graft_entry__
    lla = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    n, m = 8192, 16
    g = torch.Generator(device=dev)
    g.manual_seed(SEED)
    G = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    import ctypes
    libp = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
    if os.path.exists(libp):
        ctypes.CDLL(libp, mode=ctypes.RTLD_GLOBAL)
    Q, _ = torch.linalg.qr(G)
    del G
    d = 10.0 ** (torch.rand(n, dtype=torch.float64, device=dev, generator=g) * 6 - 3)
    B = torch.randn(n, m, dtype=torch.float64, device=dev, generator=g).T.contiguous().T
    X = torch.empty_like(B.T.contiguous()).T
    rows = []
    for kappa in (1e2, 1e4, 1e6, 1e8):
        u = torch.rand(n, dtype=torch.float64, device=dev, generator=g)
        sv = torch.exp(u * np.log(kappa))
        sv[0], sv[-1] = 1.0, kappa
        A = (Q * sv) @ Q.T
        A = (A + A.T) * 0.5
        A = A * d[:, None] * d[None, :]
        for form in ("bf16", "bf16x3", "bf16x6", "fp16", "fp16x3", "fp32"):
            lla.posv_refined_device(A.T, B, X, update=form)  # warm
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rep = lla.posv_refined_device(A.T, B, X, update=form)
            torch.cuda.synchronize()
            ms = (time.perf_counter() - t0) * 1e3
            be = backward_error(torch, A, X, B)
            rows.append({"kappa": kappa, "update": form, "iterations": rep["iterations"],
                         "converged": rep["converged"], "fell_back": rep["fell_back"],
                         "factor_failed": rep["factor_failed"],
                         "backward_error0": rep["backward_error0"], "backward_error": be, "ms": ms})
    print(json.dumps({"metric": "precision sweep n=8192 nrhs=16 (iterations, fallback)",
                      "dtype": "f64", "data": "synthetic (seeded D Q diag(s) Q^T D, D = 10^U(-3,3))",
                      "rows": rows}))


def serve_pools(torch, dev, rng):
    """Distinct systems the requests draw from, built once on the device: 48 SPD
    systems with n log-uniform in [32, 4096] and kappa log-uniform in [1e1, 1e6]
    (Q diag(s) Q^T), and 12 lower factors for the triangular-solve requests with
    n log-uniform in [32, 8192]."""
    pool, tri = [], []
    for n in sorted(np.exp(rng.uniform(np.log(32), np.log(4096), 48)).astype(int)):
        kappa = float(np.exp(rng.uniform(np.log(1e1), np.log(1e6))))
        A, _ = make_system(torch, int(n), 1, kappa, int(rng.integers(1 << 30)), dev)
        pool.append({"n": int(n), "A64": A.T.contiguous().T, "A32": A.float().T.contiguous().T})
    for n in sorted(np.exp(rng.uniform(np.log(32), np.log(8192), 12)).astype(int)):
        kappa = float(np.exp(rng.uniform(np.log(1e1), np.log(1e6))))
        A, _ = make_system(torch, int(n), 1, kappa, int(rng.integers(1 << 30)), dev)
        tri.append({"n": int(n), "L": torch.linalg.cholesky(A).T.contiguous().T})
        del A
    torch.cuda.synchronize()
    return pool, tri


def normwise_be(torch, M, X, B):
    """max_j ||b_j - M x_j||_inf / (||M||_inf ||x_j||_inf + ||b_j||_inf), in FP64."""
    M, X, B = M.double(), X.double(), B.double()
    r = B - M @ X
    return float((r.abs().amax(0) / (M.abs().sum(1).amax() * X.abs().amax(0) + B.abs().amax(0))).max())


def measure_serve(torch, lla, dev, pool, tri, rng, rate, nreq):
    """One Poisson arrival stream at `rate` requests/s: 70% solves (f64 at 1e-13 or
    f32 at 1e-6, 50/50), 20% repeat right-hand sides on kept factors, 10%
    triangular solves up to n = 8192; 40 GB admission budget.  Every result is
    checked here, independently, by an FP64 residual of the caller's copies of
    its inputs."""
    import threading
    srv = lla.Server(hbm_budget_bytes=40e9)
    for i in (0, len(pool) - 1):  # warm the slots (workspace allocation) once per path
        p = pool[i]
        srv.submit(lla.REQ_SOLVE, p["A64"], torch.randn(p["n"], 1, dtype=torch.float64,
                                                         device=dev).T.contiguous().T, tag=10**9 + i)
    srv.drain()
    srv.poll()
    reqs = []
    for _ in range(nreq):
        u = rng.random()
        m = int(rng.integers(1, 9))
        if u < 0.1:
            reqs.append(("trsm", int(rng.integers(len(tri))), m, torch.float64))
        elif u < 0.3:
            reqs.append(("resolve", int(rng.integers(len(pool))), m, torch.float64))
        else:
            reqs.append(("solve", int(rng.integers(len(pool))), m,
                         torch.float64 if rng.random() < 0.5 else torch.float32))
    # inputs materialised before the clock starts; B0 keeps a copy of every input
    Bs, B0 = [], []
    for (kind, pi, m, dt) in reqs:
        nn = tri[pi]["n"] if kind == "trsm" else pool[pi]["n"]
        b = torch.randn(nn, m, dtype=dt, device=dev).T.contiguous().T
        Bs.append(b)
        B0.append(b.clone())
    gaps = rng.exponential(1.0 / rate, len(reqs))
    handles = {}
    for (kind, pi, m, dt) in reqs:  # kept factors for the repeat-RHS requests
        if kind == "resolve" and pi not in handles:
            p = pool[pi]
            srv.submit(lla.REQ_SOLVE, p["A64"], torch.randn(p["n"], 1, dtype=torch.float64,
                                                             device=dev).T.contiguous().T,
                       keep_factor=True, tag=2 * 10**9 + pi)
            handles[pi] = None
    srv.drain()
    for r in srv.poll():
        if r["user_tag"] >= 2 * 10**9:
            handles[r["user_tag"] - 2 * 10**9] = r["factor_handle"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()

    def submitter():
        nxt = t0
        for tag, ((kind, pi, m, dt), B, gap) in enumerate(zip(reqs, Bs, gaps)):
            nxt += gap
            d = nxt - time.perf_counter()
            if d > 0:
                time.sleep(d)
            if kind == "trsm":
                srv.submit(lla.REQ_TRSM, tri[pi]["L"], B, tag=tag)
            elif kind == "resolve":
                srv.submit(lla.REQ_RESOLVE, pool[pi]["A64"], B, handle=handles[pi], tag=tag)
            else:
                p = pool[pi]
                srv.submit(lla.REQ_SOLVE, p["A64"] if dt == torch.float64 else p["A32"], B,
                           tol=1e-13 if dt == torch.float64 else 1e-6, tag=tag)
    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    srv.drain(1200.0)
    res = [r for r in srv.poll() if r["user_tag"] < len(reqs)]
    stats = srv.stats()
    for h in handles.values():
        srv.release(h)
    srv.close()
    assert len(res) == len(reqs) and all(r["status"] == 0 for r in res), \
        [r for r in res if r["status"]][:3]
    lat = np.array([(r["t_done_us"] - r["t_submit_us"]) / 1e3 for r in res])
    span = (max(r["t_done_us"] for r in res) - min(r["t_submit_us"] for r in res)) / 1e6
    # independent FP64 check of EVERY result: normwise backward error of the
    # solution the server wrote, against the caller's copy of the inputs
    worst, over_tol, paths = {}, 0, {}
    for r in res:
        kind, pi, m, dt = reqs[r["user_tag"]]
        X, b0 = Bs[r["user_tag"]], B0[r["user_tag"]]
        if kind == "trsm":
            M, nn = torch.tril(tri[pi]["L"]), tri[pi]["n"]
        else:
            M, nn = (pool[pi]["A64"] if dt == torch.float64 else pool[pi]["A32"]), pool[pi]["n"]
        be = normwise_be(torch, M, X, b0)
        eps = float(torch.finfo(dt).eps)
        tol = 1e-13 if dt == torch.float64 else 1e-6
        key = f"{r['path']}:{'f64' if dt == torch.float64 else 'f32'}:{kind}"
        worst[key] = max(worst.get(key, 0.0), be)
        paths[key] = paths.get(key, 0) + 1
        over_tol += be > tol
        assert be <= max(tol, 10 * nn * eps), (key, nn, be)
    return {"arrival_rate": rate, "requests": len(res), "throughput": len(res) / span,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "peak_hbm_gb": stats["bytes_peak"] / 1e9,
            "results_by_path": paths, "worst_backward_error_by_path": worst,
            "results_over_requested_tol": int(over_tol),
            "checked": "every result: FP64 residual of the caller's input copies (normwise backward error)"}


def run_serve(args):
    """Poisson arrivals of solve requests (the serving configuration): throughput
    and p50/p99 latency (submit -> done) per arrival rate."""
    import torch
    import __graft_entry__
    lla = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(SEED)
    pool, tri = serve_pools(torch, dev, rng)
    rates = [measure_serve(torch, lla, dev, pool, tri, rng, float(r), args.serve_requests)
             for r in args.serve_rates.split(",")]
    out = {
        "metric": "serving: throughput and p50/p99 latency vs Poisson arrival rate",
        "value": rates[-1]["throughput"], "unit": "requests/s", "n_gpus": 1,
        "higher_is_better": True, "dtype": "f64+f32", "data": "synthetic",
        "config": {"workload": f"serve {args.serve_requests} requests per rate, n 32..4096 log-uniform "
                               "(triangular solves 32..8192), kappa 1e1..1e6, f64 1e-13 / f32 1e-6, "
                               "20% repeat-RHS, 10% TRSM, 40 GB budget"},
        "rates": rates,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
