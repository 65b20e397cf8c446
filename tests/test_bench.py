"""bench.py's host-side contract, checked without a GPU: the reference arm's JSON
line, and the panel-pair schedule of the low-precision factorisation from which
the roofline's trailing-matrix bytes are computed."""
import importlib.util
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def pair_schedule(n, nb=128):
    """The tensor-core update launches of one factorisation, (first row, K, narrow),
    in the order lla_lowp.cu issues them: panel p, a narrow update of the next
    128-column block, panel p + 128, one K = 256 update of the rest."""
    out, p = [], 0
    while p < n:
        b = min(nb, n - p)
        rest = n - p - b
        if rest <= 0:
            break
        if rest > nb:
            out.append((p + nb, nb, True))
            out.append((p + 2 * nb, 2 * nb, False))
            p += 2 * nb
        else:
            out.append((p + nb, nb, False))
            p += nb
    return out


def lower_elements(rows, cols):
    """Entries on or below the diagonal of the leading rows x cols block of a
    rows x rows lower triangle."""
    return sum(min(cols, i + 1) for i in range(rows))


def test_update_schedule_bytes():
    bench = load_bench()
    for n in [129, 200, 256, 257, 385, 512, 1000, 2111, 8192, 16384]:
        sched = pair_schedule(n)
        want = 0.0
        for q, _k, narrow in sched:
            rows = n - q
            want += 8.0 * lower_elements(rows, min(128, rows) if narrow else rows)
        got, launches = bench.mixed_update_bytes(n)
        assert launches == len(sched), n
        assert abs(got - want) <= 1e-9 * max(want, 1.0), (n, got, want)
    # the launch counts the library's own accounting reports per n=16384 / n=8192 solve
    assert bench.mixed_update_bytes(16384)[1] == 127
    assert bench.mixed_update_bytes(8192)[1] == 63
    # every trailing row is reached exactly once per 256 columns: 22.9 GB at n=16384
    assert abs(bench.mixed_update_bytes(16384)[0] / 1e9 - 22.907) < 1e-3


def test_reference_arm_json_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--ref-sample-n", "192"],
                       capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"].startswith("SPD solves/s") and line["unit"] == "solves/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 1 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert line["config"]["workload"].startswith("single SPD solve n=16384")
    cb = line["cpu_baseline"]
    # the reference is single-threaded: one pinned core, and the n = 16384 figure is
    # extrapolated from the directly timed sample
    assert cb["kind"] in ("port", "reference") and cb["cores"] == 1 and cb["value"] == line["value"]
    assert line["extrapolated"] is True and cb["extrapolated"] is True
    assert line["measured"]["n"] == 192 and line["measured"]["nrhs"] == 64
    assert abs(line["ms_per_step"] - 1000 * line["measured"]["seconds_median"]) < 1e-6
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def _replica_rank(rank, world, port, outdir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        bench = load_bench()
        ms = [10.0, 12.5, 11.0, 9.0][rank]  # this rank's timed region
        got = bench.max_over_ranks(dist, ms, "cpu")
        with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
            json.dump({"max_ms": got, "rate": bench.job_rate(world, 5, got)}, f)
    finally:
        dist.destroy_process_group()


def test_replicas_max_over_ranks_gloo():
    """The N > 1 bench path (replicas, one process per GPU): every rank ends with the
    slowest rank's time, and the whole-job rate counts all ranks' solves over it."""
    import socket
    import tempfile

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    outdir = tempfile.mkdtemp(prefix="lla_gloo_")
    world = 2
    mp.spawn(_replica_rank, args=(world, port, outdir), nprocs=world, join=True)
    for r in range(world):
        with open(os.path.join(outdir, f"rank{r}.json")) as f:
            d = json.load(f)
        assert d["max_ms"] == 12.5
        assert abs(d["rate"] - world * 5 / 12.5e-3) < 1e-9
    bench = load_bench()
    assert bench.max_over_ranks(None, 7.0, "cpu") == 7.0
