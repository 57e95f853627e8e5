"""Benchmark: MI estimates/s at N=1e6, k=3 on one GB300.

Workload (one "step" = one batch through the C ABI): the large-sample
precision configuration -- four bivariate Gaussian KSG MI estimates with
rho in {0, 0.3, 0.6, 0.9} and one Frenzel-Pompe conditional MI of a 3-D
Gaussian (corr(x,y)=0.5, corr(x,z)=corr(y,z)=0.4), all float64, N=1,000,000,
k=3, seeded synthetic data (no dataset involved).

Arms:
  default          this library: batched FP32 tiles + FP64 recheck.
                   `value`   = estimates/s with inputs resident in HBM
                               (device-pointer batch), CUDA events per step;
                   `e2e`     = the same through the C ABI with host buffers
                               (H2D of the inputs and D2H of the results timed);
                   `plain`   = the all-FP64 comparator, one task per call;
                   `cpu_baseline` = the reference algorithm (SciPy cKDTree,
                               oracle/ref_port.py) on a bounded query sample.
  --impl reference the reference's CPU path (cKDTree calls of
                   ennemi/_entropy_estimators.py, oracle/ref_port.py) with all
                   host threads, each step a bounded sample of the workload.

L2 (129 MB) is flushed between timed steps by writing a 512 MB buffer,
outside the timed events.  Under torchrun each rank runs its own replica of
the batch (tasks are independent; no collective on the data path) and rank 0
prints the aggregate.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MI estimates/s, N=1e6 k=3: batched FP32+recheck vs plain GPU; counts bit-exact"
UNIT = "MI estimates/s"


def make_workload(n: int, seed: int = 0):
    """[(kind, [columns])] -- kind 'mi' (x, y) or 'cmi' (x, y, z)."""
    from ennemi_gb300 import synthetic
    return synthetic.large_sample(n, seed)


def make_tasks(work, k, cols_of=lambda c: c):
    from ennemi_gb300 import _native as N
    tasks = []
    for kind, cols in work:
        cs = [cols_of(c) for c in cols]
        n = len(cols[0])
        if kind == "mi":
            tasks.append(N.Task(N.MI, k, [cs[0]], [cs[1]], n=n))
        else:
            tasks.append(N.Task(N.CMI, k, [cs[0]], [cs[1]], [cs[2]], n=n))
    return tasks


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        # raw samples (the JSON line carries their summary); BENCH_CLOCKS_DIR
        # keeps them somewhere else
        out = os.environ.get("BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out, f"clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[4:]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for name, flag in zip(names, r[3][1:]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows),
                "reasons": sorted(reasons)}


def flush_l2(buf):
    buf.add_(1.0)


def timed_steps(run, steps, torch, flush_buf):
    """Sum of CUDA-event times of `steps` calls of run(), L2 flushed between."""
    total = 0.0
    per = []
    for _ in range(steps):
        flush_l2(flush_buf)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        run()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        per.append(ms)
        total += ms
    return total, per


def _versions():
    import scipy
    return f"numpy {np.__version__}, scipy {scipy.__version__}"


def cpu_baseline(work, k, slices, nslices, threads):
    """The reference's calls over SciPy cKDTree on a bounded sample of the
    batch: every tree built over all N points, `slices` of `nslices` query
    slices of every task searched and counted, tasks on a pool of `threads`
    workers as the reference's driver runs them; scaled to the batch."""
    from oracle import ref_port
    tasks = [(kind, tuple(cols)) for kind, cols in work]
    t0 = time.perf_counter()
    r = ref_port.sample_rate(tasks, k, slices, nslices, threads=threads)
    wall = time.perf_counter() - t0
    return {"value": len(tasks) / r["extrapolated_s"], "unit": UNIT,
            "cores": min(r["threads"], len(tasks)), "kind": "port",
            "max_threads": r["threads"],
            "sample": (f"SciPy cKDTree (the reference's calls, {_versions()}): every tree built "
                       f"over all N points, {slices} of {nslices} query slices of every task "
                       f"searched and counted, one task per worker of a {r['threads']}-thread pool "
                       f"(each task single-threaded, as the reference's driver runs them); "
                       f"time scaled to the whole batch; measured {wall:.1f} s"),
            "seconds_per_batch_extrapolated": r["extrapolated_s"]}


def config_of(args, ntask):
    """The workload, identical in both arms' lines."""
    return {"workload": "4x bivariate Gaussian KSG MI (rho 0/.3/.6/.9) + 1x 3-D Gaussian CMI "
                        "(corr .5/.4/.4), float64, seeded",
            "n": args.n, "k": args.k, "seed": args.seed, "tasks_per_step": ntask,
            "l2": "GPU arm: flushed between timed steps (512 MB write)"}


GOLDEN_HEADLINE = os.path.join(ROOT, "tests", "golden", "golden_headline.json")


def parity_check(N, dev_tasks, work, args, dev):
    """The batch once more (outside the timed region) with its internals
    kept: eps and every count array hashed and compared with the digests the
    reference produced on the same inputs (tests/golden/golden_headline.json,
    made by tests/golden/make_golden.py --headline)."""
    import hashlib
    try:
        gold = json.load(open(GOLDEN_HEADLINE))["large_sample"]
    except (OSError, ValueError, KeyError):
        return {"checked": False, "why": "no reference digests"}
    if gold["n"] != args.n or gold["k"] != args.k or gold["seed"] != args.seed:
        return {"checked": False, "why": "reference digests exist for n=1e6, k=3, seed 0 only"}

    def h(a, dt):
        return hashlib.sha256(np.ascontiguousarray(a, dtype=dt).tobytes()).hexdigest()

    inputs_same = all([h(c, "<f8") for c in cols] == g["inputs"] for (_, cols), g in zip(work, gold["tasks"]))
    vals = N.run_tasks(dev_tasks, flags=N.INPUT_DEVICE | N.KEEP_INTERNALS, device=dev)
    eps_ok, cnt_ok, dmi = True, True, 0.0
    for t, ((kind, _), g) in enumerate(zip(work, gold["tasks"])):
        eps_ok &= h(N.fetch(t, 0, args.n, device=dev), "<f8") == g["eps"]
        for s, name in enumerate(["nx", "ny"] if kind == "mi" else ["nxz", "nyz", "nz"]):
            cnt_ok &= h(N.fetch(t, 1 + s, args.n, device=dev), "<i8") == g[name]
        dmi = max(dmi, abs(float(vals[t]) - g["value"]))
    return {"checked": True, "inputs_same": bool(inputs_same), "eps_bitexact": bool(eps_ok),
            "counts_exact": bool(cnt_ok), "max_abs_dmi": dmi,
            "against": "SHA-256 of eps and counts from the reference's cKDTree calls on the same "
                       "inputs (tests/golden/golden_headline.json)"}


def run_reference(args):
    """The reference CPU arm: the whole batch, measured.

    The tasks run on a thread pool of os.cpu_count() workers, one task per
    worker and each task single-threaded, as the reference's driver runs them
    with max_threads=None (_driver.py:736-785).  Each task builds its trees
    once (timed); each of the K timed steps then searches and counts one
    contiguous 1/K slice of every task's query points, so the K steps together
    evaluate every query point of the batch exactly once.  value = tasks /
    (tree builds + sum of the steps).  The W warm-up steps run the same code
    on a 20,000-point copy of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import ref_port
    threads = os.cpu_count() or 1
    small = make_workload(20_000, args.seed)
    wb = ref_port.SlicedBatch([(kd, tuple(c)) for kd, c in small], args.k, max(args.warmup, 1), threads)
    try:
        wb.build()
        for s in range(args.warmup):
            wb.step(s)
    finally:
        wb.close()
    work = make_workload(args.n, args.seed)
    b = ref_port.SlicedBatch([(kd, tuple(c)) for kd, c in work], args.k, args.steps, threads)
    try:
        build_s = b.build()
        steps = [b.step(s) for s in range(args.steps)]
    finally:
        b.close()
    batch_s = build_s + sum(steps)
    value = len(work) / batch_s
    serial_s = sum(b.task_seconds)
    cb = {"value": value, "unit": UNIT, "cores": min(threads, len(work)), "kind": "port",
          "max_threads": threads,
          "sample": (f"the whole batch, every query point, in {args.steps} slices of every task "
                     f"(SciPy cKDTree, the reference's calls, {_versions()}); one task per worker "
                     f"of a {threads}-thread pool, each task single-threaded, as the reference's "
                     f"driver with max_threads=None"),
          "batch_s": batch_s, "tree_build_s": build_s,
          "max_threads_1_s": serial_s,
          "max_threads_1_note": "sum of the tasks' own times in this run: the reference's "
                                "max_threads=1 path runs the same tasks one after another"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * batch_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": config_of(args, len(work)),
            "step": f"1/{args.steps} of every task's query points (the steps together are one "
                    f"whole batch; tree builds timed once and included in value)",
            "estimates": b.estimates(),
            "per_step_s": steps,
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_config(args, torch, N, ctx, dev):
    """One JSON line for a batched workload: each step is the public-API
    call(s) a user makes; `value` uses the device time of the batches
    (EGB_TIMING), `e2e` the wall time of the calls (host preprocessing,
    uploads and read-back included)."""
    import ennemi_gb300 as eg
    from ennemi_gb300 import _driver, synthetic
    from ennemi_gb300 import _entropy_estimators as ee
    if args.config in ("lags", "lags_nan"):
        y, x, lags, mask = synthetic.lagged_ar(seed=args.seed + 3)
        if args.lags:  # a smaller case of the same workload (first lags only)
            lags = lags[:args.lags]
        if args.config == "lags_nan":  # uneven task lengths: NaN runs, drop_nan=True
            xn = synthetic.with_nan_runs(x)
            calls = [lambda: eg.estimate_mi(y, xn, lag=lags, mask=mask, drop_nan=True)]
        else:
            calls = [lambda: eg.estimate_mi(y, x, lag=lags, mask=mask)]
        ntask = len(lags) * x.shape[1]
        desc = ("16 coupled AR(1) series, length 200,000, estimate_mi of series 0 vs all at lags "
                f"0..{len(lags) - 1} with a ~10 % mask in runs of 1-50 (one batch)")
        if args.config == "lags_nan":
            desc += "; NaN runs of 1-50 in ~2 % of every x series, drop_nan=True (uneven N)"
    elif args.config == "pairwise":
        data, cond = synthetic.pairwise_mix(seed=args.seed + 4)
        calls = [lambda: eg.pairwise_mi(data), lambda: eg.pairwise_mi(data, cond=cond)]
        ntask = 2 * 64 * 63 // 2
        desc = ("pairwise_mi of 64 mixed columns (Gaussian, sin, Student-t 3, log-normal), "
                "N=50,000, plus the same conditional on a 2-D Gaussian (two batches)")
    else:
        cases, ent = synthetic.semidiscrete_mix(seed=args.seed + 5)
        tasks = [ee.semidiscrete_task(xc, yc, args.k) for xc, yc in cases]
        tasks.append(ee.entropy_task(ent, args.k))
        calls = [lambda: N.run_tasks(tasks, flags=_driver.run_flags, device=dev)]
        ntask = len(tasks)
        desc = ("Ross MI of x (dim 1-4, 3-component Gaussian mixtures) vs y with 2/10/25/50 "
                "Dirichlet(.5) classes + KL entropy of a 3-D mixture, N=500,000 (one batch)")

    phase_sum = {}
    work_sum = {}

    def step(flags):
        _driver.run_flags = flags
        dev_ms = 0.0
        t0 = time.perf_counter()
        phase_sum.clear()
        work_sum.clear()
        for c in calls:
            c()
            if flags & N.TIMING:
                ph = ctx.timings()
                dev_ms += ph.get("total", 0.0)
                for key, v in ph.items():
                    phase_sum[key] = phase_sum.get(key, 0.0) + v
                for key, v in ctx.stats().items():
                    work_sum[key] = work_sum.get(key, 0) + v
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1000.0, dev_ms

    def run_steps(flags, steps):
        step(flags)                                  # warm the arena
        walls, devs = [], []
        for _ in range(steps):
            w, d = step(flags)
            walls.append(w)
            devs.append(d)
        return walls, devs

    if args.profile:  # the public calls only, for a profiler's launch list
        for _ in range(max(args.warmup, 0) + args.steps):
            for c in calls:
                c()
        torch.cuda.synchronize()
        return
    old_flags = _driver.run_flags
    try:
        for _ in range(max(args.warmup - 1, 0)):
            step(0)
        with ClockSampler(dev) as clk:
            walls, _ = run_steps(0, args.steps)
        _, devs = run_steps(N.TIMING, args.steps)
        fast_phases, fast_work = dict(phase_sum), dict(work_sum)
        plain = None
        if not args.no_plain:
            _, pdevs = run_steps(N.TIMING | N.PLAIN_FP64, 1)
            plain = {"value": ntask / (pdevs[0] / 1000.0), "ms_per_step": pdevs[0],
                     "form": "all-FP64 distances, same batches"}
    finally:
        _driver.run_flags = old_flags
    ms_dev = statistics.median(devs)
    ms_wall = statistics.median(walls)
    line = {"metric": f"MI estimates/s, {args.config} workload", "value": ntask / (ms_dev / 1000.0),
            "unit": "MI estimates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_dev, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": desc, "tasks_per_step": ntask, "k": args.k,
                       "l2": "inputs re-uploaded by every call (host arrays)"},
            "e2e": {"value": ntask / (ms_wall / 1000.0), "unit": "MI estimates/s", "ms_per_step": ms_wall,
                    "host_ms_per_step": ms_wall - ms_dev},
            "phases_ms": fast_phases, "work": fast_work,
            "plain": plain,
            "speedup_vs_plain": (plain["ms_per_step"] / ms_dev) if plain else None,
            "clocks": clk.summary()}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--k", type=int, default=3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-slices", type=int, default=10,
                    help="query slices (of --cpu-nslices) timed for cpu_baseline")
    ap.add_argument("--cpu-nslices", type=int, default=50)
    ap.add_argument("--plain-steps", type=int, default=5,
                    help="timed steps of the all-FP64 comparator (median reported)")
    ap.add_argument("--profile", action="store_true", help="device-resident steps only (ncu)")
    ap.add_argument("--lags", type=int, default=0,
                    help="--config lags: the first LAGS lags only (0: all 49)")
    ap.add_argument("--config", default="large",
                    choices=["large", "lags", "lags_nan", "pairwise", "semidiscrete"],
                    help="large: the headline workload; the others time one public-API call "
                         "of the batched lag / pairwise / semidiscrete workloads")
    args = ap.parse_args()

    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()

    from ennemi_gb300 import _native as N
    ctx = N.context(dev)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    if args.config != "large":
        run_config(args, torch, N, ctx, dev)
        return

    work = make_workload(args.n, args.seed + rank)
    dcols = [[torch.from_numpy(c).cuda() for c in cols] for _, cols in work]
    dev_tasks = make_tasks([(kind, dc) for (kind, _), dc in zip(work, dcols)], args.k)
    # the end-to-end inputs live in pinned host memory (the gather kernel reads
    # them over the CPU-GPU link every step)
    pinned = []

    def to_pinned(c):
        t = torch.empty(c.shape, dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = c
        pinned.append(t)
        return t.numpy()

    host_tasks = make_tasks(work, args.k, cols_of=to_pinned)
    ntask = len(dev_tasks)
    flush_buf = torch.zeros(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step_dev():
        # device-resident columns: the batch is captured in a CUDA graph once
        # and replayed (every kernel runs every step; planning is skipped)
        N.run_tasks(dev_tasks, flags=N.INPUT_DEVICE | N.GRAPH, device=dev)

    def step_host():
        N.run_tasks(host_tasks, flags=0, device=dev)

    for _ in range(max(args.warmup, 0)):
        step_dev()
    if args.profile:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            step_dev()
        torch.cuda.synchronize()
        return

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    barrier()
    with ClockSampler(dev) as clk:
        dev_ms, per = timed_steps(step_dev, args.steps, torch, flush_buf)
    barrier()
    clocks = clk.summary()

    # end to end through the C ABI with host buffers
    for _ in range(max(1, args.warmup // 2)):
        step_host()
    barrier()
    e2e_ms, _ = timed_steps(step_host, args.steps, torch, flush_buf)
    barrier()
    h2d, d2h = ctx.transfer_bytes()

    # per-phase device times of one more step
    res = []
    N.run_tasks(dev_tasks, flags=N.INPUT_DEVICE | N.TIMING, device=dev, results_out=res)
    phases = ctx.timings()
    work_stats = ctx.stats()

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    # HBM copy bandwidth measured on the GB300s; without the file,
    # one earlier STREAM-style measurement on a GB300 (6.8 TB/s)
    hbm = peaks.get("hbm_gbs") or 6800.0
    hbm_src = "of measured (MEASURED_PEAKS.json hbm_gbs)" if peaks.get("hbm_gbs") else \
        "of fallback (6.8 TB/s, an earlier copy measurement on a GB300)"
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    max_mhz = clocks.get("sm_max_mhz") or peaks.get("sm_max_mhz") or 2070.0
    peak_ops = sms * 128 * max_mhz * 1e6

    # The dominant kernel (largest share of the step in the ncu launch list)
    # is the radix sort's pass, HBM-bound: per launch it reads and writes
    # every key (8 B) and index (4 B) of the batch's sort once.  Its time per
    # launch is the event-timed run of the batch's digit passes over their
    # number.  DRAM traffic per launch from one ncu capture of this workload
    # (cold cache, the six passes of one batch averaged): 137.6 MB read +
    # 82.5 MB written.
    keys = work_stats.get("sort_keys", 0)
    npass = work_stats.get("sort_passes", 0) or 8
    pass_ms = phases.get("sort_passes", 0.0) / npass
    pass_bytes = 24.0 * keys
    pass_gbs = pass_bytes / (pass_ms / 1000.0) / 1e9 if pass_ms > 0 else 0.0
    roofline = {"bound": "hbm", "kernel": "onesweep_pass_kernel (radix sort pass)",
                "achieved": pass_gbs, "peak": hbm, "unit": "GB/s", "frac": pass_gbs / hbm,
                "traffic": (137.61 + 82.46) * 1e6 if args.n == 1_000_000 else None,
                "traffic_unit": "bytes per launch (ncu, cold cache)",
                "algorithmic_bytes_per_launch": pass_bytes, "ms_per_launch": pass_ms,
                "launches_per_step": npass, "peak_source": hbm_src}

    # the multi-D kernels: latency- and L1-bound, far from any pipe or HBM
    # roofline; counted algorithmic operations ((2d+1) per screened
    # candidate-query pair) against the nominal FP32 lane rate, and the
    # all-pairs work of the same jobs over the screened work (an algorithmic
    # ratio, not a roofline fraction)
    knn_ms, cnt_ms = phases.get("knn_tile", 0.0), phases.get("count_tile", 0.0)
    knn_ops = work_stats.get("knn_tile_ops", 0)
    bf_ops = sum(float(args.n) ** 2 * (2 * (2 if kind == "mi" else 3) + 1) for kind, _ in work)
    kernels = {
        "wwalk_kernel (kNN, 4 x 2-D + 1 x 3-D)": {
            "ms": knn_ms, "screened_pairs": work_stats.get("knn_tile_pairs", 0),
            "achieved_gops": knn_ops / (knn_ms / 1000.0) / 1e9 if knn_ms > 0 else 0.0,
            "nominal_fp32_lane_gops": peak_ops / 1e9,
            "frac_of_nominal": (knn_ops / (knn_ms / 1000.0)) / peak_ops if knn_ms > 0 else 0.0,
            "dram_traffic_per_launch": ((114.16 + 16.75) + (40.62 + 0.03)) / 2 * 1e6
            if args.n == 1_000_000 else None,
            "algorithmic_savings": {"bruteforce_ops": bf_ops, "counted_ops": knn_ops,
                                    "ratio": bf_ops / knn_ops if knn_ops else None}},
        "wm_count_kernel (rank-space counts, 2 x 2-D)": {
            "ms": cnt_ms, "queries": 2 * args.n,
            "ns_per_query": cnt_ms * 1e6 / (2 * args.n) if cnt_ms > 0 else None,
            "dram_traffic_per_launch": (58.30 + 2.48) * 1e6 if args.n == 1_000_000 else None},
        "sorted_jobs_kernel (1-D counts)": {
            "ms": phases.get("count_1d", 0.0), "queries": sum(2 if kind == "mi" else 1
                                                              for kind, _ in work) * args.n,
            "dram_traffic_per_launch": (186.65 + 37.53) * 1e6 if args.n == 1_000_000 else None},
    }

    # sort and 1-D search passes together, on the minimal byte count of a 1-D
    # marginal: 32 N (8 N keys read, 8 N sorted keys written, 8 N eps read,
    # 8 N counts written) over the radix sort's and the 1-D counts' event
    # times -- a bound no multi-pass sort reaches (the sort moves 24 B per
    # key and pass, and sorts the grid-only columns too)
    n1d = sum(2 if kind == "mi" else 1 for kind, _ in work)
    sort_ms, c1_ms = phases.get("sort_radix", 0.0), phases.get("count_1d", 0.0)
    ss_bytes = 32.0 * args.n * n1d
    ss_gbs = ss_bytes / ((sort_ms + c1_ms) / 1000.0) / 1e9 if sort_ms + c1_ms > 0 else 0.0
    roofline_sort = {"bound": "hbm", "kernels": f"radix sort (load + {npass} single-sweep passes) + "
                                                "sorted_jobs_kernel 1-D counts",
                     "marginals_1d": n1d, "algorithmic_bytes": ss_bytes,
                     "sort_ms": sort_ms, "count_1d_ms": c1_ms,
                     "achieved": ss_gbs, "peak": hbm, "unit": "GB/s",
                     "frac": ss_gbs / hbm,
                     "peak_source": hbm_src,
                     "sorted_segments": work_stats.get("sort_segments"),
                     "sorted_keys": work_stats.get("sort_keys")}

    ms_dev = dev_ms / args.steps
    ms_e2e = e2e_ms / args.steps
    if world > 1:
        t = torch.tensor([ms_dev, ms_e2e], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_dev, ms_e2e = t.tolist()
    value = world * ntask / (ms_dev / 1000.0)
    e2e_value = world * ntask / (ms_e2e / 1000.0)

    plain = None
    if not args.no_plain:
        # the plain comparator: all-FP64 distances, one task per call; and the
        # same arithmetic batched, which splits the speed-up into its batching
        # and its FP32-screen parts
        def step_plain():
            for t in dev_tasks:
                N.run_tasks([t], flags=N.INPUT_DEVICE | N.PLAIN_FP64, device=dev)

        def step_plain_batched():
            N.run_tasks(dev_tasks, flags=N.INPUT_DEVICE | N.PLAIN_FP64, device=dev)
        psteps = max(args.plain_steps, 1)
        step_plain()
        _, p_per = timed_steps(step_plain, psteps, torch, flush_buf)
        step_plain_batched()
        _, pb_per = timed_steps(step_plain_batched, psteps, torch, flush_buf)
        p_ms, pb_ms = statistics.median(p_per), statistics.median(pb_per)
        plain = {"value": ntask / (p_ms / 1000.0), "unit": UNIT, "ms_per_step": p_ms,
                 "steps": psteps, "per_step_ms": p_per, "statistic": "median",
                 "form": "all-FP64 distances, one task per egb_run_batch call, device inputs",
                 "batched": {"value": ntask / (pb_ms / 1000.0), "ms_per_step": pb_ms,
                             "per_step_ms": pb_per,
                             "form": "all-FP64 distances, the five tasks in one batch"}}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    parity = parity_check(N, dev_tasks, work, args, dev) if rank == 0 else None

    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(work, args.k, args.cpu_slices, args.cpu_nslices, os.cpu_count())

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_dev, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": config_of(args, ntask),
        "paths": {"value": "device-resident columns, CUDA graph replay of the batch",
                  "e2e": "pinned host columns through egb_run_batch, planned every step"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e},
        "gpu_launches": work_stats.get("kernel_launches"),
        "roofline": roofline,
        "roofline_sort": roofline_sort,
        "kernels": kernels,
        "parity": parity,
        "phases_ms": phases,
        "work": work_stats,
        "estimates": [r.value for r in res],
        "clocks": clocks,
        "plain": plain,
        "speedup_vs_plain": (value / plain["value"]) if plain else None,
        "speedup_split": ({"batching": plain["ms_per_step"] / plain["batched"]["ms_per_step"],
                           "fp32_screen": plain["batched"]["ms_per_step"] / ms_dev}
                          if plain else None),
        "cpu_baseline": cpu,
        "per_step_ms": per,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
