#!/usr/bin/env python3
"""Benchmark of the relational-operator hot path on GB300.

Headline workload (the configuration the metric is quoted on): group-by
aggregation and fused filter_aggregation over 64M rows -- int32 key Zipf(1.0)
over 1M groups, int32 value uniform [0, 1000), SUM as int64 plus COUNT; the
fused variant keeps rows with value2 < 500.  One step = both operators over
the batch, output in key order (the reference's group-by order).  `value` is
input rows per second summed over the two operators, inputs resident in HBM;
`e2e` is the same metric through the public API with host inputs copied in
and results copied out every step.  Per-operator lines for the filter
(16M rows) and the join + filter + sort (R 16M, S 256M) are in `operators`.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With --impl reference the CPU restatement of the reference operators runs on
the host cores (all threads) over the same full step when the requested steps
fit in about five minutes (a bounded sample of it otherwise).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_ROWS = 1 << 26
GROUPS = 1 << 20
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(s[1]) for s in self.samples if num(s[1]) is not None]
        smax = [num(s[2]) for s in self.samples if num(s[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[5 + i].lower() == "active"})
        power = [num(s[3]) for s in self.samples if num(s[3]) is not None]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.samples),
                "power_w_max": max(power) if power else None}


def dist_init(n_gpus):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# reference arm: the CPU restatement of the reference operators on host cores
# ---------------------------------------------------------------------------
def cpu_groupby_step(key, val, val2):
    """One config-1 step (group-by + fused filter_aggregation) of the oracle port
    of the reference operators on all host threads."""
    from oracle import oracle as orc

    orc.groupby_cols(key, val, None, -(2 ** 31), 499, cap=GROUPS * 2, mt=True)
    orc.groupby_cols(key, val, val2, -(2 ** 31), 499, cap=GROUPS * 2, mt=True)


def run_reference(args, rank, world):
    """The full config-1 step (2 x 64M rows) when the requested steps fit in about
    7 minutes at the rate of a first (warm-up) step, else a sample sized to fit.
    The oracle's multi-threaded group-by merges its per-thread tables serially, a
    cost that does not shrink with the sample, so a sampled step under-reports
    the port's rate on the full workload: the budget keeps the default 300 steps
    (about 1 s each on 16 cores) on the full step."""
    if rank != 0:
        return
    import numpy as np

    from oracle import oracle as orc
    from query_on_opencl_fpga_gb300 import datagen

    orc.lib()
    threads = orc.threads()
    d = datagen.config1_groupby(N_ROWS, GROUPS, seed=0)
    key, val, val2 = d["key"].numpy(), d["val"].numpy(), d["val2"].numpy()
    t0 = time.perf_counter()
    cpu_groupby_step(key, val, val2)  # first warm-up step, also the rate estimate
    t_full = time.perf_counter() - t0
    budget_s = 420.0
    sample = N_ROWS
    while sample > (1 << 20) and t_full * sample / N_ROWS * (args.steps + args.warmup) > budget_s:
        sample //= 2
    if sample < N_ROWS:
        key, val, val2 = (np.ascontiguousarray(x[:sample]) for x in (key, val, val2))
    for _ in range(args.warmup - 1 if sample == N_ROWS else args.warmup):
        cpu_groupby_step(key, val, val2)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_groupby_step(key, val, val2)
    dt = (time.perf_counter() - t0) / args.steps
    value = 2 * sample / dt
    full = sample == N_ROWS
    wl = ("config1: groupby SUM(int64)+COUNT and fused filter_aggregation (value2<500), 64M rows, "
          "key Zipf(1.0) over 1M groups, output in key order")
    line = {
        "impl": "reference", "metric": "rows_per_s", "value": value, "unit": "rows/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32 in, int64 SUM/COUNT",
        "data": "synthetic (seeded)",
        "config": {"workload": wl if full else wl + f"; first {sample} rows per operator per step",
                   "rows_per_step": 2 * sample},
        "cpu_baseline": {"value": value, "unit": "rows/s", "cores": threads, "kind": "port",
                         "sample": "the full step (2 x 64M rows)" if full else
                         f"{sample} rows x 2 operators per step (the 64M-row batch, sampled to fit the run)"},
        "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference OpenCL CPU runtime unavailable on this box; oracle port of the reference "
                "operators (oracle/qg_oracle.c, OpenMP) on all host threads",
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def timed(ctx, fn, steps, warmup, world, stream):
    """(ms per step, {kernel: (launches, total ms)}, launches per run of `steps`).

    The timed region runs the steps alone.  The per-kernel durations come from
    the same number of steps right after it, with a CUDA event pair on the
    context's stream around every launch: those events cost about 40 us per
    headline step, so they stay out of the step time."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    launches0 = ctx.launches
    barrier(world)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        fn()
    end.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = start.elapsed_time(end) / steps
    launches = ctx.launches - launches0
    ctx.timing_report()  # drop anything logged before
    ctx.enable_timing(True)
    for _ in range(steps):
        fn()
    torch.cuda.synchronize()
    kern = ctx.timing_report()
    ctx.enable_timing(False)
    return ms, kern, launches


def roofline(kern, name, bytes_per_launch, peak_gbs, traffic=None):
    cnt, tot = kern.get(name, (0, 0.0))
    if cnt == 0:
        return None
    avg_ms = tot / cnt
    achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
            "frac": achieved / peak_gbs, "traffic": traffic, "avg_launch_ms": avg_ms,
            "algorithmic_bytes_per_launch": bytes_per_launch}


def cpu_baseline_groupby(reps=2):
    """The oracle port on all host threads over the full headline step: the
    reference arm's own code (`--impl reference`, 3 warm-up + `reps` timed steps)
    in a fresh process, so that both CPU figures are taken the same way.  Run
    inside this process, beside the GPU run's threads and pinned buffers, the
    same steps measured about half the rate."""
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    out = subprocess.run([sys.executable, str(Path(__file__).resolve()), "--impl", "reference",
                          "--steps", str(reps), "--warmup", "3"], capture_output=True, text=True, env=env,
                         timeout=900)
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    if out.returncode != 0 or not lines:
        raise RuntimeError(f"cpu baseline run failed (rc {out.returncode}): {out.stderr[-500:]}")
    ref = json.loads(lines[-1])
    cb = dict(ref["cpu_baseline"])
    cb["sample"] = cb["sample"] + f", 3 warm-up + {reps} timed steps (a separate process running --impl reference)"
    return cb


def pinned_copy_rates(hkey, hval, hval2, dev, copy_streams, reps=5):
    """The link's plain host-to-device rate for the step's three input columns
    from pinned memory (GB/s, best of reps): all three on one stream, and one
    per copy stream at once (the e2e step's pattern)."""
    import torch

    host = (hkey, hval, hval2)
    nbytes = sum(h.numel() * h.element_size() for h in host)
    out = {}
    for name, streams in (("one_stream", [copy_streams[0]] * 3), ("three_streams", copy_streams)):
        best = float("inf")
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for cs, d, h in zip(streams, dev, host):
                with torch.cuda.stream(cs):
                    d.copy_(h, non_blocking=True)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        out[name] = nbytes / best / 1e9
    return out


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    from query_on_opencl_fpga_gb300 import datagen
    from query_on_opencl_fpga_gb300.api import QG_ORDER_KEY, QG_ORDER_NONE, Context

    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    peaks, peak_kind = load_peaks()
    peak = float(peaks["hbm_gbs"])
    ctx = Context(stream)
    if args.gb_launches:
        ctx.groupby_set_single_launch(args.gb_launches == 1)

    d = datagen.config1_groupby(N_ROWS, GROUPS, seed=rank, device="cuda")
    key, val, val2, lo2, hi2 = d["key"], d["val"], d["val2"], d["lo2"], d["hi2"]
    # output capacity: the key domain (Zipf ranks over GROUPS keys), which is
    # also what sizes the group-by's spill partitions (~1024 groups each)
    cap = GROUPS

    # one set of output columns per operator, reused by every step (as a caller
    # that owns its result buffers would; no allocation inside the step)
    outs = [tuple(torch.empty(cap, dtype=dt, device="cuda") for dt in (torch.int32, torch.int64, torch.int64))
            for _ in range(2)]

    def step():
        ctx.groupby_cols(key, val, None, lo2, hi2, cap=cap, order=QG_ORDER_KEY, out=outs[0])
        ctx.groupby_cols(key, val, val2, lo2, hi2, cap=cap, order=QG_ORDER_KEY, out=outs[1])

    clocks = ClockSampler(local)
    clocks.start()
    ms, kern, launches = timed(ctx, step, args.steps, args.warmup, world, stream)
    clocks.stop()
    ms = max_over_ranks(ms, world)
    rows_per_step = 2 * N_ROWS
    value = rows_per_step * world / (ms * 1e-3)

    # dominant kernel: the dense group-by's main pass (plain or fused, whichever
    # takes longer in total); its algorithmic bytes are the input columns it reads.
    names = {"k_gbd_main": N_ROWS * 8, "k_gbd_main_fused": N_ROWS * 12}
    dom = max(names, key=lambda n: kern.get(n, (0, 0.0))[1])
    roof = roofline(kern, dom, names[dom], peak)
    traffic_path = ROOT / "profiles" / "traffic.json"
    if roof and traffic_path.exists():
        roof["traffic"] = json.loads(traffic_path.read_text()).get(dom)
    roof_other = {n: roofline(kern, n, b, peak) for n, b in names.items()}
    kern_avg = {k: {"launches": c, "avg_ms": t / c} for k, (c, t) in kern.items() if c}

    # e2e through the public API: every step copies its inputs from pinned
    # host memory and reads its results back into pinned host memory.  The
    # input copies run on a second stream into two alternating device
    # buffers, so that step i+1's inputs arrive while step i computes (how a
    # pipelined caller uses the API); the timed region holds all of it.
    hkey = key.cpu().pin_memory()
    hval = val.cpu().pin_memory()
    hval2 = val2.cpu().pin_memory()
    dev_in = [(torch.empty_like(key), torch.empty_like(val), torch.empty_like(val2)) for _ in range(2)]
    copy_streams = [torch.cuda.Stream() for _ in range(3)]  # one per column: several copy engines at once
    ready = [[torch.cuda.Event() for _ in range(3)] for _ in range(2)]
    free = [torch.cuda.Event(), torch.cuda.Event()]
    hres = [[torch.empty(cap, dtype=dt).pin_memory() for dt in (torch.int32, torch.int64, torch.int64)]
            for _ in range(2)]

    def load(slot):
        for cs, ev, d, h in zip(copy_streams, ready[slot], dev_in[slot], (hkey, hval, hval2)):
            with torch.cuda.stream(cs):
                cs.wait_event(free[slot])  # the slot's previous step has finished with it
                d.copy_(h, non_blocking=True)
                ev.record(cs)

    def e2e_run(k):
        nb = 0
        load(0)
        for i in range(k):
            s = i % 2
            if i + 1 < k:
                load(1 - s)
            for ev in ready[s]:
                stream.wait_event(ev)
            dk, dv, dv2 = dev_in[s]
            r1 = ctx.groupby_cols(dk, dv, None, lo2, hi2, cap=cap, order=QG_ORDER_KEY, out=outs[0])
            r2 = ctx.groupby_cols(dk, dv, dv2, lo2, hi2, cap=cap, order=QG_ORDER_KEY, out=outs[1])
            free[s].record(stream)
            for r, hb in zip((r1, r2), hres):
                for t, h in zip(r, hb):
                    h[: t.numel()].copy_(t, non_blocking=True)
                    nb += t.numel() * t.element_size()
        torch.cuda.synchronize()
        return nb // k

    # Enough steps that the pipeline's fill and drain (one input copy before
    # the first step, the last step's compute and read-back after the last
    # copy, about 5 ms together) weigh little against the steady state.
    e2e_steps = max(3, min(args.steps, 40))
    e2e_run(2)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    d2h = e2e_run(e2e_steps)
    barrier(world)
    e2e_ms = max_over_ranks((time.perf_counter() - t0) / e2e_steps * 1e3, world)
    e2e = {"value": rows_per_step * world / (e2e_ms * 1e-3), "unit": "rows/s",
           "h2d_bytes_per_step": 3 * N_ROWS * 4, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
           "h2d_pinned_gbs": pinned_copy_rates(hkey, hval, hval2, dev_in[0], copy_streams),
           "note": "inputs copied from pinned host memory on copy streams (one per column; the next step's "
                   "copies overlap this step's compute); results copied to pinned host memory"}

    ops = {}
    if not args.no_operators and rank == 0:
        ops = operator_lines(ctx, args, peak, stream)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_groupby()

    if rank == 0:
        line = {
            "metric": "rows_per_s", "value": value, "unit": "rows/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32 in, int64 SUM/COUNT", "data": "synthetic (seeded)",
            "config": {"workload": "config1: groupby SUM(int64)+COUNT and fused filter_aggregation "
                                   "(value2<500), 64M rows, key Zipf(1.0) over 1M groups, output in key order",
                       "rows_per_step": rows_per_step, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs 768 MB per step > 129 MB L2 (no flush needed)"},
            "roofline": roof, "roofline_kernels": roof_other, "peak_kind": peak_kind,
            "kernels": kern_avg,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks.summary(),
            "operators": ops,
        }
        print(json.dumps(line), flush=True)
    ctx.close()


def operator_lines(ctx, args, peak, stream):
    """Per-operator rows/s and roofline: filter, group-by, join and sort configurations."""
    import torch

    from query_on_opencl_fpga_gb300 import datagen
    from query_on_opencl_fpga_gb300.api import QG_ORDER_NONE

    out = {}
    steps = max(3, min(args.steps, 10))
    # config 0: filter 16M rows
    f = datagen.config0_filter(1 << 24, seed=0, device="cuda")
    n = f["key"].numel()
    res = {}

    fout = torch.empty((n, 2), dtype=torch.int32, device="cuda")  # caller-owned output, reused

    def fstep():
        res["o"] = ctx.filter_cols(f["key"], f["payload"], f["lo"], f["hi"], out=fout)

    ms, kern, _ = timed(ctx, fstep, steps, 3, 1, stream)
    sel = res["o"].shape[0]
    # The default column filter is two kernels (count, then write): its
    # roofline is the operator's algorithmic bytes over their summed launch times.
    fk = [k for k in ("k_filter_count", "k_filter_write", "k_filter_cols") if kern.get(k, (0, 0.0))[0]]
    f_ms = sum(kern[k][1] / kern[k][0] for k in fk)
    f_alg = n * 8 + sel * 8
    out["filter_config0"] = {"rows_per_s": n / (ms * 1e-3), "ms_per_op": ms, "rows": n, "selected": sel,
                             "roofline": {"bound": "hbm", "kernel": "+".join(fk),
                                          "achieved": f_alg / (f_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                                          "frac": f_alg / (f_ms * 1e-3) / 1e9 / peak, "traffic": None,
                                          "avg_launch_ms": f_ms, "algorithmic_bytes_per_launch": f_alg}}
    del f, res, fout
    # config 1 unordered variants
    d = datagen.config1_groupby(N_ROWS, GROUPS, seed=0, device="cuda")

    def gstep():
        ctx.groupby_cols(d["key"], d["val"], None, d["lo2"], d["hi2"], cap=GROUPS, order=QG_ORDER_NONE)

    ms, kern, _ = timed(ctx, gstep, steps, 3, 1, stream)
    out["groupby_config1_unordered"] = {"rows_per_s": N_ROWS / (ms * 1e-3), "ms_per_op": ms,
                                        "op_frac_of_peak": (N_ROWS * 8 + GROUPS * 20) / (ms * 1e-3) / 1e9 / peak,
                                        "path": ctx.groupby_stats()["path"],
                                        "roofline": roofline(kern, "k_gbd_main", N_ROWS * 8, peak)}

    def fgstep():
        ctx.groupby_cols(d["key"], d["val"], d["val2"], d["lo2"], d["hi2"], cap=GROUPS, order=QG_ORDER_NONE)

    ms, kern, _ = timed(ctx, fgstep, steps, 3, 1, stream)
    out["filter_groupby_config1_unordered"] = {
        "rows_per_s": N_ROWS / (ms * 1e-3), "ms_per_op": ms,
        "op_frac_of_peak": (N_ROWS * 12 + GROUPS * 20) / (ms * 1e-3) / 1e9 / peak,
        "path": ctx.groupby_stats()["path"],
        "roofline": roofline(kern, "k_gbd_main_fused", N_ROWS * 12, peak)}
    del d
    torch.cuda.empty_cache()
    # config 2: join + filter + sort
    j = datagen.config2_join(1 << 24, 1 << 28, seed=0, device="cuda")
    res = {}

    def jstep():
        res["o"] = ctx.join_filter_sort(j["rkey"], j["rpay"], j["skey"], j["spay"], j["slo"], j["shi"],
                                        cap=70_000_000)

    ms, kern, _ = timed(ctx, jstep, steps, 2, 1, stream)
    m = res["o"][0].numel()
    nR, nS = 1 << 24, 1 << 28
    alg = nR * 8 + nS * 8 + m * 12 + 2 * m * 12
    sp = int((j["spay"] <= 299).logical_and(j["skey"] < nR).sum())  # S' rows the S filter keeps
    out["join_config2"] = {"rows_per_s": nS / (ms * 1e-3), "ms_per_op": ms, "out_rows": m,
                           "op_frac_of_peak": alg / (ms * 1e-3) / 1e9 / peak,
                           "kernels_ms": {k: v[1] / steps for k, v in kern.items()},
                           "path": ctx.join_stats()["path"],
                           "roofline_sfilter": roofline(kern, "k_pj_sfilter", nS * 8 + sp * 8, peak)}
    del j, res
    torch.cuda.empty_cache()
    out["sort_64M"] = sort_line(ctx, steps, peak, stream)
    torch.cuda.empty_cache()
    if not args.no_learned:
        out["skew_join_config4"] = skew_line(ctx, stream)
        torch.cuda.empty_cache()
        out["batched_config3"] = batched_line(ctx, stream)
        torch.cuda.empty_cache()
    return out


def sort_line(ctx, steps, peak, stream):
    """In-place sort of 64M reference Records by unsigned y (radixSortImpl_sm),
    keys uniform in [0, 2^20): three 8-bit passes.  Every step sorts a fresh
    copy of the same unsorted records; the copy is outside the timed call."""
    import torch

    from query_on_opencl_fpga_gb300.datagen import records, uniform_i32

    ns = 1 << 26
    base = records(uniform_i32(ns, 0, 1 << 20, 0, "cuda"))
    rec = torch.empty_like(base)
    for _ in range(2):
        rec.copy_(base)
        ctx.sort_rec(rec)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for e0, e1 in ev:
        rec.copy_(base)
        e0.record(stream)
        ctx.sort_rec(rec)
        e1.record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    keys = rec[:, 1]
    ok = bool((keys[1:] >= keys[:-1]).all()) and int(keys.sum()) == int(base[:, 1].sum())
    ctx.timing_report()
    ctx.enable_timing(True)
    for _ in range(steps):
        rec.copy_(base)
        ctx.sort_rec(rec)
    torch.cuda.synchronize()
    kern = ctx.timing_report()
    ctx.enable_timing(False)
    passes = kern.get("k_radix_pass", (0, 0.0))[0] // steps
    alg = ns * 16 * passes  # one read and one write of the records per key pass
    del base, rec
    return {"rows_per_s": ns / (ms * 1e-3), "ms_per_op": ms, "rows": ns, "passes": passes, "sorted": ok,
            "op_frac_of_peak": alg / (ms * 1e-3) / 1e9 / peak,
            "kernels_ms": {k: v[1] / steps for k, v in kern.items()},
            "roofline": roofline(kern, "k_radix_pass", ns * 16, peak)}


def skew_line(ctx, stream):
    """Config 4: skewed join.  Plain radix partitioning (variant 1) against the
    learned partition function (variant 2), and against the engine steered by
    the learned cost model (trained on the recorded cost log, attached to the
    context: the library picks the join variant itself, judged against the
    plain one)."""
    import json as _json

    import torch

    from query_on_opencl_fpga_gb300 import costmodel, datagen

    nR, nS = 1 << 25, 1 << 28
    j = datagen.config4_skewed(nR, nS, seed=0, device="cuda")

    def step():
        ctx.join_filter_sort(j["rkey"], j["rpay"], j["skey"], j["spay"], j["slo"], j["shi"],
                             cap=int(nS * 0.3) + 1024)

    def timed_ms():
        step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / 2 * 1e3

    res = {}
    for name, v in (("radix", 1), ("learned", 2)):
        ctx.join_set_knobs(v)
        ms = timed_ms()
        res[name] = {"ms_per_op": ms, "rows_per_s": (nR + nS) / (ms * 1e-3), **ctx.join_stats()}
    ctx.join_set_knobs(0)
    recs = _json.loads((ROOT / "tests" / "golden" / "costlog.json").read_text())["records"]
    params, _ = costmodel.train(ctx, recs)
    ctx.steer_attach(params)
    try:
        ms = timed_ms()
        st = ctx.steer_stats(3)
        res["steered"] = {"ms_per_op": ms, "rows_per_s": (nR + nS) / (ms * 1e-3), **ctx.join_stats(),
                          "variant": st["last_variant"], "predicted_ms": st["last_pred_us"] / 1e3,
                          "judge": {k: st[k] for k in ("calls", "model_calls", "trials", "fallbacks")}}
    finally:
        ctx.steer_detach()
    res["learned_over_radix"] = res["radix"]["ms_per_op"] / res["learned"]["ms_per_op"]
    res["steered_over_radix"] = res["radix"]["ms_per_op"] / res["steered"]["ms_per_op"]
    res["workload"] = ("config4: R 32M distinct keys and S 256M keys from 8 Gaussians (sigma 2^20) + 5% "
                       "Zipf(1.2) heavy hitters, S.payload < 300, output sorted by key")
    return res


def batched_line(ctx, stream):
    """Config 3: 512 mixed queries: plain per-query calls, against the batch
    as one captured graph in its persistent form (filters and group-bys in one
    persistent kernel launch, the joins beside it) and in its lanes form
    (every query's own launches; variants chosen by the learned cost model);
    wall time, inputs on the GPU."""
    import json as _json

    import torch

    from query_on_opencl_fpga_gb300 import batch as qb
    from query_on_opencl_fpga_gb300 import costmodel

    qs = qb.mixed_queries(512, seed=0)
    rows = qb.input_rows(qs)
    qb.run_plain(ctx, qs)  # warm-up (arena sizes)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    qb.run_plain(ctx, qs)
    torch.cuda.synchronize()
    plain_ms = (time.perf_counter() - t0) * 1e3
    recs = _json.loads((ROOT / "tests" / "golden" / "costlog.json").read_text())["records"]
    params, _ = costmodel.train(ctx, recs)
    qb.choose_variants(ctx, params, qs)  # chosen by the library from the attached model
    ctx.steer_detach()

    def timed_batch(persistent):
        b = qb.Batch(qs, autotune=True, persistent=persistent)
        b.run()
        b.check()
        t0 = time.perf_counter()
        for _ in range(3):
            b.run()
        b.check()
        ms = (time.perf_counter() - t0) / 3 * 1e3
        info = b.info()
        b.close()
        return {"ms": ms, "rows_per_s": rows / (ms * 1e-3), **info}

    pers = timed_batch(True)
    lanes = timed_batch(False)
    nops = {qb.OP_NAMES[o]: sum(1 for q in qs if q["op"] == o) for o in qb.OP_NAMES}
    return {"queries": len(qs), "ops": nops, "input_rows": rows,
            "plain": {"ms": plain_ms, "rows_per_s": rows / (plain_ms * 1e-3)},
            "persistent": pers, "lanes_graph": lanes,
            "batched_over_plain": plain_ms / min(pers["ms"], lanes["ms"]),
            "persistent_over_plain": plain_ms / pers["ms"], "lanes_over_plain": plain_ms / lanes["ms"],
            "workload": "config3: 512 queries, op uniform over filter/groupby/fused/join, rows log-uniform "
                        "in [4096, 16M], config 0-2 distributions, seeds 0..511"}


def run_only(args):
    """One operator alone (for profiler captures): W warm-up + K timed calls."""
    import torch

    from query_on_opencl_fpga_gb300 import datagen
    from query_on_opencl_fpga_gb300.api import QG_ORDER_NONE, Context

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    ctx = Context(stream)
    rows = args.rows
    if args.only in ("groupby", "fused"):
        n = rows or N_ROWS
        d = datagen.config1_groupby(n, GROUPS, seed=0, device="cuda")
        v2 = d["val2"] if args.only == "fused" else None
        fn = lambda: ctx.groupby_cols(d["key"], d["val"], v2, d["lo2"], d["hi2"], cap=GROUPS,  # noqa: E731
                                      order=QG_ORDER_NONE)
    elif args.only == "filter":
        n = rows or (1 << 24)
        f = datagen.config0_filter(n, seed=0, device="cuda")
        fout = torch.empty((n, 2), dtype=torch.int32, device="cuda")
        fn = lambda: ctx.filter_cols(f["key"], f["payload"], f["lo"], f["hi"], out=fout)  # noqa: E731
    elif args.only == "join":
        n = rows or (1 << 28)
        nr = args.rows2 or min(1 << 24, max(n // 16, 1))
        j = datagen.config2_join(nr, n, seed=0, device="cuda")
        fn = lambda: ctx.join_filter_sort(j["rkey"], j["rpay"], j["skey"], j["spay"], j["slo"],  # noqa: E731
                                          j["shi"], cap=int(n * 0.26) + 1024)
    elif args.only == "skew":
        n = rows or (1 << 28)
        nr = args.rows2 or min(1 << 25, max(n // 8, 1))
        j = datagen.config4_skewed(nr, n, seed=0, device="cuda")
        ctx.join_set_knobs(max(args.variant, 0))
        fn = lambda: ctx.join_filter_sort(j["rkey"], j["rpay"], j["skey"], j["spay"], j["slo"],  # noqa: E731
                                          j["shi"], cap=int(n * 0.3) + 1024)
    elif args.only == "batched":
        print(json.dumps({"only": "batched", **batched_line(ctx, stream)}), flush=True)
        ctx.close()
        return
    elif args.only == "sort":
        n = rows or (1 << 26)
        from query_on_opencl_fpga_gb300.datagen import records, uniform_i32

        # every call sorts a fresh copy of the unsorted records (re-sorting the
        # sorted output would favour the ranking); ms_per_op includes that
        # copy, kernels_ms_per_op does not
        base = records(uniform_i32(n, 0, 1 << 20, 0, "cuda"))
        rec = torch.empty_like(base)

        def fn():
            rec.copy_(base)
            ctx.sort_rec(rec)
    else:
        raise SystemExit(f"unknown --only {args.only}")
    if args.variant >= 0 and args.only == "filter":
        ctx.check(ctx.lib.qg_filter_set_variant(args.variant), "qg_filter_set_variant")
    if args.variant >= 0 and args.only in ("groupby", "fused"):
        ctx.check(ctx.lib.qg_groupby_set_knobs(args.variant, 13, 0, 0), "qg_groupby_set_knobs")
    if args.variant >= 0 and args.only == "sort":
        ctx.check(ctx.lib.qg_sort_set_rank(args.variant), "qg_sort_set_rank")
    if args.gb_launches:
        ctx.groupby_set_single_launch(args.gb_launches == 1)
    ms, kern, launches = timed(ctx, fn, args.steps, args.warmup, 1, stream)
    extra = {"groupby_stats": ctx.groupby_stats()} if args.only in ("groupby", "fused") else {}
    if args.only in ("join", "skew"):
        extra = {"join_stats": ctx.join_stats()}
    print(json.dumps({"only": args.only, "rows": n, "variant": args.variant, "ms_per_op": ms,
                      "rows_per_s": n / (ms * 1e-3),
                      "kernels_ms_per_op": {k: v[1] / args.steps for k, v in kern.items()},
                      "gpu_launches": launches, **extra}), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None, help="groupby|fused|filter|join|skew|sort|batched: one operator alone")
    ap.add_argument("--rows", type=int, default=0, help="row count for --only (default: the config size)")
    ap.add_argument("--variant", type=int, default=-1,
                    help="--only filter: kernel variant; groupby/fused: knob mode; sort: ranking form (0, 3, 4)")
    ap.add_argument("--rows2", type=int, default=0, help="build-side rows for --only join")
    ap.add_argument("--gb-launches", type=int, default=0, choices=[0, 1, 4],
                    help="group-by: the dense-window steps as one cooperative launch (1) or four (4); 0: the library default")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-operators", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the config 3 / config 4 lines")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.only:
        run_only(args)
        return
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        run_reference(args, rank, int(os.environ.get("WORLD_SIZE", "1")))
        return
    rank, world, local = dist_init(args.gpus)
    run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
