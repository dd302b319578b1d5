"""Learned cost model: chooses operator variants and fills the planner's cost
table from timings the engine records on this GPU.

The reference plans with a static table of per-variant unit costs for FPGA
images (host/dynamic_programming.cpp:152-167).  On the GPU each operator has
several bit-identical kernel variants whose speed depends on the input:

  filter   0 one tile per CTA with look-back, 1 persistent CTAs with a bulk-copy ring, 2 two passes (count, write)
  groupby  0 two-pass shared-memory tables (carry sums), 1 global hash table, 2 two-pass with 64-bit shared adds
  fused    as groupby, with the value2 predicate
  join     0 auto partition, 1 radix partition, 2 learned partition, 3 global hash table + radix sort

`collect` times every variant of a grid of workloads with the engine's own
per-launch event log (Context.timing_span); `train` fits the 16 -> 64 -> 1
MLP on the GPU with the library's forward/backward/Adam kernels (qg_mlp.cu)
to predict log(ms); `choose` picks the variant with the lowest prediction.
Without a model the engine's default variants (DEFAULT_VARIANT) are used.

  python -m query_on_opencl_fpga_gb300.costmodel collect --out costlog.json
"""
from __future__ import annotations

import argparse
import json
import math
import sys

import torch

OPS = ("filter", "groupby", "fused", "join")
VARIANTS = {"filter": (0, 1, 2), "groupby": (0, 1, 2), "fused": (0, 1, 2), "join": (0, 1, 2, 3)}
DEFAULT_VARIANT = {"filter": 2, "groupby": 0, "fused": 0, "join": 0}
NFEAT = 16


def features(op: str, variant: int, n: int, n2: int = 0, sel: float = 1.0, skew: int = 0) -> list[float]:
    """The 16 plan features of one operator variant on one input.

    n: input rows (S rows for a join); n2: build rows (join) or groups
    (group-by), 0 for a filter; sel: fraction of rows the predicate keeps;
    skew: 1 for a heavy-tailed key distribution."""
    f = [0.0] * NFEAT
    f[OPS.index(op)] = 1.0
    f[4 + variant] = 1.0
    ln = math.log2(max(n, 1)) / 32.0
    l2 = math.log2(max(n2, 0) + 1) / 32.0
    f[8] = ln
    f[9] = l2
    f[10] = float(sel)
    f[11] = float(skew)
    f[12] = ln * ln
    f[13] = ln * skew
    f[14] = l2 * skew
    f[15] = 1.0
    return f


def workloads() -> list[dict]:
    """The collection grid: sizes log-spaced, uniform and skewed keys."""
    w = []
    for lg in (14, 16, 18, 20, 22, 24):
        for sel in (0.02, 0.3, 0.9):
            w.append({"op": "filter", "n": 1 << lg, "n2": 0, "sel": sel, "skew": 0})
    for lg in (16, 18, 20, 22, 24):
        for g in (6, 12, 18):
            for skew in (0, 1):
                w.append({"op": "groupby", "n": 1 << lg, "n2": 1 << g, "sel": 1.0, "skew": skew})
            w.append({"op": "fused", "n": 1 << lg, "n2": 1 << g, "sel": 0.5, "skew": 1})
    for lg in (16, 18, 20, 22, 24):
        for skew in (0, 1):
            w.append({"op": "join", "n": 1 << lg, "n2": max(1024, (1 << lg) // 16), "sel": 0.3, "skew": skew})
    for i, x in enumerate(w):
        x["id"] = i
    return w


def _set_variant(ctx, op: str, v: int) -> None:
    if op == "filter":
        ctx.check(ctx.lib.qg_filter_set_variant(v), "qg_filter_set_variant")
    elif op in ("groupby", "fused"):
        ctx.check(ctx.lib.qg_groupby_set_knobs(v, 13, 0, 0), "qg_groupby_set_knobs")
    else:
        ctx.join_set_knobs(v)


def _reset_variants(ctx) -> None:
    ctx.lib.qg_filter_set_variant(DEFAULT_VARIANT["filter"])
    ctx.lib.qg_groupby_set_knobs(0, 13, 0, 0)
    ctx.join_set_knobs(0)


def make_op(ctx, w: dict, device="cuda"):
    """A callable running workload w once through the public API."""
    from . import datagen
    from .api import QG_ORDER_NONE

    op, n = w["op"], w["n"]
    if op == "filter":
        d = datagen.config0_filter(n, seed=w.get("id", 0), device=device)
        hi = int(w["sel"] * 2 ** 31) - 1
        return lambda: ctx.filter_cols(d["key"], d["payload"], -(2 ** 31), hi)
    if op in ("groupby", "fused"):
        d = datagen.config1_groupby(n, w["n2"], 1.0 if w["skew"] else 0.0, seed=w.get("id", 0), device=device)
        v2 = d["val2"] if op == "fused" else None
        return lambda: ctx.groupby_cols(d["key"], d["val"], v2, d["lo2"], d["hi2"], cap=2 * w["n2"] + 1024,
                                        order=QG_ORDER_NONE)
    if w["skew"]:
        d = datagen.config4_skewed(w["n2"], n, seed=w.get("id", 0), device=device)
    else:
        d = datagen.config2_join(w["n2"], n, seed=w.get("id", 0), device=device)
    return lambda: ctx.join_filter_sort(d["rkey"], d["rpay"], d["skey"], d["spay"], d["slo"], d["shi"],
                                        cap=int(n * 0.35) + 1024)


def time_variant(ctx, fn, reps: int = 3) -> float:
    """Engine-recorded device span of one call (min over reps, after a warm-up)."""
    fn()
    best = float("inf")
    for _ in range(reps):
        ctx.timing_report()
        ctx.enable_timing(True)
        fn()
        span = ctx.timing_span()
        ctx.enable_timing(False)
        if span > 0:
            best = min(best, span)
    return best


def collect(ctx, ws: list[dict] | None = None) -> list[dict]:
    recs = []
    for w in ws or workloads():
        fn = make_op(ctx, w)
        for v in VARIANTS[w["op"]]:
            _set_variant(ctx, w["op"], v)
            try:
                ms = time_variant(ctx, fn, reps=3 if w["n"] <= (1 << 22) else 2)
            finally:
                _reset_variants(ctx)
            recs.append({**w, "variant": v, "ms": ms})
        del fn
        torch.cuda.empty_cache()
    return recs


def dataset(recs: list[dict], device="cuda"):
    X = torch.tensor([features(r["op"], r["variant"], r["n"], r["n2"], r["sel"], r["skew"]) for r in recs],
                     dtype=torch.float32, device=device)
    y = torch.tensor([math.log(r["ms"]) for r in recs], dtype=torch.float32, device=device)
    return X, y


def train(ctx, recs: list[dict], steps: int = 3000, lr: float = 3e-3, seed: int = 0):
    """Fit the cost model on the GPU; returns (params, final loss)."""
    X, y = dataset(recs)
    params = ctx.mlp_init(seed)
    opt = torch.zeros(3 * params.numel(), dtype=torch.float32, device="cuda")
    t = [0]
    loss = ctx.mlp_train(params, X, y, steps, lr, opt, t)
    return params, loss


def predict_ms(ctx, params, op: str, variants, n, n2=0, sel=1.0, skew=0) -> list[float]:
    X = torch.tensor([features(op, v, n, n2, sel, skew) for v in variants], dtype=torch.float32, device="cuda")
    return [math.exp(float(x)) for x in ctx.mlp_predict(params, X).cpu()]


def choose(ctx, params, op: str, n, n2=0, sel=1.0, skew=0) -> int:
    """Variant with the lowest predicted time (the default variant without a model)."""
    if params is None:
        return DEFAULT_VARIANT[op]
    vs = VARIANTS[op]
    p = predict_ms(ctx, params, op, vs, n, n2, sel, skew)
    return vs[min(range(len(vs)), key=lambda i: p[i])]


def regret(ctx, params, recs: list[dict]) -> dict:
    """Total recorded time of the chosen variants vs the best and the default."""
    by = {}
    for r in recs:
        by.setdefault(r["id"], {})[r["variant"]] = r
    tot = {"chosen": 0.0, "default": 0.0, "best": 0.0}
    for vs in by.values():
        r0 = next(iter(vs.values()))
        c = choose(ctx, params, r0["op"], r0["n"], r0["n2"], r0["sel"], r0["skew"])
        tot["chosen"] += vs[c]["ms"]
        tot["default"] += vs[DEFAULT_VARIANT[r0["op"]]]["ms"]
        tot["best"] += min(x["ms"] for x in vs.values())
    return tot


def plan_table(ctx, params, size_m: float = 64.0):
    """Planner rows (include/qg_plan.h) whose unit costs are the model's
    predictions, in ms per million rows, of the operator implementing each
    primitive: the filter chain (scan, map, write) by the filter, the sort,
    label, group write and aggregate by the group-by.  One variant per
    primitive (the GPU has no resource model)."""
    from . import _lib

    n = int(size_m * (1 << 20))
    f_ms = min(predict_ms(ctx, params, "filter", VARIANTS["filter"], n, 0, 0.1, 0))
    g_ms = min(predict_ms(ctx, params, "groupby", VARIANTS["groupby"], n, 1 << 20, 1.0, 1))
    rows = (_lib.PlanVariant * 9)()
    share = {0: f_ms / 5, 1: f_ms / 5, 2: f_ms / 5, 3: f_ms / 5, 4: f_ms / 5,
             5: g_ms / 4, 6: g_ms / 4, 7: g_ms / 4, 8: g_ms / 4}
    for k in range(9):
        rows[k] = _lib.PlanVariant(f"gpu_k{k}".encode(), k, 0, 0, 0, 0, share[k] / size_m, 0.0, 0.0)
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["collect"])
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    from .api import Context

    ctx = Context()
    recs = collect(ctx)
    with open(a.out, "w") as f:
        json.dump({"device": torch.cuda.get_device_name(0), "records": recs}, f, indent=0)
    print(f"{len(recs)} records -> {a.out}", file=sys.stderr)


if __name__ == "__main__":
    main()
