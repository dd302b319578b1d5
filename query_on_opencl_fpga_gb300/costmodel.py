"""Learned cost model: chooses operator variants and fills the planner's cost
table from timings the engine records on this GPU.

The reference plans with a static table of per-variant unit costs for FPGA
images (host/dynamic_programming.cpp:152-167).  On the GPU each operator has
several bit-identical kernel variants whose speed depends on the input:

  filter   0 one tile per CTA with look-back, 1 persistent CTAs with a bulk-copy ring, 2 two passes (count, write)
  groupby  0 dense key window first (two-pass when it does not apply), 1 global hash table,
           2 two-pass with 64-bit shared adds, 3 two-pass shared-memory tables (carry sums)
  fused    as groupby, with the value2 predicate
  join     0 auto partition, 1 radix partition, 2 learned partition, 3 global hash table + radix sort

`collect` times every variant of a grid of workloads with the engine's own
per-launch event log (Context.timing_span); `train` fits the 16 -> 64 -> 1
MLP on the GPU with the library's forward/backward/Adam kernels (qg_mlp.cu)
to predict log(ms); `choose` picks the variant with the lowest prediction.
Without a model the engine's default variants (DEFAULT_VARIANT) are used.

The features of a record are the ones the engine can compute at call time
(csrc/qg_steer.cu, which runs the trained model inside the library): the
second size is the build rows of a join and the output capacity of a
group-by; the filter's selectivity is its predicate's share of the int32
range; the other operators are predicted at the selectivity they were
recorded with (OP_SEL).  `skew` is the workload's; the engine, which cannot
see it before the call, predicts with 0.

  python -m query_on_opencl_fpga_gb300.costmodel collect --out costlog.json
"""
from __future__ import annotations

import argparse
import json
import math
import sys

import torch

OPS = ("filter", "groupby", "fused", "join")
VARIANTS = {"filter": (0, 1, 2), "groupby": (0, 1, 2, 3), "fused": (0, 1, 2, 3), "join": (0, 1, 2, 3)}
DEFAULT_VARIANT = {"filter": 2, "groupby": 0, "fused": 0, "join": 0}
OP_SEL = {"groupby": 1.0, "fused": 0.5, "join": 0.3}
STEER_OP = {"filter": 0, "groupby": 1, "fused": 2, "join": 3}
NFEAT = 16


def range_share(lo: int, hi: int) -> float:
    """A predicate's share of the int32 range (the engine's selectivity estimate)."""
    return (hi - lo + 1) / 2 ** 32


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
            hi = int(sel * 2 ** 31) - 1  # keys uniform in [0, 2^31): `sel` of them kept
            w.append({"op": "filter", "n": 1 << lg, "n2": 0, "sel": sel, "fsel": range_share(-(2 ** 31), hi),
                      "skew": 0})
    for lg in (16, 18, 20, 22, 24):
        for g in (6, 12, 18):
            cap = 2 * (1 << g) + 1024  # the output capacity the call passes
            for skew in (0, 1):
                w.append({"op": "groupby", "n": 1 << lg, "groups": 1 << g, "n2": cap, "sel": 1.0,
                          "fsel": OP_SEL["groupby"], "skew": skew})
            w.append({"op": "fused", "n": 1 << lg, "groups": 1 << g, "n2": cap, "sel": 0.5,
                      "fsel": OP_SEL["fused"], "skew": 1})
    for lg in (16, 18, 20, 22, 24):
        for skew in (0, 1):
            w.append({"op": "join", "n": 1 << lg, "n2": max(1024, (1 << lg) // 16), "sel": 0.3,
                      "fsel": OP_SEL["join"], "skew": skew})
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
    ctx.lib.qg_groupby_set_knobs(DEFAULT_VARIANT["groupby"], 13, 0, 0)
    ctx.join_set_knobs(DEFAULT_VARIANT["join"])


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
        d = datagen.config1_groupby(n, w["groups"], 1.0 if w["skew"] else 0.0, seed=w.get("id", 0), device=device)
        v2 = d["val2"] if op == "fused" else None
        return lambda: ctx.groupby_cols(d["key"], d["val"], v2, d["lo2"], d["hi2"], cap=w["n2"],
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
    X = torch.tensor([features(r["op"], r["variant"], r["n"], r["n2"], r["fsel"], r["skew"]) for r in recs],
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
        c = choose(ctx, params, r0["op"], r0["n"], r0["n2"], r0["fsel"], r0["skew"])
        tot["chosen"] += vs[c]["ms"]
        tot["default"] += vs[DEFAULT_VARIANT[r0["op"]]]["ms"]
        tot["best"] += min(x["ms"] for x in vs.values())
    return tot


def judged_regret(ctx, params, recs: list[dict], tol: float = 0.25) -> dict:
    """Recorded totals with the library's judge in the loop (csrc/qg_steer.cu):
    a workload whose model choice is not the default and takes longer than
    (1 + tol) x its prediction gets one run of the default variant, and the
    faster of the two is kept.  `judged` is that steady state, `model` the
    model's choices alone."""
    by = {}
    for r in recs:
        by.setdefault(r["id"], {})[r["variant"]] = r
    tot = {"judged": 0.0, "model": 0.0, "default": 0.0, "best": 0.0}
    for vs in by.values():
        r0 = next(iter(vs.values()))
        op, d = r0["op"], DEFAULT_VARIANT[r0["op"]]
        p = predict_ms(ctx, params, op, VARIANTS[op], r0["n"], r0["n2"], r0["fsel"], r0["skew"])
        c = VARIANTS[op][min(range(len(p)), key=lambda i: p[i])]
        j = c
        if c != d and vs[c]["ms"] > p[VARIANTS[op].index(c)] * (1.0 + tol):
            j = d if vs[d]["ms"] < vs[c]["ms"] else c
        tot["judged"] += vs[j]["ms"]
        tot["model"] += vs[c]["ms"]
        tot["default"] += vs[d]["ms"]
        tot["best"] += min(x["ms"] for x in vs.values())
    return tot


def plan_table(ctx, params, size_m: float = 64.0, op: str = "groupby"):
    """Planner rows (include/qg_plan.h) of the model's predictions at size_m M
    rows: for each primitive of the operator, one row per variant holding
    that variant's predicted ms per M rows split over the operator's
    primitives; the scan primitives, fused into the operators' kernels, at
    zero cost.  The same table qg_steer_plan builds inside the library."""
    from . import _lib

    prims = {"filter": (3, 4), "groupby": (5, 6, 7, 8), "fused": (3, 4, 5, 6, 7, 8)}[op]
    n = int(size_m * (1 << 20))
    n2 = 0 if op == "filter" else 1 << 20
    sel = 0.1 if op == "filter" else OP_SEL[op]
    ms = predict_ms(ctx, params, op, VARIANTS[op], n, n2, sel, 0)
    rows = []
    for k in range(9):
        if k not in prims:
            rows.append(_lib.PlanVariant(b"fused_into_operator", k, 0, 0, 0, 0, 0.0, 0.0, 0.0))
            continue
        for v in VARIANTS[op]:
            rows.append(_lib.PlanVariant(f"gpu_{op}_v{v}".encode(), k, 0, 0, 0, 0, ms[v] / len(prims) / size_m,
                                         0.0, 0.0))
    return (_lib.PlanVariant * len(rows))(*rows), len(rows)


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
