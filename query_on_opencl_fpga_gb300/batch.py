"""Batched mixed queries: many filter / group-by / fused / join+sort queries
of uneven sizes as one captured CUDA graph (include/qg.h qg_batch_*) -- the
filter and group-by queries inside one persistent kernel launch, or every
query as its operator's launches spread over lanes -- next to the plain form
that calls the operators one by one.

The mixed workload draws each query's operator uniformly from {filter,
group-by, filter_aggregation, join+sort} and its row count log-uniformly in
[4096, 16M], with the input distributions of the single-operator workloads:
filter keys uniform with ~10 % selected, group-by keys Zipf(1.0) over 1M
groups (value2 < 500 for the fused form), join build side = rows/16 unique
keys, probe keys 80 % in the build side, S.payload < 300.
"""
from __future__ import annotations

import ctypes
import math
from ctypes import byref, c_void_p

import torch

from . import _lib, datagen
from .api import QG_ORDER_NONE, QGError

OP_FILTER, OP_GROUPBY, OP_FUSED, OP_JOIN = 0, 1, 2, 3
OP_NAMES = {OP_FILTER: "filter", OP_GROUPBY: "groupby", OP_FUSED: "fused", OP_JOIN: "join"}
GROUPS = 1 << 20


def _rows(rng: torch.Generator, lo: int, hi: int) -> int:
    u = float(torch.rand(1, generator=rng))
    return int(round(math.exp(math.log(lo) + u * (math.log(hi) - math.log(lo)))))


def mixed_queries(nq: int = 512, seed: int = 0, lo: int = 4096, hi: int = 1 << 24, device="cuda",
                  ops=(OP_FILTER, OP_GROUPBY, OP_FUSED, OP_JOIN)) -> list[dict]:
    """Inputs and output buffers of nq queries (data seeds seed..seed+nq-1)."""
    rng = torch.Generator().manual_seed(seed)
    qs = []
    for i in range(nq):
        op = ops[int(torch.randint(0, len(ops), (1,), generator=rng))]
        n = _rows(rng, lo, hi)
        s = seed + i
        q = {"op": op, "n": n, "seed": s, "variant": -1}
        if op == OP_FILTER:
            d = datagen.config0_filter(n, seed=s, device=device)
            q.update(inp=[d["key"], d["payload"]], lo=d["lo"], hi=d["hi"], n2=0, cap=n)
            q["out"] = [torch.empty((n, 2), dtype=torch.int32, device=device)]
        elif op in (OP_GROUPBY, OP_FUSED):
            d = datagen.config1_groupby(n, GROUPS, seed=s, device=device)
            cap = min(n, GROUPS)
            q.update(inp=[d["key"], d["val"], d["val2"]], lo=d["lo2"], hi=d["hi2"], n2=GROUPS, cap=cap)
            q["out"] = [torch.empty(cap, dtype=torch.int32, device=device),
                        torch.empty(cap, dtype=torch.int64, device=device),
                        torch.empty(cap, dtype=torch.int64, device=device)]
        else:
            nr = max(n // 16, 16)
            d = datagen.config2_join(nr, n, seed=s, device=device)
            cap = int(n * 0.3) + 1024
            q.update(inp=[d["rkey"], d["rpay"], d["skey"], d["spay"]], lo=d["slo"], hi=d["shi"], n2=nr, cap=cap)
            q["out"] = [torch.empty(cap, dtype=torch.int32, device=device) for _ in range(3)]
        q["count"] = torch.zeros(1, dtype=torch.int64, device=device)
        qs.append(q)
    return qs


def input_rows(qs: list[dict]) -> int:
    """Rows the queries read (a join: both sides)."""
    return sum(q["n"] + (q["n2"] if q["op"] == OP_JOIN else 0) for q in qs)


def choose_variants(ctx, params, qs: list[dict]) -> None:
    """Per-query variants chosen by the library (qg_steer_choose) from the
    learned cost model attached to ctx; joins in a graph always take the
    hash + device-planned sort form."""
    from .costmodel import range_share

    ctx.steer_attach(params)
    for q in qs:
        if q["op"] == OP_JOIN:
            q["variant"] = -1
            continue
        sel = range_share(q["lo"], q["hi"]) if q["op"] == OP_FILTER else 1.0
        n2 = 0 if q["op"] == OP_FILTER else q["cap"]
        q["variant"] = ctx.steer_choose(q["op"], q["n"], n2, sel)[0]


class Batch:
    """A captured batch (qg_batch).  Inputs and outputs must outlive it."""

    def __init__(self, queries: list[dict], autotune: bool = True, persistent: bool = False):
        """persistent: filter / group-by / fused queries in one persistent kernel
        launch (joins beside it); False (default): every query as its
        operator's launches, spread over lanes."""
        self.lib = _lib.load()
        self.queries = queries
        arr = (_lib.Query * len(queries))()
        for i, q in enumerate(queries):
            a = arr[i]
            a.op, a.variant, a.n, a.n2 = q["op"], q["variant"], q["n"], q["n2"]
            for j, t in enumerate(q["inp"]):
                a.inp[j] = t.data_ptr()
            a.lo, a.hi = q["lo"], q["hi"]
            for j, t in enumerate(q["out"]):
                a.out[j] = t.data_ptr()
            a.cap = q["cap"]
            a.d_count = q["count"].data_ptr()
        h = c_void_p()
        self.lib.qg_batch_set_persistent(int(persistent))
        try:
            st = self.lib.qg_batch_create(arr, len(queries), int(autotune), byref(h))
        finally:
            self.lib.qg_batch_set_persistent(0)
        if st != 0:
            raise QGError(st, "qg_batch_create")
        self.handle = h

    def run(self, stream=None):
        s = (stream or torch.cuda.current_stream()).cuda_stream
        st = self.lib.qg_batch_run(self.handle, c_void_p(s))
        if st != 0:
            raise QGError(st, "qg_batch_run")

    def check(self, stream=None):
        s = (stream or torch.cuda.current_stream()).cuda_stream
        st = self.lib.qg_batch_check(self.handle, c_void_p(s))
        if st != 0:
            raise QGError(st, "qg_batch_check")

    def info(self) -> dict:
        out = (ctypes.c_int32 * 4)()
        self.lib.qg_batch_info(self.handle, out)
        return {"hot_slots_log2": out[0], "join_table_factor": out[1], "replay_us": out[2], "graph_nodes": out[3]}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.qg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass


def run_plain(ctx, qs: list[dict]) -> list:
    """The plain form: one public-API call per query, default variants."""
    res = []
    for q in qs:
        i = q["inp"]
        if q["op"] == OP_FILTER:
            res.append(ctx.filter_cols(i[0], i[1], q["lo"], q["hi"], cap=q["cap"]))
        elif q["op"] in (OP_GROUPBY, OP_FUSED):
            v2 = i[2] if q["op"] == OP_FUSED else None
            res.append(ctx.groupby_cols(i[0], i[1], v2, q["lo"], q["hi"], cap=q["cap"], order=QG_ORDER_NONE))
        else:
            res.append(ctx.join_filter_sort(i[0], i[1], i[2], i[3], q["lo"], q["hi"], cap=q["cap"]))
    return res


def batch_results(qs: list[dict]) -> list:
    """The batch's outputs, trimmed to each query's count, in plain-form shape."""
    res = []
    for q in qs:
        m = int(q["count"].item())
        if q["op"] == OP_FILTER:
            res.append(q["out"][0][:m])
        else:
            res.append(tuple(t[:m] for t in q["out"]))
    return res
