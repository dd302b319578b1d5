"""Torch-tensor front end over the C ABI (include/qg.h).

Device memory and streams come from PyTorch; every operator runs in libqg.so.
Records are int32 tensors of shape (n, 2) holding the reference's uint2
{x, y} (y = key, x = payload / row id; host/host/common.h:27-28).
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_int, c_int64, c_void_p

import torch

from . import _lib
from ._lib import QGError, QG_ERR_CAPACITY, QG_ORDER_KEY, QG_ORDER_NONE

INT32_MIN = -(2 ** 31)
INT32_MAX = 2 ** 31 - 1


def _ptr(t: torch.Tensor | None) -> c_void_p:
    if t is None:
        return c_void_p(0)
    return c_void_p(t.data_ptr())


def _check_dev(*ts: torch.Tensor | None) -> None:
    for t in ts:
        if t is None:
            continue
        if not t.is_cuda:
            raise ValueError("operator inputs must be CUDA tensors")
        if not t.is_contiguous():
            raise ValueError("operator inputs must be contiguous")


class Context:
    """A qg_ctx bound to a CUDA stream (default: torch's current stream)."""

    def __init__(self, stream: torch.cuda.Stream | None = None):
        self.lib = _lib.load()
        self.stream = stream or torch.cuda.current_stream()
        h = c_void_p()
        st = self.lib.qg_ctx_create(byref(h), c_void_p(self.stream.cuda_stream))
        if st != 0:
            raise QGError(st, "qg_ctx_create")
        self.handle = h

    def close(self) -> None:
        self.release_out_buffers()
        if getattr(self, "handle", None):
            self.lib.qg_ctx_destroy(self.handle)
            self.handle = None

    def release_out_buffers(self) -> None:
        """Forget the output buffer sets remembered by groupby_cols(out=...)."""
        self.__dict__.pop("_gb_out", None)

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def check(self, st: int, where: str) -> None:
        if st != 0:
            msg = self.lib.qg_last_error_message(self.handle).decode(errors="replace")
            raise QGError(st, where, msg)

    @property
    def launches(self) -> int:
        return int(self.lib.qg_ctx_launch_count(self.handle))

    def enable_timing(self, on: bool = True) -> None:
        """Bracket every kernel launch with CUDA events on this context's stream."""
        self.check(self.lib.qg_ctx_enable_timing(self.handle, int(on)), "qg_ctx_enable_timing")

    def timing_report(self) -> dict[str, tuple[int, float]]:
        """{kernel name: (launches, total ms)} since the last report; clears the log."""
        buf = ctypes.create_string_buffer(1 << 16)
        k = self.lib.qg_ctx_timing_report(self.handle, buf, len(buf))
        if k < 0:
            raise QGError(2, "qg_ctx_timing_report")
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt, ms = line.split()
            out[name] = (int(cnt), float(ms))
        return out

    def timing_span(self) -> float:
        """Device ms from the first logged launch's start to the last one's end (-1: none)."""
        return float(self.lib.qg_ctx_timing_span(self.handle))

    # ---- learned cost model (qg_mlp.cu) ----------------------------------
    def mlp_init(self, seed: int = 0) -> torch.Tensor:
        p = torch.empty(int(self.lib.qg_mlp_param_count()), dtype=torch.float32, device="cuda")
        self.check(self.lib.qg_mlp_init(self.handle, _ptr(p), seed & 0xFFFFFFFF), "qg_mlp_init")
        return p

    def mlp_predict(self, params: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
        _check_dev(params, X)
        out = torch.empty(X.shape[0], dtype=torch.float32, device=X.device)
        self.check(self.lib.qg_mlp_predict(self.handle, _ptr(params), _ptr(X), X.shape[0], _ptr(out)),
                   "qg_mlp_predict")
        return out

    def mlp_grad(self, params: torch.Tensor, X: torch.Tensor, y: torch.Tensor):
        """(loss, gradient) of mean((f(X) - y)^2), computed by the GPU kernels."""
        _check_dev(params, X, y)
        g = torch.empty_like(params)
        loss = torch.empty(1, dtype=torch.float32, device=X.device)
        self.check(self.lib.qg_mlp_grad(self.handle, _ptr(params), _ptr(X), _ptr(y), X.shape[0], _ptr(g),
                                        _ptr(loss)), "qg_mlp_grad")
        return float(loss.item()), g

    def mlp_train(self, params: torch.Tensor, X: torch.Tensor, y: torch.Tensor, steps: int, lr: float,
                  opt: torch.Tensor | None = None, t: list | None = None) -> float:
        """Full-batch Adam steps on the GPU; returns the last step's loss."""
        _check_dev(params, X, y)
        if opt is None:
            opt = torch.zeros(3 * params.numel(), dtype=torch.float32, device=params.device)
        tt = ctypes.c_int(t[0] if t else 0)
        loss = torch.empty(1, dtype=torch.float32, device=X.device)
        self.check(self.lib.qg_mlp_train(self.handle, _ptr(params), _ptr(X), _ptr(y), X.shape[0], steps, lr,
                                         _ptr(opt), byref(tt), _ptr(loss)), "qg_mlp_train")
        if t is not None:
            t[0] = tt.value
        return float(loss.item())

    def set_spin_limit(self, polls: int) -> None:
        self.check(self.lib.qg_ctx_set_spin_limit(self.handle, polls), "qg_ctx_set_spin_limit")

    def sync(self) -> None:
        self.check(self.lib.qg_ctx_sync(self.handle), "qg_ctx_sync")

    def device_check(self) -> None:
        self.check(self.lib.qg_ctx_check(self.handle), "qg_ctx_check")

    # ---- filter ---------------------------------------------------------
    def filter_range_rec(self, rec: torch.Tensor, lo: int, hi: int, cap: int | None = None):
        """Stable selection of records with lo <= (int)y <= hi (filterImpl)."""
        _check_dev(rec)
        n = rec.shape[0]
        cap = n if cap is None else cap
        out = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=rec.device)
        cnt = c_int64()
        st = self.lib.qg_filter_range_rec(self.handle, _ptr(rec), n, lo, hi, _ptr(out), cap, byref(cnt))
        self.check(st, "qg_filter_range_rec")
        return out[: cnt.value]

    def filter_cols(self, key: torch.Tensor, pay: torch.Tensor, lo: int, hi: int,
                    cap: int | None = None, out: torch.Tensor | None = None):
        """Rows with lo <= key <= hi as int32 (row_id, payload) pairs, input order.

        out: optional contiguous CUDA int32 tensor of shape (>= cap, 2) to
        write into instead of allocating; the result is a view of it."""
        _check_dev(key, pay)
        n = key.numel()
        cap = n if cap is None else cap
        if out is None:
            out = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=key.device)
        elif (out.dtype != torch.int32 or not out.is_cuda or not out.is_contiguous() or out.dim() != 2
              or out.shape[1] != 2 or out.shape[0] < max(cap, 1)):
            raise ValueError("out: contiguous CUDA int32 tensor of shape (>= cap, 2)")
        cnt = c_int64()
        st = self.lib.qg_filter_cols(self.handle, _ptr(key), _ptr(pay), n, lo, hi, _ptr(out), cap,
                                     byref(cnt))
        self.check(st, "qg_filter_cols")
        return out[: cnt.value]

    # ---- scan / sort ------------------------------------------------------
    def scan_excl(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        _check_dev(x)
        out = torch.empty_like(x) if out is None else out
        self.check(self.lib.qg_scan_excl_i32(self.handle, _ptr(x), _ptr(out), x.numel()), "qg_scan_excl_i32")
        return out

    def sort_rec(self, rec: torch.Tensor) -> torch.Tensor:
        """In-place ascending sort of records by unsigned y."""
        _check_dev(rec)
        self.check(self.lib.qg_sort_rec_by_y(self.handle, _ptr(rec), rec.shape[0]), "qg_sort_rec_by_y")
        return rec

    # ---- group-by ---------------------------------------------------------
    def groupby_rec(self, rec: torch.Tensor, sorted_out: torch.Tensor | None = None):
        """Sort by key, return (sorted records, startPos[numGroups])."""
        _check_dev(rec)
        n = rec.shape[0]
        sorted_out = torch.empty_like(rec) if sorted_out is None else sorted_out
        sp = torch.empty(max(n, 1), dtype=torch.int32, device=rec.device)
        g = c_int64()
        st = self.lib.qg_groupby_rec(self.handle, _ptr(rec), n, _ptr(sorted_out), _ptr(sp), n, byref(g))
        self.check(st, "qg_groupby_rec")
        return sorted_out, sp[: g.value]

    def aggregate_groups(self, sorted_rec: torch.Tensor, start_pos: torch.Tensor, op: int):
        _check_dev(sorted_rec, start_pos)
        g = start_pos.numel()
        agg = torch.empty(max(g, 1), dtype=torch.int32, device=sorted_rec.device)
        st = self.lib.qg_aggregate_groups(self.handle, _ptr(sorted_rec), sorted_rec.shape[0],
                                          _ptr(start_pos), g, op, _ptr(agg))
        self.check(st, "qg_aggregate_groups")
        return agg[:g]

    def groupby_cols(self, key, val, val2=None, lo2: int = INT32_MIN, hi2: int = INT32_MAX,
                     cap: int = 1 << 20, order: int = QG_ORDER_KEY, out=None):
        """Per-group (key, SUM(val) int64, COUNT int64), optionally only rows with lo2<=val2<=hi2.

        out: optional (key int32, sum int64, count int64) CUDA tensors of at
        least `cap` elements to write into instead of allocating; the returned
        tensors are views of them.  The context remembers its last 4 such sets
        (validated pointers and result views, so they stay allocated) until
        release_out_buffers() or close()."""
        _check_dev(key, val, val2)
        n = key.numel()
        if out is None:
            dev = key.device
            gk = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
            gs = torch.empty(max(cap, 1), dtype=torch.int64, device=dev)
            gc = torch.empty(max(cap, 1), dtype=torch.int64, device=dev)
            ent = None
            ptrs = (_ptr(gk), _ptr(gs), _ptr(gc))
        else:
            gk, gs, gc = out
            ent = self._out_entry(out, cap)
            ptrs = ent[2]
        g = c_int64()
        st = self.lib.qg_groupby_cols(self.handle, _ptr(key), _ptr(val), _ptr(val2), lo2, hi2, n,
                                      ptrs[0], ptrs[1], ptrs[2], cap, order, byref(g))
        self.check(st, "qg_groupby_cols")
        m = g.value
        if ent is not None:
            # the same output buffers and group count as a recent call: the
            # views made then are the result (they alias the buffers anyway)
            views = ent[3].get(m)
            if views is None:
                views = (gk[:m], gs[:m], gc[:m])
                if len(ent[3]) >= 4:
                    ent[3].clear()
                ent[3][m] = views
            return views
        return gk[:m], gs[:m], gc[:m]

    def _out_entry(self, out, cap):
        """Validated (key, sum, count) output buffers, remembered for the last
        few buffer sets: (tensors, data pointers, c_void_p pointers, views by count)."""
        cache = self.__dict__.setdefault("_gb_out", [])
        dptr = tuple(t.data_ptr() for t in out)
        for ent in cache:
            if (ent[0][0] is out[0] and ent[0][1] is out[1] and ent[0][2] is out[2] and ent[1] == dptr
                    and all(t.numel() >= max(cap, 1) for t in out)):
                return ent
        for t, dt in zip(out, (torch.int32, torch.int64, torch.int64)):
            if t.dtype != dt or not t.is_cuda or not t.is_contiguous() or t.numel() < max(cap, 1):
                raise ValueError("out: contiguous CUDA (int32, int64, int64) tensors of at least cap elements")
        ent = (tuple(out), dptr, tuple(c_void_p(p) for p in dptr), {})
        cache.insert(0, ent)
        del cache[4:]
        return ent

    def groupby_stats(self) -> dict:
        """Path and spill diagnostics of the last groupby_cols call."""
        out = (ctypes.c_uint32 * 4)()
        self.check(self.lib.qg_groupby_stats(self.handle, out), "qg_groupby_stats")
        path = {0: "two_pass", 1: "global_table", 2: "dense"}[out[0]]
        return {"path": path, "flags": out[1], "fullest_bucket": out[2], "bucket_cap": out[3]}

    # ---- join ---------------------------------------------------------------
    def join_filter_sort(self, rkey, rpay, skey, spay, slo: int = INT32_MIN, shi: int = INT32_MAX,
                         cap: int | None = None):
        """(key, R.payload, S.payload) of R join S on key, S filtered on payload, sorted by key."""
        _check_dev(rkey, rpay, skey, spay)
        nR, nS = rkey.numel(), skey.numel()
        dev = skey.device
        if cap is None:
            cap = nS
        while True:
            ok = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
            orp = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
            osp = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
            m = c_int64()
            st = self.lib.qg_join_filter_sort(self.handle, _ptr(rkey), _ptr(rpay), nR, _ptr(skey),
                                              _ptr(spay), nS, slo, shi, _ptr(ok), _ptr(orp), _ptr(osp),
                                              cap, byref(m))
            if st == QG_ERR_CAPACITY and m.value > cap:
                cap = m.value
                continue
            self.check(st, "qg_join_filter_sort")
            return ok[: m.value], orp[: m.value], osp[: m.value]

    def reduce_rec(self, rec: torch.Tensor, op: int) -> int:
        """SUM / MAX / MIN / AVERAGE (QG_REDUCE_*) of Record.y, unsigned 32-bit as the reference checks it."""
        _check_dev(rec)
        r = ctypes.c_uint32()
        self.check(self.lib.qg_reduce_rec(self.handle, _ptr(rec), rec.shape[0], op, byref(r)), "qg_reduce_rec")
        return r.value

    def split_rec(self, rec: torch.Tensor, parts: int):
        """(records grouped by y mod parts, stable; int32 start of each partition)."""
        _check_dev(rec)
        out = torch.empty_like(rec)
        bound = torch.empty(parts, dtype=torch.int32, device=rec.device)
        self.check(self.lib.qg_split_rec(self.handle, _ptr(rec), rec.shape[0], parts, _ptr(out), _ptr(bound)),
                   "qg_split_rec")
        return out, bound

    def join_set_knobs(self, variant: int = 0, buckets_log2: int = 0, bucket_s_max: int = 0,
                       bucket_r_max: int = 0):
        """Join algorithm: 0 auto, 1 radix partitions, 2 learned partitions, 3 hash + sort."""
        self.check(self.lib.qg_join_set_knobs(variant, buckets_log2, bucket_s_max, bucket_r_max),
                   "qg_join_set_knobs")

    def groupby_set_single_launch(self, enable: bool):
        """Dense-window group-by as one cooperative launch or four launches (default); results are identical."""
        self.check(self.lib.qg_groupby_set_single_launch(1 if enable else 0), "qg_groupby_set_single_launch")

    def join_set_dense(self, enable: bool = True):
        """Dense build side (unique R keys over a dense span) on or off; results are identical."""
        self.check(self.lib.qg_join_set_dense(1 if enable else 0), "qg_join_set_dense")

    def join_stats(self) -> dict:
        """Path and partition diagnostics of the last join_filter_sort call."""
        out = (ctypes.c_uint32 * 8)()
        self.check(self.lib.qg_join_stats(self.handle, out), "qg_join_stats")
        names = {0: "none", 1: "radix", 2: "learned", 3: "hash_sort", 4: "dense"}
        return {"path": names.get(out[0], str(out[0])), "buckets": out[1], "outside_buckets": out[2],
                "outside_rows": out[3], "merge_buckets": out[4], "knots": out[5], "heavy_keys": out[6],
                "auto_switched": out[7]}

    def part_learn(self, keys: torch.Tensor, nbuckets: int) -> torch.Tensor:
        """Fit the learned partition function on int32/uint32 keys; returns the device model."""
        _check_dev(keys)
        model = torch.empty(int(self.lib.qg_part_model_bytes()), dtype=torch.uint8, device=keys.device)
        self.check(self.lib.qg_part_learn(self.handle, _ptr(keys), keys.numel(), nbuckets, _ptr(model)),
                   "qg_part_learn")
        return model

    def part_eval(self, keys: torch.Tensor, model: torch.Tensor | None = None, kmin: int = 0,
                  shift: int = 0) -> torch.Tensor:
        """Bucket of each key under the learned model, or radix (key - kmin) >> shift."""
        _check_dev(keys)
        out = torch.empty(keys.numel(), dtype=torch.int32, device=keys.device)
        mp = _ptr(model) if model is not None else None
        self.check(self.lib.qg_part_eval(self.handle, mp, kmin & 0xFFFFFFFF, shift, _ptr(keys), keys.numel(),
                                         _ptr(out)), "qg_part_eval")
        return out

    def hash_join_ref(self, r_pairs: torch.Tensor, s_pairs: torch.Tensor, cap: int | None = None):
        """Reference-layout join: (key, val) pairs in, (S.val, R.val) pairs out."""
        _check_dev(r_pairs, s_pairs)
        nR, nS = r_pairs.shape[0], s_pairs.shape[0]
        cap = nS if cap is None else cap
        while True:
            out = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=s_pairs.device)
            m = c_int64()
            st = self.lib.qg_hash_join_ref(self.handle, _ptr(r_pairs), nR, _ptr(s_pairs), nS,
                                           _ptr(out), cap, byref(m))
            if st == QG_ERR_CAPACITY and m.value > cap:
                cap = m.value
                continue
            self.check(st, "qg_hash_join_ref")
            return out[: m.value]

    # ---- the learned cost model steering the engine ------------------------
    def steer_attach(self, params: torch.Tensor, tolerance: float = 0.25):
        """Let the context's operator calls run the variants the model (device
        params from costmodel.train) predicts fastest, judged against the
        plain variant when a call is slower than (1 + tolerance) x predicted."""
        _check_dev(params)
        self.check(self.lib.qg_steer_attach(self.handle, _ptr(params), tolerance), "qg_steer_attach")

    def steer_detach(self):
        self.check(self.lib.qg_steer_detach(self.handle), "qg_steer_detach")

    def steer_choose(self, op: int, n: int, n2: int = 0, sel: float = 1.0):
        """(variant, predicted ms) the context would run for operator op (0 filter,
        1 group-by, 2 fused, 3 join)."""
        v = c_int()
        ms = ctypes.c_float()
        self.check(self.lib.qg_steer_choose(self.handle, op, n, n2, sel, byref(v), byref(ms)), "qg_steer_choose")
        return v.value, ms.value

    def steer_stats(self, op: int) -> dict:
        out = (c_int64 * 10)()
        self.check(self.lib.qg_steer_stats(self.handle, op, out), "qg_steer_stats")
        keys = ("calls", "model_calls", "default_calls", "trials", "fallbacks", "confirmed", "last_variant",
                "last_us", "last_pred_us", "cells_nondefault")
        return dict(zip(keys, list(out)))

    def steer_plan(self, sub_index: int, size_m: float):
        """(plan, operator variant) of the DP over the model's cost table."""
        from ._lib import Plan

        p = Plan()
        v = c_int()
        self.check(self.lib.qg_steer_plan(self.handle, sub_index, size_m, byref(p), byref(v)), "qg_steer_plan")
        return p, v.value

    def hash_build_ref(self, r_pairs: torch.Tensor) -> torch.Tensor:
        """Build the reference-layout hash table of R's (key, val) pairs into a
        new device buffer (qg_hash_table_bytes bytes) and return it."""
        _check_dev(r_pairs)
        nR = r_pairs.shape[0]
        tb = int(self.lib.qg_hash_table_bytes(nR))
        if tb < 0:
            raise ValueError("build side too large")
        table = torch.empty(tb, dtype=torch.uint8, device=r_pairs.device)
        self.check(self.lib.qg_hash_build_ref(self.handle, _ptr(r_pairs), nR, _ptr(table), tb), "qg_hash_build_ref")
        return table

    def hash_probe_ref(self, table: torch.Tensor, s_pairs: torch.Tensor, cap: int | None = None):
        """Probe a table from hash_build_ref: (S.val, R.val) pairs of every match."""
        _check_dev(table, s_pairs)
        nS = s_pairs.shape[0]
        cap = nS if cap is None else cap
        while True:
            out = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=s_pairs.device)
            m = c_int64()
            st = self.lib.qg_hash_probe_ref(self.handle, _ptr(table), _ptr(s_pairs), nS, _ptr(out), cap, byref(m))
            if st == QG_ERR_CAPACITY and m.value > cap:
                cap = m.value
                continue
            self.check(st, "qg_hash_probe_ref")
            return out[: m.value]


__all__ = ["Context", "QGError", "QG_ORDER_KEY", "QG_ORDER_NONE", "INT32_MIN", "INT32_MAX"]
