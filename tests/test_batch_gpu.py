"""GPU parity of the batched executor (one captured CUDA graph for many
queries) against the plain per-query calls of the same operators."""
import numpy as np
import pytest
import torch

from query_on_opencl_fpga_gb300 import batch as qb

pytestmark = pytest.mark.gpu


def _rows(t):
    a = [x.cpu().numpy() for x in (t if isinstance(t, tuple) else (t,))]
    if len(a) == 1:
        return a[0].reshape(-1, 2).astype(np.int64)
    return np.stack([x.astype(np.int64) for x in a], 1)


def _same(op, got, exp):
    g, e = _rows(got), _rows(exp)
    assert g.shape == e.shape
    if op == qb.OP_FILTER:  # stable: input order on both paths
        assert np.array_equal(g, e)
        return
    if op == qb.OP_JOIN:  # sorted by unsigned key on both paths; equal keys in any order
        k = (g[:, 0] & 0xFFFFFFFF)
        assert (k[1:] >= k[:-1]).all()
    gs = g[np.lexsort(g.T[::-1])]
    es = e[np.lexsort(e.T[::-1])]
    assert np.array_equal(gs, es)


@pytest.mark.parametrize("persistent", [True, False])
@pytest.mark.parametrize("autotune", [False, True])
def test_batch_matches_plain_calls(ctx, autotune, persistent):
    qs = qb.mixed_queries(24, seed=7, lo=4096, hi=1 << 18)
    plain = qb.run_plain(ctx, qs)
    b = qb.Batch(qs, autotune=autotune, persistent=persistent)
    try:
        for _ in range(2):  # replays give the same results
            for q in qs:
                q["count"].fill_(-1)
            b.run()
            b.check()
            for q, got, exp in zip(qs, qb.batch_results(qs), plain):
                _same(q["op"], got, exp)
        info = b.info()
        assert info["replay_us"] > 0
        if persistent:  # one persistent launch for the filters and group-bys; the joins beside it
            assert info["hot_slots_log2"] in (13, 14) and info["graph_nodes"] < len(qs) * 5
        else:
            assert info["graph_nodes"] > len(qs) and info["hot_slots_log2"] in (12, 13)
        assert info["join_table_factor"] in (2, 4)
    finally:
        b.close()


def test_batch_variants_are_bit_identical(ctx):
    qs = qb.mixed_queries(12, seed=11, lo=4096, hi=1 << 17, ops=(qb.OP_FILTER, qb.OP_GROUPBY, qb.OP_FUSED))
    plain = qb.run_plain(ctx, qs)
    for q in qs:
        q["variant"] = 1  # filter: bulk-copy ring; group-by: global table
    b = qb.Batch(qs, autotune=False, persistent=False)  # variants are the lanes form's
    try:
        b.run()
        b.check()
        for q, got, exp in zip(qs, qb.batch_results(qs), plain):
            _same(q["op"], got, exp)
    finally:
        b.close()


def test_batch_join_over_capacity_reports_error(ctx):
    from query_on_opencl_fpga_gb300._lib import QGError

    qs = qb.mixed_queries(1, seed=3, lo=8192, hi=8193, ops=(qb.OP_JOIN,))
    qs[0]["cap"] = 10  # far fewer than the matches
    with pytest.raises(QGError) as e:
        qb.Batch(qs, autotune=False)
    assert e.value.status == 3  # QG_ERR_CAPACITY, seen by the eager run
    # the context of ordinary calls is unaffected
    ctx.check(ctx.lib.qg_ctx_check(ctx.handle), "qg_ctx_check")


@pytest.mark.parametrize("persistent", [True, False])
@pytest.mark.parametrize("lanes", [1, 3, 16])
def test_batch_lanes_match_plain_calls(ctx, lanes, persistent):
    # The queries spread over `lanes` streams, each with a private context, in
    # one fork/join graph (persistent form: lane 0 runs the persistent kernel,
    # the joins the others): the same results whatever the number of lanes.
    qs = qb.mixed_queries(20, seed=13, lo=4096, hi=1 << 18)
    plain = qb.run_plain(ctx, qs)
    lib = ctx.lib
    assert lib.qg_batch_set_lanes(lanes) == 0
    try:
        b = qb.Batch(qs, autotune=False, persistent=persistent)
        try:
            b.run()
            b.check()
            for q, got, exp in zip(qs, qb.batch_results(qs), plain):
                _same(q["op"], got, exp)
        finally:
            b.close()
    finally:
        lib.qg_batch_set_lanes(8)
    assert lib.qg_batch_set_lanes(0) != 0 and lib.qg_batch_set_lanes(17) != 0


def test_batch_queries_match_oracle(ctx, orc):
    # Every query of a batch holding all four operators, checked against the
    # CPU oracle: the filter in input order, group-by and fused as groups by
    # key, the join as a key-sorted multiset.
    qs = qb.mixed_queries(16, seed=23, lo=4096, hi=1 << 17)
    assert {q["op"] for q in qs} == {qb.OP_FILTER, qb.OP_GROUPBY, qb.OP_FUSED, qb.OP_JOIN}
    for persistent in (False, True):
        _check_batch_against_oracle(qs, orc, persistent)


def _check_batch_against_oracle(qs, orc, persistent):
    b = qb.Batch(qs, autotune=False, persistent=persistent)
    try:
        b.run()
        b.check()
        for q, got in zip(qs, qb.batch_results(qs)):
            i = [t.cpu().numpy() for t in q["inp"]]
            if q["op"] == qb.OP_FILTER:
                exp = orc.filter_cols(i[0], i[1], q["lo"], q["hi"])
                assert np.array_equal(got.cpu().numpy(), exp)
            elif q["op"] in (qb.OP_GROUPBY, qb.OP_FUSED):
                v2 = i[2] if q["op"] == qb.OP_FUSED else None
                ek, es, ec = orc.groupby_cols(i[0], i[1], v2, q["lo"], q["hi"])
                gk, gs, gc = [t.cpu().numpy() for t in got]
                o = np.argsort(gk.view(np.uint32), kind="stable")
                assert np.array_equal(gk[o], ek) and np.array_equal(gs[o], es) and np.array_equal(gc[o], ec)
            else:
                exp = orc.join_filter_sort(i[0], i[1], i[2], i[3], q["lo"], q["hi"], cap=q["cap"])
                _same(q["op"], got, tuple(torch.from_numpy(x) for x in exp))
    finally:
        b.close()


def _query(op, key, val, val2=None, lo=0, hi=0, cap=None):
    n = key.size
    q = {"op": op, "n": n, "variant": -1, "lo": lo, "hi": hi, "count": torch.zeros(1, dtype=torch.int64, device="cuda")}
    if op == qb.OP_FILTER:
        q.update(inp=[torch.from_numpy(key).cuda(), torch.from_numpy(val).cuda()], n2=0, cap=n if cap is None else cap)
        q["out"] = [torch.empty((max(q["cap"], 1), 2), dtype=torch.int32, device="cuda")]
    else:
        w = val2 if val2 is not None else np.zeros_like(key)
        q.update(inp=[torch.from_numpy(key).cuda(), torch.from_numpy(val).cuda(), torch.from_numpy(w).cuda()],
                 n2=0, cap=n if cap is None else cap)
        q["out"] = [torch.empty(max(q["cap"], 1), dtype=t, device="cuda") for t in (torch.int32, torch.int64,
                                                                                      torch.int64)]
    return q


def test_batch_persistent_edge_cases(ctx, orc):
    # The persistent kernel's tiles and tails: 1 to 5 rows, a ragged last
    # tile, key -1 (the shared table's empty mark, which goes to the L2 table)
    # and INT_MIN, INT_MIN/INT_MAX values (int64 sums with carries), the fused
    # predicate, a group count above the capacity (count reported, cap rows
    # written), and filters at the range bounds; two replays.
    rng = np.random.default_rng(99)
    qs = []
    for n in (1, 3, 5, 4097, 70001):
        k = rng.choice(np.array([-1, 0, 7, -(2 ** 31), 2 ** 31 - 1], np.int64), n)
        k = np.where(rng.random(n) < 0.5, k, rng.integers(0, 3000, n)).astype(np.int32)
        v = rng.choice(np.array([-(2 ** 31), 2 ** 31 - 1, -1, 0, 999], np.int64), n).astype(np.int32)
        w = rng.integers(0, 1000, n).astype(np.int32)
        qs.append(_query(qb.OP_GROUPBY, k, v))
        qs.append(_query(qb.OP_FUSED, k, v, w, -(2 ** 31), 499))
        fk = rng.integers(-(2 ** 31), 2 ** 31, n, dtype=np.int64).astype(np.int32)
        fk[0] = 100
        qs.append(_query(qb.OP_FILTER, fk, rng.integers(0, 1000, n).astype(np.int32), lo=-5, hi=2 ** 30))
    kk = np.arange(1500, dtype=np.int32)
    qs.append(_query(qb.OP_GROUPBY, kk, kk, cap=1000))  # 1500 groups, room for 1000 (table of 2048)
    b = qb.Batch(qs, autotune=False, persistent=True)
    try:
        for _ in range(2):
            for q in qs:
                q["count"].fill_(-1)
            b.run()
            b.check()
            for q in qs:
                i = [t.cpu().numpy() for t in q["inp"]]
                m = int(q["count"].item())
                if q["op"] == qb.OP_FILTER:
                    exp = orc.filter_cols(i[0], i[1], q["lo"], q["hi"])
                    assert m == exp.shape[0]
                    assert np.array_equal(q["out"][0][:m].cpu().numpy(), exp)
                    continue
                v2 = i[2] if q["op"] == qb.OP_FUSED else None
                ek, es, ec = orc.groupby_cols(i[0], i[1], v2, q["lo"], q["hi"])
                assert m == ek.size
                w = min(m, q["cap"])
                gk, gs, gc = [t[:w].cpu().numpy() for t in q["out"]]
                if w == m:
                    o = np.argsort(gk.view(np.uint32), kind="stable")
                    assert np.array_equal(gk[o], ek) and np.array_equal(gs[o], es) and np.array_equal(gc[o], ec)
                else:  # the first cap groups written are genuine groups
                    pos = np.searchsorted(ek.view(np.uint32), gk.view(np.uint32))
                    assert np.array_equal(ek[pos], gk) and np.array_equal(es[pos], gs) and np.array_equal(ec[pos], gc)
    finally:
        b.close()


def test_batch_persistent_table_overflow_reports_error(ctx):
    # More groups than the query's table holds (2 x cap rounded up to a power
    # of two): the persistent kernel records QG_ERR_TABLE_FULL, seen by the
    # batch's eager run; ordinary calls are unaffected.
    from query_on_opencl_fpga_gb300._lib import QGError

    kk = np.arange(20000, dtype=np.int32)
    with pytest.raises(QGError) as e:
        qb.Batch([_query(qb.OP_GROUPBY, kk, kk, cap=1000)], autotune=False, persistent=True)
    assert e.value.status == 4
    ctx.check(ctx.lib.qg_ctx_check(ctx.handle), "qg_ctx_check")


def test_batch_dense_window_group_bys(ctx):
    # Group-by queries whose keys fit a window run the dense-window path inside
    # the graph; a query whose keys spread over 2^30 values takes the two-pass
    # path.  Both equal the plain calls.  A replay after a dense query's keys
    # were spread as wide reports the rows it could not place instead of a
    # wrong result.
    from query_on_opencl_fpga_gb300._lib import QGError

    qs = qb.mixed_queries(8, seed=21, lo=1 << 16, hi=1 << 18, ops=(qb.OP_GROUPBY, qb.OP_FUSED))
    qs[0]["inp"][0].mul_(1024)  # keys over [0, 2^30): no window holds them
    plain = qb.run_plain(ctx, qs)
    b = qb.Batch(qs, autotune=False)
    try:
        for q in qs:
            q["count"].fill_(-1)
        b.run()
        b.check()
        for q, got, exp in zip(qs, qb.batch_results(qs), plain):
            _same(q["op"], got, exp)
        qs[1]["inp"][0].mul_(1024)
        b.run()
        with pytest.raises(QGError) as ei:
            b.check()
        assert ei.value.status == 7  # QG_ERR_UNSUPPORTED
    finally:
        b.close()
