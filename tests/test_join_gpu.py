"""GPU parity: hash join + filter + sort (keys bit-exact and nondecreasing;
rows compared as a multiset per key since the order among equal keys is
unspecified) and the reference-layout hash build/probe."""
import numpy as np
import pytest
import torch

from query_on_opencl_fpga_gb300 import datagen

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def as_sorted_rows(k, a, b):
    k, a, b = [np.asarray(x) for x in (k, a, b)]
    o = np.lexsort((b, a, k.view(np.uint32)))
    return k[o], a[o], b[o]


def check_join(got, exp):
    gk, ga, gb = [t.cpu().numpy() for t in got]
    u = gk.view(np.uint32)
    assert (u[1:] >= u[:-1]).all(), "output not sorted by key"
    g = as_sorted_rows(gk, ga, gb)
    e = as_sorted_rows(*exp)
    for x, y in zip(g, e):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("nR,nS,keyspace", [(1, 1, 1), (10, 1000, 20), (4096, 100003, 8192),
                                            (1 << 16, 1 << 20, 1 << 17), (100, 50000, 50)])
def test_join_small(ctx, orc, nR, nS, keyspace):
    rng = np.random.default_rng(nR + nS)
    rkey = rng.integers(0, keyspace, nR).astype(np.int32)   # duplicates when nR > keyspace
    rpay = rng.integers(0, 1000, nR).astype(np.int32)
    skey = rng.integers(0, keyspace * 2, nS).astype(np.int32)
    spay = rng.integers(0, 1000, nS).astype(np.int32)
    got = ctx.join_filter_sort(dev(rkey), dev(rpay), dev(skey), dev(spay), -(2 ** 31), 299)
    exp = orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 299, cap=nS * max(1, nR // keyspace + 8))
    check_join(got, exp)


def test_join_negative_and_sentinel_keys(ctx, orc):
    rkey = np.array([-1, -1, 5, -(2 ** 31), 2 ** 31 - 1, 7], np.int32)
    rpay = np.array([-1, 3, 4, 5, 6, -1], np.int32)
    skey = np.tile(rkey, 50)
    spay = np.arange(skey.size, dtype=np.int32) % 1000
    got = ctx.join_filter_sort(dev(rkey), dev(rpay), dev(skey), dev(spay))
    check_join(got, orc.join_filter_sort(rkey, rpay, skey, spay, cap=skey.size * rkey.size))


def test_join_config2_shape_medium(ctx, orc):
    d = datagen.config2_join(1 << 20, 1 << 24, seed=1)
    args = [d[k].numpy() for k in ("rkey", "rpay", "skey", "spay")]
    got = ctx.join_filter_sort(*[dev(a) for a in args], d["slo"], d["shi"])
    check_join(got, orc.join_filter_sort(*args, d["slo"], d["shi"], mt=True))


def test_join_config2_full_size(ctx):
    # Full config-2 size (R 16M, S 256M): size-independent checks --
    # sortedness, row count equal to the filtered hit count, and every row's
    # R.payload equal to R's payload for that key (R keys are a permutation).
    d = datagen.config2_join(1 << 24, 1 << 28, seed=0, device="cuda")
    ok, orp, osp = ctx.join_filter_sort(d["rkey"], d["rpay"], d["skey"], d["spay"], d["slo"], d["shi"],
                                        cap=70_000_000)
    assert ctx.join_stats()["path"] == "dense"  # R's keys are a permutation of [0, 2^24)
    m = (d["spay"] <= 299) & (d["skey"] < (1 << 24))
    assert ok.numel() == int(m.sum())
    assert bool((ok[1:] >= ok[:-1]).all())
    rmap = torch.empty(1 << 24, dtype=torch.int32, device="cuda")
    rmap[d["rkey"].long()] = d["rpay"]
    assert torch.equal(orp, rmap[ok.long()])
    # S payload multiset per key: compare sorted (key, spay) of both sides
    ks = d["skey"][m]
    ss = d["spay"][m]
    e = torch.sort(ks.long() * 1024 + ss.long()).values
    g = torch.sort(ok.long() * 1024 + osp.long()).values
    assert torch.equal(e, g)


def test_join_capacity_error(ctx):
    # 10 build rows and 1000 probe rows on one key: 10000 matches into room for 5.
    from ctypes import byref, c_int64, c_void_p

    r = torch.zeros(10, dtype=torch.int32, device="cuda")
    s = torch.zeros(1000, dtype=torch.int32, device="cuda")
    out = torch.empty(5, dtype=torch.int32, device="cuda")
    m = c_int64()
    p = lambda t: c_void_p(t.data_ptr())  # noqa: E731
    st = ctx.lib.qg_join_filter_sort(ctx.handle, p(r), p(r), 10, p(s), p(s), 1000, -(2 ** 31), 2 ** 31 - 1,
                                     p(out), p(out), p(out), 5, byref(m))
    assert st == 3 and m.value == 10000
    # the wrapper retries with the reported size
    k, a, b = ctx.join_filter_sort(r, r, s, s)
    assert k.numel() == 10000 and int(k.abs().sum()) == 0


@pytest.mark.parametrize("nR,nS,keyspace", [(1, 1, 1), (1000, 20000, 700), (1 << 16, 1 << 18, 1 << 16)])
def test_hash_join_ref(ctx, orc, nR, nS, keyspace):
    rng = np.random.default_rng(nR)
    r = np.stack([rng.integers(0, keyspace, nR), rng.integers(0, 1 << 30, nR)], 1).astype(np.int32)
    s = np.stack([rng.integers(0, keyspace, nS), rng.integers(0, 1 << 30, nS)], 1).astype(np.int32)
    got = ctx.hash_join_ref(dev(r), dev(s)).cpu().numpy()
    exp = orc.hash_join_ref(r, s, cap=nS * 8)
    assert np.array_equal(np.sort(got.view(np.int64).ravel()), np.sort(exp.view(np.int64).ravel()))


def test_hash_build_once_probe_three_batches(ctx, orc):
    # buildHashTable once, probeHashTable with three S batches (as the
    # reference's split kernels allow); each batch equals the oracle's join,
    # including duplicate build keys and the all-ones (key -1, val -1) row.
    rng = np.random.default_rng(77)
    nR = 50000
    r = np.stack([rng.integers(0, 30000, nR), rng.integers(0, 1 << 30, nR)], 1).astype(np.int32)
    r[5] = (-1, -1)
    table = ctx.hash_build_ref(dev(r))
    assert table.numel() == ctx.lib.qg_hash_table_bytes(nR)
    for b, nS in enumerate((1, 70001, 1 << 18)):
        s = np.stack([rng.integers(-10, 33000, nS), rng.integers(0, 1 << 30, nS)], 1).astype(np.int32)
        if nS > 10:
            s[7, 0] = -1
        got = ctx.hash_probe_ref(table, dev(s)).cpu().numpy()
        exp = orc.hash_join_ref(r, s, cap=nS * 8)
        assert np.array_equal(np.sort(got.view(np.int64).ravel()), np.sort(exp.view(np.int64).ravel())), b
    # a table buffer smaller than qg_hash_table_bytes is refused
    from ctypes import c_void_p

    st = ctx.lib.qg_hash_build_ref(ctx.handle, c_void_p(dev(r).data_ptr()), nR, c_void_p(table.data_ptr()),
                                   table.numel() - 8)
    assert st == 3
