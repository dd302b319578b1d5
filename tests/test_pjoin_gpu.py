"""GPU parity of the join variants (radix / learned range partitions, hash +
sort) against the oracle, including the buckets that leave the shared-memory
bucket kernel (single-key cross products and recursive sub-joins), skewed
keys with heavy hitters, and the learned partition function itself."""
import numpy as np
import pytest
import torch

from query_on_opencl_fpga_gb300 import datagen

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def check_join(got, exp):
    gk, ga, gb = [t.cpu().numpy() for t in got]
    u = gk.view(np.uint32)
    assert (u[1:] >= u[:-1]).all(), "output not sorted by key"
    ek, ea, eb = [np.asarray(x) for x in exp]
    assert gk.size == ek.size
    g = np.lexsort((gb, ga, u))
    e = np.lexsort((eb, ea, ek.view(np.uint32)))
    assert np.array_equal(gk[g], ek[e])
    assert np.array_equal(ga[g], ea[e])
    assert np.array_equal(gb[g], eb[e])


@pytest.fixture
def knobs(ctx):
    yield ctx.join_set_knobs
    ctx.join_set_knobs(0, 0, 0, 0)


CASES = [
    # nR, nS, R keyspace, S keyspace (duplicates in R when nR > keyspace)
    (1, 1, 1, 1),
    (10, 1000, 20, 40),
    (4096, 100003, 8192, 16384),
    (1 << 16, 1 << 20, 1 << 17, 1 << 18),
    (100, 50000, 50, 100),
    (3000, 200000, 1 << 31, 1 << 31),  # sparse keys: wide buckets, bitonic path
]


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("nR,nS,kr,ks", CASES)
def test_join_variants(ctx, orc, knobs, variant, nR, nS, kr, ks):
    knobs(variant)
    rng = np.random.default_rng(nR * 7 + nS + variant)
    rkey = (rng.integers(0, kr, nR) - (kr // 2 if kr > 1 << 30 else 0)).astype(np.int64).astype(np.int32)
    rpay = rng.integers(0, 1000, nR).astype(np.int32)
    skey = (rng.integers(0, ks, nS) - (ks // 2 if ks > 1 << 30 else 0)).astype(np.int64).astype(np.int32)
    if ks > 1 << 30:  # make sparse keys hit R too
        pick = rng.random(nS) < 0.5
        skey[pick] = rkey[rng.integers(0, nR, int(pick.sum()))]
    spay = rng.integers(0, 1000, nS).astype(np.int32)
    got = ctx.join_filter_sort(dev(rkey), dev(rpay), dev(skey), dev(spay), -(2 ** 31), 299)
    exp = orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 299,
                               cap=nS * max(1, nR // max(1, min(kr, nR)) + 8), mt=True)
    check_join(got, exp)


@pytest.mark.parametrize("variant", [1, 2])
def test_join_outside_buckets(ctx, orc, knobs, variant):
    # Tiny bucket capacities and few buckets: most buckets leave the bucket
    # kernel -- heavy single keys become cross products, the rest take the
    # sort-merge path.
    knobs(variant, 4, 64, 32)
    rng = np.random.default_rng(5)
    base = rng.integers(0, 1 << 20, 3000)
    rkey = np.concatenate([base, np.full(5, 777), np.full(3, -5)]).astype(np.int32)
    rpay = rng.integers(0, 1000, rkey.size).astype(np.int32)
    skey = np.concatenate([rng.choice(base, 40000), np.full(3000, 777), np.full(500, -5),
                           rng.integers(0, 1 << 21, 5000)]).astype(np.int32)
    rng.shuffle(skey)
    spay = rng.integers(0, 1000, skey.size).astype(np.int32)
    got = ctx.join_filter_sort(dev(rkey), dev(rpay), dev(skey), dev(spay), -(2 ** 31), 499)
    st = ctx.join_stats()
    assert st["outside_buckets"] > 0
    exp = orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 499, cap=skey.size * 8, mt=True)
    check_join(got, exp)


@pytest.mark.parametrize("variant", [1, 2])
def test_join_sort_merge_with_duplicate_build_keys(ctx, orc, knobs, variant):
    # Every build key three times, tiny bucket capacities: the oversize buckets
    # hold several keys each (the sort-merge path) and every probe row that
    # hits matches three build rows.
    knobs(variant, 6, 256, 96)
    rng = np.random.default_rng(9)
    keys = rng.choice(1 << 22, 20000, replace=False).astype(np.int32)
    rkey = np.repeat(keys, 3)
    rng.shuffle(rkey)
    rpay = rng.integers(0, 1000, rkey.size).astype(np.int32)
    skey = np.concatenate([rng.choice(keys, 150000), rng.integers(0, 1 << 22, 20000)]).astype(np.int32)
    spay = rng.integers(0, 1000, skey.size).astype(np.int32)
    got = ctx.join_filter_sort(dev(rkey), dev(rpay), dev(skey), dev(spay), -(2 ** 31), 599, cap=skey.size * 4)
    st = ctx.join_stats()
    assert st["merge_buckets"] > 0
    exp = orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 599, cap=skey.size * 4, mt=True)
    check_join(got, exp)


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_join_skewed_mixture(ctx, orc, knobs, variant):
    knobs(variant)
    d = datagen.config4_skewed(1 << 17, 1 << 21, seed=3)
    args = [d[k].numpy() for k in ("rkey", "rpay", "skey", "spay")]
    got = ctx.join_filter_sort(*[dev(a) for a in args], d["slo"], d["shi"])
    st = ctx.join_stats()
    assert st["path"] == {0: st["path"], 1: "radix", 2: "learned"}[variant]
    check_join(got, orc.join_filter_sort(*args, d["slo"], d["shi"], mt=True))


def test_learned_spreads_skew_better_than_radix(ctx, knobs):
    # On the skewed mixture, radix partitioning leaves most rows in buckets
    # too big for shared memory; the learned partition function does not.
    d = datagen.config4_skewed(1 << 18, 1 << 22, seed=4, device="cuda")
    rows = {}
    for v in (1, 2):
        knobs(v)
        ctx.join_filter_sort(d["rkey"], d["rpay"], d["skey"], d["spay"], d["slo"], d["shi"])
        rows[v] = ctx.join_stats()["outside_rows"]
    assert rows[2] * 4 < rows[1]


def test_part_model_monotone_and_heavy_keys_isolated(ctx):
    keys = datagen.skewed_keys(1 << 20, 9, device="cuda")
    nb = 4096
    model = ctx.part_learn(keys, nb)
    u = torch.unique(keys.to(torch.int64) & 0xFFFFFFFF)  # ascending unsigned
    probe = torch.cat([u, u + 1, u - 1]).clamp(0, 2 ** 32 - 1)
    probe = torch.unique(probe)
    probe32 = (probe - (probe >= 2 ** 31).to(torch.int64) * 2 ** 32).to(torch.int32)
    b = ctx.part_eval(probe32, model).to(torch.int64)
    assert int(b.min()) >= 0 and int(b.max()) < nb
    assert bool((b[1:] >= b[:-1]).all()), "bucket function not monotone in the unsigned key"
    # the most frequent key owns its bucket
    vals, cnt = torch.unique(keys, return_counts=True)
    top = vals[cnt.argmax()].reshape(1)
    tb = int(ctx.part_eval(top, model)[0])
    same = probe32[(b == tb)]
    assert same.numel() == 1 and int(same[0]) == int(top[0])
    # buckets are balanced within a few times the mean on the sample itself
    hb = torch.bincount(ctx.part_eval(keys, model).to(torch.int64), minlength=nb)
    heavy_mass = int(cnt.max())
    assert int(hb.max()) <= max(8 * keys.numel() // nb, heavy_mass)


def test_part_radix_eval(ctx):
    keys = torch.tensor([5, 6, 1029, -1], dtype=torch.int32, device="cuda")
    b = ctx.part_eval(keys, None, kmin=5, shift=10).cpu().tolist()
    assert b == [0, 0, 1, (2 ** 32 - 1 - 5) >> 10]


@pytest.mark.parametrize("variant", [1, 2])
def test_join_config4_full_size(ctx, knobs, variant):
    # The skewed config at the size the bench quotes (R 32M unique keys, S 256M
    # keys from 8 Gaussians + 5 % Zipf(1.2) heavy hitters, S.payload < 300),
    # radix (1) and learned (2) partitioning; both leave rows in oversize
    # buckets, so the sort-merge and cross-product paths run.  Size-independent
    # exact checks: the row count equals the filtered S rows whose key is in R,
    # keys ascend (unsigned), every R.payload is R's payload for that key, and
    # the multiset of (key, S.payload) equals the filtered, matching S rows'.
    knobs(variant)
    d = datagen.config4_skewed(1 << 25, 1 << 28, seed=0, device="cuda")
    ok, orp, osp = ctx.join_filter_sort(d["rkey"], d["rpay"], d["skey"], d["spay"], d["slo"], d["shi"],
                                        cap=120_000_000)
    st = ctx.join_stats()
    assert st["path"] == {1: "radix", 2: "learned"}[variant]
    assert st["outside_rows"] > 0, st
    ru = d["rkey"].long() & 0xFFFFFFFF
    ru_sorted, order = torch.sort(ru)
    rpay_sorted = d["rpay"][order]
    del ru, order
    m = d["spay"] <= 299
    sk = d["skey"][m].long() & 0xFFFFFFFF
    ss = d["spay"][m].long()
    del m
    pos = torch.searchsorted(ru_sorted, sk).clamp_(max=ru_sorted.numel() - 1)
    hit = ru_sorted[pos] == sk
    sk, ss = sk[hit], ss[hit]
    del pos, hit
    assert ok.numel() == sk.numel()
    gu = ok.long() & 0xFFFFFFFF
    assert bool((gu[1:] >= gu[:-1]).all())
    gpos = torch.searchsorted(ru_sorted, gu)
    assert torch.equal(orp, rpay_sorted[gpos])
    del gpos
    e = torch.sort(sk * 1024 + ss).values
    del sk, ss
    g = torch.sort(gu * 1024 + osp.long()).values
    assert torch.equal(e, g)


@pytest.fixture
def dense_knob(ctx):
    yield ctx.join_set_dense
    ctx.join_set_dense(True)


@pytest.mark.parametrize("wide_pay", [False, True])
@pytest.mark.parametrize("nR,nS,gap,base", [
    (1, 5, 1, 7),
    (1000, 50000, 1, 0),
    (1 << 16, 1 << 20, 1, 1000),
    (1 << 16, 1 << 20, 2, -(1 << 20)),      # every other key, all negative (one unsigned span)
    (50000, 3 << 20, 1, (1 << 31) - 25000),  # keys across 0x7fffffff / 0x80000000 (unsigned order)
])
def test_join_dense_build_side(ctx, orc, knobs, dense_knob, nR, nS, gap, base, wide_pay):
    # Unique R keys over a dense span: R becomes a payload table indexed by
    # key - min -- absent keys marked by a sentinel payload that no R row holds,
    # or, when R's payloads span every candidate (wide_pay), by a presence
    # bitmap -- and only S is partitioned.  Equal to the oracle, to the general
    # path (dense build side off) and to the learned partitioning (which takes
    # the general path).
    rng = np.random.default_rng(nR + nS + gap)
    rk = (rng.permutation(nR).astype(np.int64) * gap + base)
    rkey = ((rk + (1 << 31)) % (1 << 32) - (1 << 31)).astype(np.int32)
    rpay = rng.integers(-1000, 1000, nR).astype(np.int32)
    if wide_pay:
        rpay[0] = -(2 ** 31)
        rpay[-1] = 2 ** 31 - 1
    sk = rng.integers(base - 300, base + nR * gap + 300, nS)
    skey = ((sk + (1 << 31)) % (1 << 32) - (1 << 31)).astype(np.int32)
    spay = rng.integers(0, 1000, nS).astype(np.int32)
    skey[0], spay[0] = rkey[0], 0  # at least one S row passes the filters
    exp = orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 299, cap=nS + 16, mt=True)
    args = [dev(a) for a in (rkey, rpay, skey, spay)]
    check_join(ctx.join_filter_sort(*args, -(2 ** 31), 299), exp)
    assert ctx.join_stats()["path"] == "dense"
    knobs(0, 0, 1024, 0)  # groups of at most 1024 rows: the 512-thread form of the dense bucket kernel
    check_join(ctx.join_filter_sort(*args, -(2 ** 31), 299), exp)
    assert ctx.join_stats()["path"] == "dense"
    knobs(0)
    dense_knob(False)
    check_join(ctx.join_filter_sort(*args, -(2 ** 31), 299), exp)
    assert ctx.join_stats()["path"] == "radix"
    dense_knob(True)
    knobs(2)
    check_join(ctx.join_filter_sort(*args, -(2 ** 31), 299), exp)
    assert ctx.join_stats()["path"] == "learned"


def test_join_dense_span_duplicate_key_takes_general_path(ctx, orc):
    # A dense span with one key twice: the bitmap sees the duplicate, and the
    # general path (R records after all) joins both build rows.
    rng = np.random.default_rng(21)
    rkey = rng.permutation(20000).astype(np.int32)
    rkey[5] = rkey[6]
    rpay = rng.integers(0, 1000, rkey.size).astype(np.int32)
    skey = rng.integers(-10, 20010, 300000).astype(np.int32)
    spay = rng.integers(0, 1000, skey.size).astype(np.int32)
    got = ctx.join_filter_sort(dev(rkey), dev(rpay), dev(skey), dev(spay), -(2 ** 31), 299)
    assert ctx.join_stats()["path"] == "radix"
    check_join(got, orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 299, cap=skey.size * 2, mt=True))


def test_join_dense_oversize_bucket_falls_back(ctx, orc):
    # Unique R keys over a dense span, but one S key holds 200K rows: its
    # bucket exceeds the bucket kernel, so R's records are made after all and
    # the general path (with its outside buckets) finishes the join.
    rng = np.random.default_rng(22)
    nR = 1 << 16
    rkey = rng.permutation(nR).astype(np.int32)
    rpay = rng.integers(0, 1000, nR).astype(np.int32)
    skey = np.concatenate([rng.integers(0, nR, 1 << 20), np.full(200000, 4321)]).astype(np.int32)
    rng.shuffle(skey)
    spay = rng.integers(0, 1000, skey.size).astype(np.int32)
    got = ctx.join_filter_sort(dev(rkey), dev(rpay), dev(skey), dev(spay), -(2 ** 31), 299)
    st = ctx.join_stats()
    assert st["path"] == "radix" and st["outside_buckets"] > 0, st
    check_join(got, orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 299, cap=skey.size + 16, mt=True))


@pytest.mark.parametrize("full", [True, False])
def test_join_dense_capacity_error(ctx, orc, full):
    # The dense bucket kernel writes only below `cap` and the call reports the
    # size needed (QG_ERR_CAPACITY); the wrapper then retries with it.  With
    # and without every S' row matching (a permutation of the span, or gaps).
    from ctypes import byref, c_int64, c_void_p

    rng = np.random.default_rng(41)
    nR, nS = 1 << 14, 1 << 18
    rkey = (rng.permutation(nR) * (1 if full else 2)).astype(np.int32)
    rpay = rng.integers(0, 1000, nR).astype(np.int32)
    skey = rng.integers(0, nR * (1 if full else 2), nS).astype(np.int32)
    spay = rng.integers(0, 1000, nS).astype(np.int32)
    exp = orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 299, cap=nS + 16, mt=True)
    need = len(exp[0])
    r, rp, s, sp = (dev(a) for a in (rkey, rpay, skey, spay))
    small = need // 3
    out = [torch.full((small + 64,), 7, dtype=torch.int32, device="cuda") for _ in range(3)]
    m = c_int64()
    p = lambda t: c_void_p(t.data_ptr())  # noqa: E731
    st = ctx.lib.qg_join_filter_sort(ctx.handle, p(r), p(rp), nR, p(s), p(sp), nS, -(2 ** 31), 299,
                                     p(out[0]), p(out[1]), p(out[2]), small, byref(m))
    assert st == 3 and m.value == need
    assert ctx.join_stats()["path"] == "dense"
    assert all(int((o[small:] != 7).sum()) == 0 for o in out), "a row was written past cap"
    check_join(ctx.join_filter_sort(r, rp, s, sp, -(2 ** 31), 299), exp)
