"""The CPU oracle against the reference: golden vectors made from the
reference's own generator and validators (tests/golden/make_golden.py), and,
where the reference checkout is present, the reference code itself."""
import hashlib

import numpy as np
import pytest


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_generator_matches_reference_digest(orc, golden):
    meta, _ = golden
    c = meta["cases"]["filter"]
    assert sha(orc.generate_rand(c["maxmax"], c["n"], c["seed"])) == c["input_sha"]
    s = meta["cases"]["scan"]
    assert sha(orc.generate_rand_int(s["n"], s["n"], 0)) == s["input_sha"]


def test_generator_glibc_negative_keys(orc):
    # generator.cpp:70 under glibc (RAND_MAX = 2^31-1): rand()<<1 wraps, so
    # keys fall in (-maxmax, maxmax) -- reproduced, not "fixed".
    r = orc.generate_rand(100, 4096, 0)
    assert (r[:, 1] < 0).any() and (r[:, 1] > -100).all() and (r[:, 1] < 100).all()
    assert np.array_equal(r[:, 0], np.arange(4096))


def test_filter_golden(orc, golden):
    meta, arrs = golden
    c = meta["cases"]["filter"]
    rin = orc.generate_rand(100, c["n"], 0)
    out = orc.filter_rec(rin, c["small"], c["large"])
    assert out.shape[0] == c["out_n"]
    assert np.array_equal(out, arrs["filter_out"])
    assert c["validator_output"] == "filter passed"


def test_filter_cols_matches_rec_form(orc):
    rng = np.random.default_rng(1)
    key = rng.integers(-50, 50, 10000).astype(np.int32)
    pay = rng.integers(0, 1000, 10000).astype(np.int32)
    out = orc.filter_cols(key, pay, -3, 7)
    sel = np.nonzero((key >= -3) & (key <= 7))[0]
    assert np.array_equal(out[:, 0], sel) and np.array_equal(out[:, 1], pay[sel])
    assert np.array_equal(orc.filter_cols(key, pay, -3, 7, mt=True), out)


def test_scan_golden(orc, golden):
    meta, _ = golden
    s = meta["cases"]["scan"]
    sin = orc.generate_rand_int(s["n"], s["n"], 0)
    assert sha(orc.scan_excl(sin)) == s["output_sha"]


def test_scan_wraps():
    from oracle import oracle as orc

    x = np.array([2 ** 31 - 1, 5, -7], np.int32)
    assert orc.scan_excl(x).tolist() == [0, 2 ** 31 - 1, -(2 ** 31) + 4]


@pytest.mark.parametrize("n", [2048, 1 << 15, 100003])
def test_sort_golden(orc, golden, n):
    meta, _ = golden
    c = meta["cases"][f"sort_{n}"]
    rin = orc.generate_rand(200, n, 0)
    assert sha(rin) == c["input_sha"]
    srt = orc.sort_rec(rin)
    assert sha(srt[:, 1]) == c["keys_sorted_sha"]
    # unsigned order; payloads are a permutation of the input's
    u = srt[:, 1].view(np.uint32)
    assert (u[1:] >= u[:-1]).all()
    assert np.array_equal(np.sort(srt[:, 0]), np.sort(rin[:, 0]))


def test_groupby_golden(orc, golden):
    meta, arrs = golden
    c = meta["cases"]["groupby"]
    rin = orc.generate_rand(64, c["n"], 0)
    rin[:, 1] = np.mod(rin[:, 1], 64)
    assert sha(rin) == c["input_sha"]
    sp = orc.group_startpos(orc.sort_rec(rin))
    assert sp.size == c["num_groups"]
    assert np.array_equal(sp, arrs["groupby_startpos"])


@pytest.mark.parametrize("op,name", [(0, "sum"), (1, "max"), (2, "min"), (3, "avg")])
def test_aggregate_golden(orc, golden, op, name):
    meta, arrs = golden
    c = meta["cases"]["aggregate"]
    rin = orc.generate_rand(50, c["n"], 0)
    rin[:, 1] = np.mod(rin[:, 1], 50)
    srt = orc.sort_rec(rin)
    sp = orc.group_startpos(srt)
    assert np.array_equal(orc.aggregate_groups(srt, sp, op), arrs[f"agg_{name}"])
    assert c[f"{name}_validator_output"] == "Test Passed!"


def test_aggregate_reference_inits(orc):
    # MAX starts at 0 and MIN at 1<<30 (group_by_cu_op_dp.cl:560-564):
    # all-negative groups give 0 for MAX, large values clamp MIN at 1<<30.
    rec = np.array([[-5, 1], [-3, 1], [2 ** 30 + 5, 2], [2 ** 31 - 1, 2]], np.int32)
    sp = np.array([0, 2], np.int32)
    assert orc.aggregate_groups(rec, sp, 1).tolist() == [0, 2 ** 31 - 1]
    assert orc.aggregate_groups(rec, sp, 2).tolist() == [-5, 1 << 30]
    assert orc.aggregate_groups(rec, sp, 3).tolist() == [-4, ((2 ** 30 + 5 + 2 ** 31 - 1) - 2 ** 32) // 2 + 0]


def test_groupby_cols_oracle_matches_numpy(orc):
    rng = np.random.default_rng(2)
    key = rng.integers(-1000, 1000, 50000).astype(np.int32)
    val = rng.integers(-500, 1000, 50000).astype(np.int32)
    val2 = rng.integers(0, 1000, 50000).astype(np.int32)
    for v2 in (None, val2):
        m = np.ones(key.size, bool) if v2 is None else (v2 <= 499)
        gk, gs, gc = orc.groupby_cols(key, val, v2, -(2 ** 31), 499)
        uk = np.unique(key[m].view(np.uint32)).view(np.int32)
        assert np.array_equal(gk, uk)
        exp_s = np.array([val[m][key[m] == k].astype(np.int64).sum() for k in uk])
        exp_c = np.array([(key[m] == k).sum() for k in uk])
        assert np.array_equal(gs, exp_s) and np.array_equal(gc, exp_c)
        gk2, gs2, gc2 = orc.groupby_cols(key, val, v2, -(2 ** 31), 499, mt=True)
        assert np.array_equal(gk2, gk) and np.array_equal(gs2, gs) and np.array_equal(gc2, gc)


def test_join_oracle_matches_bruteforce(orc):
    rng = np.random.default_rng(3)
    rkey = rng.integers(0, 300, 400).astype(np.int32)  # duplicates on the build side
    rpay = rng.integers(0, 1000, 400).astype(np.int32)
    skey = rng.integers(0, 400, 3000).astype(np.int32)
    spay = rng.integers(0, 1000, 3000).astype(np.int32)
    ok, orp, osp = orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 299)
    exp = sorted((int(k), int(rp), int(sp)) for k, sp in zip(skey, spay) if sp <= 299
                 for kk, rp in zip(rkey, rpay) if kk == k)
    assert list(zip(ok.tolist(), orp.tolist(), osp.tolist())) == exp
    ok2, orp2, osp2 = orc.join_filter_sort(rkey, rpay, skey, spay, -(2 ** 31), 299, mt=True)
    got = sorted(zip(ok2.tolist(), orp2.tolist(), osp2.tolist()))
    assert got == exp and (np.diff(ok2.view(np.uint32).astype(np.int64)) >= 0).all()


def test_hash_join_ref_oracle(orc):
    r = np.array([[5, 50], [7, 70], [5, 51]], np.int32)
    s = np.array([[5, 1], [9, 2], [7, 3]], np.int32)
    out = orc.hash_join_ref(r, s)
    assert sorted(map(tuple, out.tolist())) == [(1, 50), (1, 51), (3, 70)]


@pytest.mark.skipif(not __import__("oracle.oracle", fromlist=["x"]).REF_TOOL.exists(),
                    reason="reference checkout not present (oracle/_ref not built)")
def test_validators_accept_oracle_live(orc, tmp_path):
    # Live run of the reference's validateFilter on an oracle output at a new size.
    n = 20011
    rin, = [orc.generate_rand(100, n, 3)]
    out = orc.filter_rec(rin, 10, 40)
    pin, pout = tmp_path / "in.bin", tmp_path / "out.bin"
    rin.tofile(pin)
    out.tofile(pout)
    assert "filter passed" in orc.ref_tool("validate_filter", pin, n, pout, out.shape[0], 10, 40)
