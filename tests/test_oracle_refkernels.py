"""The oracle against the reference's own OpenCL kernels, run on host cores
(oracle/_ref/libref_kernels.so: kernel/filter/filter_op.cl,
kernel/aggregation/1/group_by_cu_op_dp.cl and
kernel/hj_filter_sort/1/hj_filter_sort_op.cl compiled through
oracle/ref_kernels/clshim.h, driven as the reference host code drives them).

Skipped where the reference checkout is absent (the library is built from it);
tests/golden/golden_refk.json holds digests of the same reference outputs for
test_oracle_matches_reference_kernel_digests, which runs everywhere."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as orc

needs_rk = pytest.mark.skipif(orc.ref_kernels() is None, reason="reference kernels not built here")
GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_refk.json"


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@needs_rk
@pytest.mark.parametrize("n", [1 << 17, 1 << 18])
@pytest.mark.parametrize("maxmax,lo,hi", [(1000, 10, 400), (1 << 20, -(1 << 19), 1 << 18), (64, 0, 0)])
def test_filter_chain_matches_reference_kernels(n, maxmax, lo, hi):
    # generateRand under glibc gives negative keys too: the signed compare of
    # filter_op.cl:19-21 is exercised.
    rin = orc.generate_rand(maxmax, n, 1)
    assert np.array_equal(orc.refk_filter_rec(rin, lo, hi), orc.filter_rec(rin, lo, hi))


@needs_rk
@pytest.mark.parametrize("n", [1 << 17, 1 << 19])
def test_scan_matches_reference_kernels(n):
    x = np.random.default_rng(n).integers(-(2 ** 31), 2 ** 31, n, dtype=np.int64).astype(np.int32)
    assert np.array_equal(orc.refk_scan(x), orc.scan_excl(x))  # int32 wrap-around included


@needs_rk
@pytest.mark.parametrize("n", [2048, 1 << 14, 1 << 16])
def test_sort_matches_reference_kernels(n):
    # bitonicSortShared / bitonicMergeGlobal compare .y unsigned and are not
    # stable: keys must agree position by position, records as a multiset.
    rin = orc.generate_rand(1 << 24, n, 2)
    got, exp = orc.refk_sort_rec(rin), orc.sort_rec(rin)
    assert np.array_equal(got[:, 1], exp[:, 1])
    key = lambda a: a[np.lexsort((a[:, 0], a[:, 1].view(np.uint32)))]  # noqa: E731
    assert np.array_equal(key(got), key(exp))


@needs_rk
@pytest.mark.parametrize("n,groups", [(1 << 17, 50), (1 << 18, 4000)])
def test_groupby_and_aggregates_match_reference_kernels(n, groups):
    rin = orc.generate_rand(1 << 20, n, 3)
    rin[:, 1] = np.mod(rin[:, 1], groups)
    srt, sp = orc.refk_groupby_rec(rin)
    assert np.array_equal(srt[:, 1], orc.sort_rec(rin)[:, 1])
    assert np.array_equal(sp, orc.group_startpos(srt))
    for op in range(4):  # SUM, MAX, MIN, AVG as group_by_cu_op_dp.cl:547-716
        assert np.array_equal(orc.refk_aggregate(srt, sp, op), orc.aggregate_groups(srt, sp, op)), op


@needs_rk
def test_hash_join_matches_reference_kernels():
    rng = np.random.default_rng(4)
    nr, ns = 4096, 1 << 16
    r = np.stack([rng.permutation(nr * 3)[:nr], rng.integers(0, 1000, nr)], 1).astype(np.int32)
    s = np.stack([rng.integers(0, nr * 4, ns), rng.integers(0, 1000, ns)], 1).astype(np.int32)
    got, exp = orc.refk_hash_join(r, s), orc.hash_join_ref(r, s)
    key = lambda a: a[np.lexsort((a[:, 1], a[:, 0]))]  # noqa: E731
    assert np.array_equal(key(got), key(exp))


def test_oracle_matches_reference_kernel_digests():
    """Digests of the reference kernels' outputs (tests/golden/make_golden.py)
    against the oracle on the same inputs."""
    meta = json.loads(GOLDEN.read_text())
    for c in meta["filter"]:
        rin = orc.generate_rand(c["maxmax"], c["n"], c["seed"])
        out = orc.filter_rec(rin, c["lo"], c["hi"])
        assert (out.shape[0], sha(out)) == (c["count"], c["sha"]), c
    for c in meta["sort_keys"]:
        rin = orc.generate_rand(c["maxmax"], c["n"], c["seed"])
        assert sha(orc.sort_rec(rin)[:, 1]) == c["sha"], c
    for c in meta["groupby"]:
        rin = orc.generate_rand(c["maxmax"], c["n"], c["seed"])
        rin[:, 1] = np.mod(rin[:, 1], c["groups"])
        srt = orc.sort_rec(rin)
        sp = orc.group_startpos(srt)
        assert sha(sp) == c["startpos_sha"], c
        for op in range(4):
            assert sha(orc.aggregate_groups(srt, sp, op)) == c["agg_sha"][op], (c, op)
