"""GPU parity: single-pass filter vs the oracle (bit-exact, positional:
filterImpl's scatter is stable, kernel/filter/filter_op.cl:220-238)."""
import numpy as np
import pytest
import torch

from query_on_opencl_fpga_gb300 import datagen

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_filter_rec_golden(ctx, orc, golden):
    meta, arrs = golden
    c = meta["cases"]["filter"]
    rin = orc.generate_rand(100, c["n"], 0)
    out = ctx.filter_range_rec(dev(rin), c["small"], c["large"]).cpu().numpy()
    assert np.array_equal(out, arrs["filter_out"])


@pytest.mark.parametrize("n", [0, 1, 2, 3, 5, 31, 4095, 4096, 4097, 8191, 100003, 1 << 20])
def test_filter_rec_sizes(ctx, orc, n):
    rin = orc.generate_rand(1000, n, n) if n else np.zeros((0, 2), np.int32)
    for lo, hi in [(0, 99), (-1000, 1000), (500, 400), (-(2 ** 31), 2 ** 31 - 1)]:
        exp = orc.filter_rec(rin, lo, hi)
        got = ctx.filter_range_rec(dev(rin) if n else torch.zeros((0, 2), dtype=torch.int32, device="cuda"),
                                   lo, hi).cpu().numpy()
        assert got.shape == exp.shape and np.array_equal(got, exp), (n, lo, hi)


def test_filter_rec_capacity(ctx, orc):
    from query_on_opencl_fpga_gb300 import QGError

    rin = orc.generate_rand(10, 10000, 1)
    with pytest.raises(QGError) as e:
        ctx.filter_range_rec(dev(rin), -100, 100, cap=5)
    assert e.value.status == 3
    # the context stays usable
    got = ctx.filter_range_rec(dev(rin), 0, 3).cpu().numpy()
    assert np.array_equal(got, orc.filter_rec(rin, 0, 3))


@pytest.mark.parametrize("n", [0, 1, 7, 4096, 65537, 1 << 21])
def test_filter_cols(ctx, orc, n):
    d = datagen.config0_filter(n, seed=n)
    key, pay = d["key"].numpy(), d["payload"].numpy()
    exp = orc.filter_cols(key, pay, d["lo"], d["hi"])
    got = ctx.filter_cols(dev(key), dev(pay), d["lo"], d["hi"]).cpu().numpy()
    assert np.array_equal(got, exp)


def test_filter_cols_config0_full_size(ctx, orc):
    # Full config-0 size: 16M rows, ~10 % selectivity, bit-exact.
    d = datagen.config0_filter(1 << 24, seed=0, device="cuda")
    got = ctx.filter_cols(d["key"], d["payload"], d["lo"], d["hi"])
    key, pay = d["key"].cpu().numpy(), d["payload"].cpu().numpy()
    exp = orc.filter_cols(key, pay, d["lo"], d["hi"], mt=True)
    assert got.shape[0] == exp.shape[0]
    assert np.array_equal(got.cpu().numpy(), exp)


def test_filter_cols_into_caller_buffer(ctx, orc):
    # out=: one caller-owned (cap, 2) buffer reused by calls of different selectivity
    d = datagen.config0_filter(1 << 20, seed=12)
    key, pay = d["key"].numpy(), d["payload"].numpy()
    out = torch.empty((1 << 20, 2), dtype=torch.int32, device="cuda")
    for lo, hi in ((d["lo"], d["hi"]), (0, 1 << 30), (5, 4)):
        got = ctx.filter_cols(dev(key), dev(pay), lo, hi, out=out)
        assert got.numel() == 0 or got.data_ptr() == out.data_ptr()  # an empty view reports 0
        assert np.array_equal(got.cpu().numpy(), orc.filter_cols(key, pay, lo, hi))
    with pytest.raises(ValueError):
        ctx.filter_cols(dev(key), dev(pay), 0, 1, out=out[:10])


def test_filter_repeat_is_deterministic(ctx):
    d = datagen.config0_filter(1 << 22, seed=5, device="cuda")
    a = ctx.filter_cols(d["key"], d["payload"], 0, 1 << 29).clone()
    for _ in range(3):
        b = ctx.filter_cols(d["key"], d["payload"], 0, 1 << 29)
        assert torch.equal(a, b)


def test_lookback_timeout_reports_and_recovers(ctx, orc):
    # A poll limit of 0 makes every look-back give up at once: the call must
    # report a timeout (no hang, no fault) and the context must stay usable.
    from query_on_opencl_fpga_gb300 import QGError

    rin = orc.generate_rand(100, 1 << 16, 0)
    ctx.set_spin_limit(0)
    try:
        with pytest.raises(QGError) as e:
            ctx.filter_range_rec(dev(rin), 0, 50)
        assert e.value.status == 5
    finally:
        ctx.set_spin_limit(1 << 22)
    got = ctx.filter_range_rec(dev(rin), 0, 50).cpu().numpy()
    assert np.array_equal(got, orc.filter_rec(rin, 0, 50))


@pytest.mark.parametrize("variant", [0, 1])
def test_filter_cols_timeout_reports_and_recovers(ctx, orc, variant):
    # Poll limit 0 on the single-pass column filters: every wait (look-back,
    # and for variant 1 the bulk-copy ring's barriers) gives up at once.  The
    # call reports a timeout, the ring stops refilling and drains its copies,
    # and the next call with the default limit is exact.
    from query_on_opencl_fpga_gb300 import QGError

    ctx.check(ctx.lib.qg_filter_set_variant(variant), "variant")
    d = datagen.config0_filter(1 << 22, seed=41)
    key, pay = d["key"].numpy(), d["payload"].numpy()
    try:
        ctx.set_spin_limit(0)
        try:
            with pytest.raises(QGError) as e:
                ctx.filter_cols(dev(key), dev(pay), d["lo"], d["hi"])
            assert e.value.status == 5
        finally:
            ctx.set_spin_limit(1 << 22)
        got = ctx.filter_cols(dev(key), dev(pay), d["lo"], d["hi"]).cpu().numpy()
        assert np.array_equal(got, orc.filter_cols(key, pay, d["lo"], d["hi"]))
    finally:
        ctx.lib.qg_filter_set_variant(2)


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("n", [1, 4095, 4099, 300007, 1 << 22, 1048576 + 4096 * 300 + 5])
def test_filter_cols_variants(ctx, orc, variant, n):
    ctx.check(ctx.lib.qg_filter_set_variant(variant), "variant")
    try:
        d = datagen.config0_filter(n, seed=n + variant)
        key, pay = d["key"].numpy(), d["payload"].numpy()
        got = ctx.filter_cols(dev(key), dev(pay), d["lo"], d["hi"]).cpu().numpy()
        assert np.array_equal(got, orc.filter_cols(key, pay, d["lo"], d["hi"]))
    finally:
        ctx.lib.qg_filter_set_variant(2)  # the default
