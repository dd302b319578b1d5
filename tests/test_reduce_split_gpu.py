"""GPU parity of the whole-column reduce (the check of host/host/Validate.cpp:
372-468) and the radix split (host/host/testSplit.cpp:156-209) against the oracle."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("op", [0, 1, 2, 3])
@pytest.mark.parametrize("n", [1, 7, 4097, 1 << 20])
def test_reduce_matches_oracle(ctx, orc, op, n):
    rng = np.random.default_rng(n + op)
    rec = np.stack([rng.integers(0, 1 << 20, n), rng.integers(-2 ** 31, 2 ** 31, n)], 1).astype(np.int32)
    assert ctx.reduce_rec(dev(rec), op) == orc.reduce_rec(rec, op)


def test_reduce_generated_input(ctx, orc):
    rec = orc.generate_rand(1 << 24, 1 << 18, 0)  # the reference generator's records
    for op in range(4):
        assert ctx.reduce_rec(dev(rec), op) == orc.reduce_rec(rec, op)


@pytest.mark.parametrize("parts", [1, 3, 64, 256, 1000, 70000])
@pytest.mark.parametrize("n", [1, 5000, 300007])
def test_split_matches_oracle(ctx, orc, parts, n):
    rng = np.random.default_rng(parts * 31 + n)
    rec = np.stack([np.arange(n), rng.integers(-2 ** 31, 2 ** 31, n)], 1).astype(np.int32)
    out, bound = ctx.split_rec(dev(rec), parts)
    eout, ebound = orc.split_rec(rec, parts)
    assert np.array_equal(out.cpu().numpy(), eout)  # stable: exactly the oracle's order
    assert np.array_equal(bound.cpu().numpy(), ebound)


def test_split_reference_wrapper(ctx, orc):
    from query_on_opencl_fpga_gb300._lib import QgBuf

    n, parts = 10000, 16
    rec = orc.generate_rand(1 << 20, n, 5)
    d_in, d_out = dev(rec), torch.empty((n, 2), dtype=torch.int32, device="cuda")
    d_b = torch.empty(parts, dtype=torch.int32, device="cuda")
    buf = lambda t: QgBuf(t.data_ptr(), t.numel() * 4)  # noqa: E731
    ctx.lib.splitImpl(buf(d_in), n, parts, buf(d_out), buf(d_b), 256, 512, 0, ctx.handle)
    assert ctx.lib.qg_ref_last_status() == 0
    eout, ebound = orc.split_rec(rec, parts)
    assert np.array_equal(d_out.cpu().numpy(), eout) and np.array_equal(d_b.cpu().numpy(), ebound)
