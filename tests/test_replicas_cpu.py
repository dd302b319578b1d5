"""The multi-process (replica) path of bench.py on CPU: two gloo ranks, each
working on its own seeded shard, joined by the bench's barrier and
max-over-ranks timing, with the whole-job value summed over ranks.  The path
shards by replicas only; no collective touches the data."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import numpy as np
    import torch.distributed as dist

    import bench
    from oracle import oracle as orc

    r, w, local = bench.dist_init(world)
    assert (r, w, local) == (rank, world, rank)
    # each rank filters its own shard (replica work), timed locally
    key = np.random.default_rng(rank).integers(0, 2 ** 31, 1 << 16).astype(np.int32)
    pay = np.arange(key.size, dtype=np.int32)
    got = orc.filter_cols(key, pay, -(2 ** 31), 214748363)
    local_ms = 1.0 + rank  # stand-in for the rank's measured step time
    bench.barrier(w)
    ms = bench.max_over_ranks(local_ms, w)
    rows = key.size * w
    out[rank] = (ms, rows / (ms * 1e-3), int(got.shape[0]))
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_replicas_take_the_max_time():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 2.0  # max over ranks
    assert out[0][1] == out[1][1] == (2 * (1 << 16)) / 2e-3
    assert out[0][2] > 0 and out[1][2] > 0
