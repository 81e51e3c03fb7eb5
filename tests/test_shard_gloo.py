"""The multi-GPU host logic with two gloo ranks on the CPU: shard ranges cover all
orbits once, in whole DOP853 batches; timings reduce to the maximum over ranks;
host gathers concatenate in rank order."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from gala_gb300.shard import shard_range


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("n,world,granule", [(100000, 2, 100), (1050, 2, 100), (7, 3, 100), (0, 2, 100),
                                             (262144, 8, 1), (999, 4, 10)])
def test_shard_ranges_cover_once_in_whole_batches(n, world, granule):
    ranges = [shard_range(n, r, world, granule) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    for (a0, a1), (b0, b1) in zip(ranges, ranges[1:]):
        assert a1 == b0 and a0 <= a1
    for a0, a1 in ranges:
        assert a0 % granule == 0 or a0 == n
        assert a1 % granule == 0 or a1 == n
    units = [(a1 - a0 + granule - 1) // granule for a0, a1 in ranges]
    assert max(units) - min(units) <= 1


def test_shard_range_rejects_bad_ranks():
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)
    with pytest.raises(ValueError):
        shard_range(10, 0, 0)


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from gala_gb300.shard import gather_orbits, max_over_ranks

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n = 1050
        lo, hi = shard_range(n, rank, world, 100)
        w = np.arange(6 * n, dtype=np.float64).reshape(6, n)[:, lo:hi]   # this rank's orbits
        t_ms = 10.0 + 5.0 * rank                                          # this rank's timing
        t_max = max_over_ranks(t_ms)
        full = gather_orbits(w, axis=1)
        dist.barrier()
        q.put((rank, lo, hi, t_max, None if full is None else full.tolist()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_time_and_gather():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [(o[1], o[2]) for o in out] == [(0, 600), (600, 1050)]
    assert all(o[3] == 15.0 for o in out)                  # max over ranks, on every rank
    full = np.asarray(out[0][4])
    assert np.array_equal(full, np.arange(6 * 1050, dtype=np.float64).reshape(6, 1050))
    assert out[1][4] is None
