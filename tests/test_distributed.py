"""Multi-rank host logic on CPU: two gloo ranks shard regions with no data-path collective and reduce
their timings (max) and cell counts (sum) the way bench.py does under torchrun."""
import os
import socket

import numpy as np
import pytest

from gatk_gb300 import sharding


def test_partition_by_cells_covers_and_balances():
    rng = np.random.default_rng(0)
    cells = rng.lognormal(17, 1, size=1000).astype(np.int64)
    parts = sharding.partition_by_cells(cells, 4)
    allr = np.sort(np.concatenate(parts))
    assert np.array_equal(allr, np.arange(1000))
    loads = [int(cells[p].sum()) for p in parts]
    assert max(loads) - min(loads) <= cells.max()


def test_block_range_is_disjoint():
    assert sharding.block_range(10000, 0) == (0, 10000)
    assert sharding.block_range(10000, 3) == (30000, 40000)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from gatk_gb300 import sharding as S

        cells = np.arange(1, 101, dtype=np.int64) * 1000
        mine = S.partition_by_cells(cells, world)[rank]
        local_cells = float(cells[mine].sum())
        local_ms = 10.0 + rank  # rank 1 is the slower one
        total = S.reduce_sum(local_cells)
        slowest = S.reduce_max(local_ms)
        q.put((rank, mine.tolist(), total, slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    owned = sorted(out[0][1] + out[1][1])
    assert owned == list(range(100))
    assert not set(out[0][1]) & set(out[1][1])
    for _, _, total, slowest in out:
        assert total == float(np.arange(1, 101).sum() * 1000)
        assert slowest == 11.0
