"""The N > 1 host logic of bench.py on CPU with gloo (world size 2):
contiguous shards cover the options exactly once, each rank prices its shard
independently (no data-path collective), and only the timing is reduced."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    import oracle
    from p3arsec_gb300 import books
    dist.init_process_group("gloo", rank=rank, world_size=world)
    book = books.generate(n, seed=77)
    off, ln = bench.shard_range(n, rank, world)
    part = oracle.price_ref(book.slice(off, off + ln))
    np.save(os.path.join(out_dir, f"part{rank}.npy"), part)
    np.save(os.path.join(out_dir, f"range{rank}.npy"), np.array([off, ln]))
    t = bench.reduce_max(dist, float(rank + 1.5))
    np.save(os.path.join(out_dir, f"max{rank}.npy"), np.array([t]))
    bench.barrier(dist)
    dist.destroy_process_group()


@pytest.mark.parametrize("n", [10007, 3])
def test_two_rank_shards(tmp_path, n):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, n, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    import oracle
    from p3arsec_gb300 import books
    full = oracle.price_ref(books.generate(n, seed=77))
    parts = [np.load(tmp_path / f"part{r}.npy") for r in range(2)]
    ranges = [np.load(tmp_path / f"range{r}.npy") for r in range(2)]
    assert ranges[0][0] == 0 and ranges[0][0] + ranges[0][1] == ranges[1][0]
    assert ranges[1][0] + ranges[1][1] == n
    got = np.concatenate(parts)
    assert np.array_equal(got.view(np.uint32), full.view(np.uint32))
    for r in range(2):
        assert float(np.load(tmp_path / f"max{r}.npy")[0]) == 2.5


def test_shard_range_rule():
    import bench
    for n in (0, 1, 7, 100, 10_000_001):
        for w in (1, 2, 3, 8):
            spans = [bench.shard_range(n, r, w) for r in range(w)]
            assert sum(l for _, l in spans) == n
            assert all(spans[i][0] + spans[i][1] == spans[i + 1][0] for i in range(w - 1))
            assert max(l for _, l in spans) - min(l for _, l in spans) <= 1
