"""Books past 2^31 options (60 GB of inputs on the device): every index
computation of the map, the batched-books kernel and the no-alloc entry
point runs in 64 bits.  Size-independent checks: an option priced at index
2^31 + i gets the same bits as the same option priced in a small book, and
sampled prices agree with the CPU FP64 oracle within the reference's 1e-4."""
import numpy as np
import pytest

import oracle
from p3arsec_gb300 import Context, abi, books

pytestmark = pytest.mark.gpu

N = (1 << 31) + 4101  # past the int32 range, not a multiple of any vector width


@pytest.fixture(scope="module")
def big():
    import torch
    dev = books.generate_device(N, seed=2024)
    out = torch.empty(N, dtype=torch.float32, device="cuda:0")
    # the context prices on its own stream: torch's work must be done first
    torch.cuda.synchronize()
    ctx = Context(0, max_options=1)
    ctx.price_soa(*dev, out, n=N, num_runs=2, device=True)  # graph of two passes
    torch.cuda.synchronize()
    yield dev, out, ctx
    ctx.close()
    del dev, out
    torch.cuda.empty_cache()


def _sample(dev, out, idx):
    import torch
    it = torch.from_numpy(idx).to("cuda:0")
    arrays = [a.index_select(0, it).cpu().numpy() for a in dev]
    return books.Book(*arrays), out.index_select(0, it).cpu().numpy()


def test_map_past_2p31_options(big):
    dev, out, ctx = big
    rng = np.random.default_rng(3)
    idx = np.unique(np.concatenate([
        np.arange(N - 70_000, N), np.arange((1 << 31) - 2000, (1 << 31) + 2000),
        np.arange(0, 2000), rng.integers(0, N, 200_000)])).astype(np.int64)
    book, got = _sample(dev, out, idx)
    # position independence: the same options as a small host book
    host_ctx = Context(0, max_options=len(book))
    small = host_ctx.price_book(book, num_runs=1)
    host_ctx.close()
    assert np.array_equal(small.view(np.uint32), got.view(np.uint32))
    # the reference's check (blackscholes.c:333-339) against the FP64 oracle
    want = oracle.price_fp64(book)
    assert np.abs(got.astype(np.float64) - want).max() <= 1e-4


def test_batch_and_noalloc_segments_past_2p31(big):
    import torch
    dev, out, ctx = big
    b = 1 << 31
    # disjoint books inside the pool: a 1M-option book ending below 2^31,
    # one across it, two past it, the last option alone
    segs = [(0, 1000), (b - (1 << 20), (1 << 20) - 800), (b - 777, 3000), (b + 2500, 1000),
            (N - 500, 499), (N - 1, 1)]
    assert all(o + n <= N for o, n in segs)
    for how in ("batch", "noalloc"):
        res = torch.full((N,), -1.0, dtype=torch.float32, device="cuda:0")
        torch.cuda.synchronize()  # the fill runs on torch's stream, the batch on the context's
        if how == "batch":
            ctx.price_batch(dev, res, N, segs, num_runs=1)
        else:
            st = abi.price_batch_noalloc(dev, res, N, segs,
                                         stream=torch.cuda.current_stream().cuda_stream)
            assert st == 0
        torch.cuda.synchronize()
        for o, n in segs:
            a = res[o:o + n].cpu().numpy()
            b = out[o:o + n].cpu().numpy()
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (how, o, n)
        # outside the segments nothing is written
        assert float(res[1000:2000].max()) == -1.0 and float(res[N - 501]) == -1.0
        del res
