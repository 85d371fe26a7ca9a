"""bsg_price_batch_noalloc: the allocation-free batch entry point.

Callers that cannot allocate (fixed memory budgets, foreign allocators,
real-time loops) price books through this entry point; its scratch is a
fixed device array shared by all calls.  Checked through the C ABI against
bsg_price_batch on two calls in a row with different books, so a table or
counter left over from the first call would show up in the second.  This
file is collected last.
"""
import numpy as np
import pytest

from p3arsec_gb300 import abi, books

pytestmark = pytest.mark.gpu


def _layout(rng, nseg, max_len):
    segs, off = [], 0
    for _ in range(nseg):
        off += int(rng.integers(0, 40))
        n = int(np.exp(rng.uniform(0, np.log(max_len))))
        segs.append((off, n))
        off += n
    return segs, off


def _run_pair(gpu_ctx, torch, seed, nseg, max_len):
    rng = np.random.default_rng(seed)
    segs, pool_len = _layout(rng, nseg, max_len)
    segs[0] = (segs[0][0], 0)  # an empty book
    book = books.generate(pool_len, seed=seed)
    pool = [torch.from_numpy(a).cuda() for a in book.arrays()]
    want = torch.full((pool_len,), -1.0, device="cuda:0")
    got = torch.full((pool_len,), -1.0, device="cuda:0")
    gpu_ctx.price_batch(pool, want, pool_len, segs)
    torch.cuda.synchronize()
    st = abi.price_batch_noalloc(pool, got, pool_len, segs,
                                 stream=torch.cuda.current_stream().cuda_stream)
    assert st == 0, abi.STATUS.get(st, st)
    torch.cuda.synchronize()
    w = want.cpu().numpy()
    g = got.cpu().numpy()
    # same arithmetic as bsg_price_batch: bit-identical (within any tolerance
    # the other tests use), gaps between books untouched
    assert np.array_equal(g.view(np.uint32), w.view(np.uint32))


def test_noalloc_matches_batch_two_calls_in_a_row(gpu_ctx):
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    _run_pair(gpu_ctx, torch, seed=1, nseg=700, max_len=1 << 15)
    _run_pair(gpu_ctx, torch, seed=2, nseg=abi.NOALLOC_MAX_SEGMENTS, max_len=1 << 12)


def test_noalloc_rejects_more_segments_than_its_scratch(gpu_ctx):
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    book = books.generate(8192, seed=3)
    pool = [torch.from_numpy(a).cuda() for a in book.arrays()]
    out = torch.zeros(8192, device="cuda:0")
    segs = [(i, 1) for i in range(abi.NOALLOC_MAX_SEGMENTS + 1)]
    assert abi.price_batch_noalloc(pool, out, 8192, segs) == -5  # BSG_ERR_CAPACITY
    assert abi.price_batch_noalloc(pool, out, 8192, [(8000, 500)]) == -1  # outside the pool
