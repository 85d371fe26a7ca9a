"""Batched books (persistent kernel + tile cursor) and the accuracy report."""
import numpy as np
import pytest

import oracle
from p3arsec_gb300 import books
from p3arsec_gb300.abi import BsgError

pytestmark = pytest.mark.gpu


def pool_on_device(torch, book):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in book.arrays()]


def layout(sizes, rng, gap_max=37):
    """Offsets with random gaps (unaligned starts) for the given sizes."""
    segs, off = [], 0
    for n in sizes:
        off += int(rng.integers(0, gap_max))
        segs.append((off, int(n)))
        off += int(n)
    return segs, off


@pytest.mark.parametrize("seed,mode", [(0, "fast"), (1, "fast"), (2, "fast"), (3, "sfu_ref"),
                                       (4, "libm_ref")])
def test_batch_equals_per_book_and_plain(gpu_ctx, seed, mode):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(0, np.log(1 << 16), 300)).astype(np.int64)
    sizes[:5] = [0, 1, 2, 3, 8193]
    rng.shuffle(sizes)
    segs, pool_len = layout(sizes, rng)
    book = books.generate(pool_len, seed=100 + seed)
    pool = pool_on_device(torch, book)
    out_b = torch.full((pool_len,), -1.0, device="cuda:0")
    out_p = torch.full((pool_len,), -1.0, device="cuda:0")
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
    gpu_ctx.price_batch(pool[:6], out_b, pool_len, segs, num_runs=1, mode=mode)
    gpu_ctx.price_batch(pool[:6], out_p, pool_len, segs, num_runs=1, plain=True, mode=mode)
    torch.cuda.synchronize()
    b = out_b.cpu().numpy()
    p = out_p.cpu().numpy()
    whole = gpu_ctx.price_book(book, mode=mode)
    covered = np.zeros(pool_len, dtype=bool)
    for o, l in segs:
        covered[o:o + l] = True
    assert np.array_equal(b.view(np.uint32), p.view(np.uint32))
    assert np.array_equal(b[covered].view(np.uint32), whole[covered].view(np.uint32))
    assert np.all(b[~covered] == -1.0)  # gaps untouched


def test_batch_graph_runs_and_reuse(gpu_ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    segs, pool_len = layout(rng.integers(1, 20000, 64), rng)
    book = books.generate(pool_len, seed=7)
    pool = pool_on_device(torch, book)
    out = torch.zeros(pool_len, device="cuda:0")
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
    for runs in (1, 100, 100, 3):
        gpu_ctx.price_batch(pool, out, pool_len, segs, num_runs=runs)
    torch.cuda.synchronize()
    ref = gpu_ctx.price_book(book)
    got = out.cpu().numpy()
    for o, l in segs:
        assert np.array_equal(got[o:o + l].view(np.uint32), ref[o:o + l].view(np.uint32))


def test_batch_rejects_bad_segments(gpu_ctx):
    torch = pytest.importorskip("torch")
    book = books.generate(1000, seed=8)
    pool = pool_on_device(torch, book)
    out = torch.zeros(1000, device="cuda:0")
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
    with pytest.raises(BsgError):
        gpu_ctx.price_batch(pool, out, 1000, [(990, 20)])
    with pytest.raises(BsgError):
        gpu_ctx.price_batch(pool, out, 1000, [(0, 100), (50, 10)])
    with pytest.raises(BsgError):
        gpu_ctx.price_batch(pool, out, 1000 + (1 << 30), [(0, 10)])  # pool past its allocation
    gpu_ctx.price_batch(pool, out, 1000, [(0, 1000)])


@pytest.mark.parametrize("dist", ["plain", "tails"])
def test_error_report_matches_cpu(gpu_ctx, dist):
    torch = pytest.importorskip("torch")
    book = books.generate(200000, seed=21, dist=dist)
    pool = pool_on_device(torch, book)
    prices = gpu_ctx.price_book(book)
    dprices = torch.from_numpy(prices).cuda()
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
    edges = np.array([0.0, 0.5, 1.0, 2.0, 3.0, 4.0, 6.0, np.inf])
    rep = gpu_ctx.error_report(pool, dprices, len(book), edges, rel_floor=1e-3)
    fp64 = oracle.price_fp64(book)
    d1 = np.abs(oracle.d1_fp64(book))
    err = np.abs(prices.astype(np.float64) - fp64)
    idx = np.clip(np.searchsorted(edges, d1, side="right") - 1, 0, len(edges) - 2)
    # bucket membership can differ for an option sitting on an edge (device
    # FP64 may fuse multiply-adds): counts within 2, totals exact
    assert sum(b["count"] for b in rep) == len(book)
    for i, bk in enumerate(rep):
        assert abs(bk["count"] - int((idx == i).sum())) <= 2
    assert max(b["max_abs"] for b in rep) == pytest.approx(err.max(), rel=1e-9, abs=1e-12)
    assert sum(b["sum_sq_abs"] for b in rep) == pytest.approx((err ** 2).sum(), rel=1e-6)
    if dist == "plain":
        assert max(b["max_abs"] for b in rep) <= 1e-4


def test_batch_autotune_and_every_shape_gives_the_same_bits(gpu_ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    segs, pool_len = layout(rng.integers(1, 30000, 120), rng)
    book = books.generate(pool_len, seed=12)
    pool = pool_on_device(torch, book)
    out = torch.zeros(pool_len, device="cuda:0")
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
    saved = gpu_ctx.get_batch_tune()
    try:
        chosen = gpu_ctx.autotune_batch(pool, out, pool_len, segs)
        assert chosen["tile_options"] in (2048, 4096, 8192, 16384, 32768)
        ref = gpu_ctx.price_book(book)
        for tile in (2048, 32768):
            for bps in (1, 0):
                gpu_ctx.set_batch_tune(tile, bps)
                out.zero_()
                torch.cuda.synchronize()
                gpu_ctx.price_batch(pool, out, pool_len, segs, num_runs=2)
                torch.cuda.synchronize()
                got = out.cpu().numpy()
                for o, l in segs:
                    assert np.array_equal(got[o:o + l].view(np.uint32), ref[o:o + l].view(np.uint32))
    finally:
        gpu_ctx.set_batch_tune(**saved)


def test_batch_of_many_tiny_books(gpu_ctx):
    """100,000 books of 0 to 9 options (most shorter than one vector group,
    every start unaligned): one tile each, all priced as the map prices
    them, gaps untouched."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(29)
    segs, pool_len = layout(rng.integers(0, 10, 100_000), rng, gap_max=5)
    book = books.generate(pool_len, seed=31)
    pool = pool_on_device(torch, book)
    out = torch.full((pool_len,), -1.0, device="cuda:0")
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
    gpu_ctx.price_batch(pool, out, pool_len, segs, num_runs=3)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    whole = gpu_ctx.price_book(book)
    covered = np.zeros(pool_len, dtype=bool)
    for o, l in segs:
        covered[o:o + l] = True
    assert np.array_equal(got[covered].view(np.uint32), whole[covered].view(np.uint32))
    assert np.all(got[~covered] == -1.0)
