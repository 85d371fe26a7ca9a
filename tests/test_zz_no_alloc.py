"""bsg_price_batch_noalloc: the allocation-free batch entry point.

Callers that cannot allocate (fixed memory budgets, foreign allocators,
real-time loops) price books through this entry point; its scratch is a
fixed device array shared by all calls.  Checked through the C ABI against
bsg_price_batch on two calls in a row with different books, so a table or
counter left over from the first call would show up in the second; against
the CPU FP64 oracle directly (the ERR_CHK bound, 1e-4); with two
asynchronous calls queued back to back on one stream; and on a pool from an
allocator that maps memory piece by piece.  This file is collected last.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from p3arsec_gb300 import abi, books

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _layout(rng, nseg, max_len):
    segs, off = [], 0
    for _ in range(nseg):
        off += int(rng.integers(0, 40))
        n = int(np.exp(rng.uniform(0, np.log(max_len))))
        segs.append((off, n))
        off += n
    return segs, off


def _run_pair(gpu_ctx, torch, seed, nseg, max_len, oracle_lib=None):
    rng = np.random.default_rng(seed)
    segs, pool_len = _layout(rng, nseg, max_len)
    segs[0] = (segs[0][0], 0)  # an empty book
    book = books.generate(pool_len, seed=seed)
    pool = [torch.from_numpy(a).cuda() for a in book.arrays()]
    want = torch.full((pool_len,), -1.0, device="cuda:0")
    got = torch.full((pool_len,), -1.0, device="cuda:0")
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
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
    if oracle_lib is not None:
        # and directly against the CPU FP64 oracle: every priced option
        # within the reference's ERR_CHK bound, every gap option untouched
        mask = np.zeros(pool_len, dtype=bool)
        for o, n in segs:
            mask[o:o + n] = True
        fp64 = oracle_lib.price_fp64(book)
        assert np.abs(g[mask].astype(np.float64) - fp64[mask]).max() <= 1e-4
        assert np.all(g[~mask] == -1.0)


def test_noalloc_matches_batch_two_calls_in_a_row(gpu_ctx, oracle_lib):
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    _run_pair(gpu_ctx, torch, seed=1, nseg=700, max_len=1 << 15, oracle_lib=oracle_lib)
    _run_pair(gpu_ctx, torch, seed=2, nseg=abi.NOALLOC_MAX_SEGMENTS, max_len=1 << 12,
              oracle_lib=oracle_lib)


def test_noalloc_async_calls_queued_back_to_back(gpu_ctx):
    """Two BSG_ASYNC calls with different books on one stream and no
    synchronisation between them: the second call's table upload, counter
    reset and kernel are ordered after the first call's kernel by the
    stream, so both give bsg_price_batch's bits."""
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    cases = []
    for seed, nseg, max_len in ((5, 900, 1 << 14), (6, 3000, 1 << 11)):
        rng = np.random.default_rng(seed)
        segs, pool_len = _layout(rng, nseg, max_len)
        book = books.generate(pool_len, seed=seed)
        pool = [torch.from_numpy(a).cuda() for a in book.arrays()]
        want = torch.full((pool_len,), -1.0, device="cuda:0")
        torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
        gpu_ctx.price_batch(pool, want, pool_len, segs)
        got = torch.full((pool_len,), -1.0, device="cuda:0")
        cases.append((segs, pool_len, pool, want, got))
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    for segs, pool_len, pool, _, got in cases:
        st = abi.price_batch_noalloc(pool, got, pool_len, segs, stream=stream, asynchronous=True)
        assert st == 0, abi.STATUS.get(st, st)
    torch.cuda.synchronize()
    for segs, pool_len, pool, want, got in cases:
        assert torch.equal(got.view(torch.int32), want.view(torch.int32))


_EXPANDABLE = textwrap.dedent("""
    import sys
    import numpy as np
    import torch
    sys.path.insert(0, {root!r})
    from p3arsec_gb300 import abi, books, Context
    torch.cuda.set_device(0)
    # grow the pool piece by piece: small tensors first, then books that
    # span several of the allocator's mapped pieces
    keep = [torch.empty(3 << 20, dtype=torch.uint8, device="cuda:0") for _ in range(5)]
    n = 12_000_000  # 48 MB per array, > 20 MB pieces
    book = books.generate(n, seed=9)
    pool = [torch.from_numpy(a).cuda() for a in book.arrays()]
    got = torch.full((n,), -1.0, device="cuda:0")
    want = torch.full((n,), -1.0, device="cuda:0")
    segs = [(0, 5_000_001), (5_000_064, n - 5_000_064)]
    st = abi.price_batch_noalloc(pool, got, n, segs)
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
    with Context(0, 1) as ctx:
        ctx.price_batch(pool, want, n, segs)
    torch.cuda.synchronize()
    same = torch.equal(got.view(torch.int32), want.view(torch.int32))
    # a size far past the mapped pieces is still refused
    over = abi.price_batch_noalloc(pool, got, 1 << 35, [(0, 1)])
    print("STATUS", st, "SAME", int(same), "OVER", over)
""")


def test_noalloc_on_a_pool_mapped_piece_by_piece():
    """torch's expandable segments map device memory in pieces into one
    virtual range (the VMM API); arrays that span pieces are valid device
    memory, and both batch entry points must accept and price them."""
    env = dict(os.environ, PYTORCH_CUDA_ALLOC_CONF="expandable_segments:True")
    r = subprocess.run([sys.executable, "-c", _EXPANDABLE.format(root=ROOT)], cwd=ROOT, env=env,
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "STATUS 0 SAME 1 OVER -1" in r.stdout, r.stdout + r.stderr[-3000:]


def test_noalloc_rejects_more_segments_than_its_scratch(gpu_ctx):
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    book = books.generate(8192, seed=3)
    pool = [torch.from_numpy(a).cuda() for a in book.arrays()]
    out = torch.zeros(8192, device="cuda:0")
    segs = [(i, 1) for i in range(abi.NOALLOC_MAX_SEGMENTS + 1)]
    assert abi.price_batch_noalloc(pool, out, 8192, segs) == -5  # BSG_ERR_CAPACITY
    assert abi.price_batch_noalloc(pool, out, 8192, [(8000, 500)]) == -1  # outside the pool
