"""GPU parity: the sm_103a kernels, called through the C ABI, against the
oracle and the reference's golden outputs.

Tolerances (FP32 output):
  * fast (production) vs the FP64 oracle: max |err| <= 1e-4 on the plain
    distribution (the accuracy gate; the reference itself reaches ~8e-5),
    and <= 2e-4 + 2 ulp(price) on the tails (FP32 cannot resolve 1e-4 above
    2048; the reference reaches 5e-4 there).
  * vs the reference's own FP32 prices: <= 2e-4 (both sides ~1e-4 from FP64).
  * libm_ref (reference operation order, correctly rounded exp/log) vs the
    same order with exp/log rounded through double on the CPU: bit-identical
    on >= 99.99 % of options; vs the reference (glibc's expf/logf, not
    correctly rounded on ~0.1 % of arguments): bit-identical on >= 99 %,
    the rest within 5e-5 + 4 ulp of the price.
  * FP64 kernel vs the CPU FP64 oracle: rtol 1e-12.
"""
import os

import numpy as np
import pytest

from conftest import load_golden
from p3arsec_gb300 import books

pytestmark = pytest.mark.gpu

CASES = ["plain_4096", "tails_4096", "edge"]


def ulp(x):
    return np.spacing(np.abs(x).astype(np.float32)).astype(np.float64)


@pytest.mark.parametrize("name", CASES)
def test_fast_vs_fp64_and_reference(gpu_ctx, name):
    book, ref, fp64 = load_golden(name)
    got = gpu_ctx.price_book(book, num_runs=1, mode="fast").astype(np.float64)
    err = np.abs(got - fp64)
    if name == "tails_4096":
        assert np.all(err <= 2e-4 + 2 * ulp(fp64))
    else:
        assert err.max() <= 1e-4, err.max()
        assert np.abs(got - ref).max() <= 2e-4


@pytest.mark.parametrize("name", CASES)
def test_sfu_ref_close_to_reference(gpu_ctx, name):
    book, ref, fp64 = load_golden(name)
    got = gpu_ctx.price_book(book, num_runs=1, mode="sfu_ref").astype(np.float64)
    tol = 1e-3 if name == "tails_4096" else 5e-4
    assert np.all(np.abs(got - fp64) <= tol + 4 * ulp(fp64))


@pytest.mark.parametrize("name", CASES)
def test_libm_ref_tracks_reference_bits(gpu_ctx, name):
    book, ref, _ = load_golden(name)
    got = gpu_ctx.price_book(book, num_runs=1, mode="libm_ref")
    diff = np.abs(got.astype(np.float64) - ref)
    # where glibc's expf/logf misround by an ulp, S or K times an ulp of
    # N(d) near 1 gives a few 1e-5 (S <= 200) or an ulp of S (tails)
    scale = np.maximum(book.sptprice, book.strike)
    assert np.all(diff <= 5e-5 + 4 * ulp(scale)), diff.max()
    same = np.mean(got.view(np.uint32) == ref.view(np.uint32))
    assert same >= 0.99, same


@pytest.mark.parametrize("dist", ["plain", "tails"])
def test_libm_ref_is_the_correctly_rounded_reference_order(gpu_ctx, oracle_lib, dist):
    """1M options: the float-float exp/log round as exp/log through double
    do (both correct to within near-midpoint cases), so the GPU's
    reference-order prices equal the CPU restatement's with correctly
    rounded exp/log, and the reference's own wherever glibc rounds
    correctly."""
    book = books.generate(1 << 20, seed=29, dist=dist)
    got = gpu_ctx.price_book(book, num_runs=1, mode="libm_ref")
    cr = oracle_lib.price_ref_cr(book)
    same_cr = np.mean(got.view(np.uint32) == cr.view(np.uint32))
    assert same_cr >= 0.9999, same_cr
    ref = oracle_lib.price_ref(book)
    same_ref = np.mean(got.view(np.uint32) == ref.view(np.uint32))
    assert same_ref >= 0.99, same_ref
    # where they differ, an ulp of N(d) or of e^{-rT} is multiplied by S or
    # K, so the bound scales with max(S, K), not with the (possibly small)
    # price
    finite = np.isfinite(ref)
    scale = np.maximum(book.sptprice, book.strike)[finite]
    diff = np.abs(got[finite].astype(np.float64) - ref[finite])
    assert np.all(diff <= 5e-5 + 4 * ulp(scale)), diff.max()


@pytest.mark.parametrize("name", CASES)
def test_fp64_kernel_matches_cpu_oracle(gpu_ctx, name):
    book, _, fp64 = load_golden(name)
    out = np.empty(len(book), dtype=np.float64)
    gpu_ctx.price_fp64(*book.arrays(), out)
    np.testing.assert_allclose(out, fp64, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 9, 31, 127, 128, 129, 1023, 4099, 65537, 100003])
def test_ragged_sizes_equal_bits_of_a_big_run(gpu_ctx, n):
    """A prefix priced alone equals the same options priced in a larger call
    (vector body, ragged tail and scalar paths compute the same bits)."""
    book = books.generate(131072, seed=11)
    full = gpu_ctx.price_book(book)
    part = gpu_ctx.price_book(book.slice(0, n))
    assert np.array_equal(part.view(np.uint32), full[:n].view(np.uint32))


def test_empty_and_zero_runs(gpu_ctx):
    book = books.generate(0, seed=1)
    out = np.empty(0, dtype=np.float32)
    gpu_ctx.price_soa(*book.arrays(), out, n=0, num_runs=100)
    book = books.generate(10, seed=1)
    out = np.full(10, -7.0, dtype=np.float32)
    gpu_ctx.price_soa(*book.arrays(), out, num_runs=0)
    assert np.all(out == -7.0)


def test_num_runs_graph_equals_single_run(gpu_ctx):
    book = books.generate(300001, seed=12)
    one = gpu_ctx.price_book(book, num_runs=1)
    hundred = gpu_ctx.price_book(book, num_runs=100)
    out = np.empty(len(book), dtype=np.float32)
    gpu_ctx.price_soa(*book.arrays(), out, num_runs=7, graph=False)
    assert np.array_equal(one.view(np.uint32), hundred.view(np.uint32))
    assert np.array_equal(one.view(np.uint32), out.view(np.uint32))


def _dev(torch, book, pad=0):
    arrs = []
    for a in book.arrays():
        t = torch.zeros(len(a) + pad, dtype=torch.float32 if a.dtype == np.float32 else torch.int32,
                        device="cuda:0")
        t[pad:] = torch.from_numpy(a).cuda()
        arrs.append(t)
    return arrs


@pytest.mark.parametrize("mode", ["fast", "sfu_ref", "libm_ref"])
def test_device_pointers_and_misaligned_scalar_path(gpu_ctx, mode):
    """Pointers offset by 1 or 3 floats take the scalar kernel (one option
    per thread, scalar arithmetic); aligned ones the vector kernel (packed
    f32x2 arithmetic in the fast and libm modes): every mode gives the same
    bits either way -- a packed product fused into a packed add would not."""
    torch = pytest.importorskip("torch")
    book = books.generate(50001, seed=13, dist="tails")
    host = gpu_ctx.price_book(book, mode=mode)
    for pad in (0, 1, 3):
        d = _dev(torch, book, pad)
        out = torch.zeros(len(book) + pad, dtype=torch.float32, device="cuda:0")
        views = [x[pad:] for x in d]
        torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
        gpu_ctx.price_soa(*views, out[pad:], n=len(book), num_runs=2, mode=mode, device=True)
        torch.cuda.synchronize()
        got = out[pad:].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), host.view(np.uint32)), pad


def test_all_tunings_give_identical_bits(gpu_ctx):
    book = books.generate(200003, seed=14)
    base = gpu_ctx.price_book(book)
    saved = gpu_ctx.get_tune()
    try:
        for lp in (0, 1, 2, 3, 4, 5, 6, 7, 8):
            for vpt in (1, 2, 4):
                if lp >= 2 and vpt == 4:
                    continue
                for block in (128, 256, 512):
                    for bps, pdl in ((0, 0), (4, 0), (0, 1), (4, 1)):
                        gpu_ctx.set_tune(vpt, block, bps, lp, pdl)
                        got = gpu_ctx.price_book(book, num_runs=3)
                        assert np.array_equal(got.view(np.uint32), base.view(np.uint32)), (lp, vpt, block, bps, pdl)
    finally:
        gpu_ctx.set_tune(**saved)


def test_resident_prefix_path_on_a_book_larger_than_l2(gpu_ctx):
    """Load path 7 keeps a prefix of the book (a tuned number of 32nds of
    the L2) resident and streams the rest: on a 4M-option book (112 MB) both
    parts, and the boundary between them, give the bits of the plain path
    for every prefix size the tuning accepts."""
    book = books.generate(4_000_001, seed=16)
    saved = gpu_ctx.get_tune()
    try:
        gpu_ctx.set_tune(1, 256, 0, 0, 0)
        base = gpu_ctx.price_book(book, num_runs=1)
        for vpt, block, bps, pdl in ((1, 256, 0, 1), (2, 512, 4, 1), (1, 128, 8, 0)):
            for r32 in (0, 1, 8, 15, 24):
                gpu_ctx.set_tune(vpt, block, bps, 7, pdl, r32)
                assert gpu_ctx.get_tune()["resident_32nds"] == (r32 or 15)
                got = gpu_ctx.price_book(book, num_runs=3)
                assert np.array_equal(got.view(np.uint32), base.view(np.uint32)), \
                    (vpt, block, bps, pdl, r32)
    finally:
        gpu_ctx.set_tune(**saved)


def test_alternating_path_every_pass_count(gpu_ctx):
    """Load path 8 walks odd passes from the last tile to the first: any
    number of passes, on a book larger than the L2 and on a ragged small
    one, gives the bits of the plain path."""
    saved = gpu_ctx.get_tune()
    try:
        for n in (4_000_003, 1001):
            book = books.generate(n, seed=17)
            gpu_ctx.set_tune(1, 256, 0, 0, 0)
            base = gpu_ctx.price_book(book, num_runs=1)
            for vpt, block, bps, pdl in ((1, 128, 4, 1), (2, 256, 0, 1), (1, 512, 2, 0)):
                gpu_ctx.set_tune(vpt, block, bps, 8, pdl)
                for runs in (1, 2, 3, 100):
                    got = gpu_ctx.price_book(book, num_runs=runs)
                    assert np.array_equal(got.view(np.uint32), base.view(np.uint32)), \
                        (n, vpt, block, bps, pdl, runs)
    finally:
        gpu_ctx.set_tune(**saved)


def test_out_of_range_device_arguments_are_errors(gpu_ctx):
    """A size larger than the allocation is refused on the host before any
    kernel runs; the context stays usable.  (torch sub-allocates from larger
    driver allocations, so the overrun is made far larger than any segment.)"""
    torch = pytest.importorskip("torch")
    from p3arsec_gb300.abi import BsgError
    book = books.generate(1000, seed=15)
    d = _dev(torch, book)
    out = torch.zeros(1000, dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
    with pytest.raises(BsgError) as e:
        gpu_ctx.price_soa(*d, out, n=1000 + (1 << 30), device=True)
    assert e.value.status == -1
    host = np.zeros(4, dtype=np.float32)
    with pytest.raises(BsgError):
        gpu_ctx.price_soa(*d, host, n=4, device=True)  # host pointer as device
    with pytest.raises(BsgError) as e:
        big = books.generate(gpu_ctx.max_options + 1, seed=1)
        gpu_ctx.price_book(big)
    assert e.value.status == -5
    gpu_ctx.price_soa(*d, out, n=1000, device=True)  # still fine


def test_reference_batch_signature(gpu_ctx):
    from p3arsec_gb300 import BlkSchlsEqEuroNoDiv
    book, ref, fp64 = load_golden("plain_4096")
    out = np.zeros(len(book), dtype=np.float32)
    BlkSchlsEqEuroNoDiv(out, len(book), *book.arrays(), 0.0)
    assert np.abs(out - fp64).max() <= 1e-4


@pytest.mark.parametrize("name", CASES)
def test_fp64_product_mode_tracks_reference_simd_double(gpu_ctx, name):
    import os
    import oracle
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    book, _, _ = load_golden(name)
    wide = oracle.widened(book)
    out = np.zeros(len(book), dtype=np.float64)
    gpu_ctx.price_soa_f64(*wide, book.otype, out, num_runs=3)
    np.testing.assert_allclose(out, z["simd2_prices"], rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("name", ["plain_4096", "edge"])
def test_fast_vs_reference_simd_float(gpu_ctx, name):
    import os
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    book, _, _ = load_golden(name)
    got = gpu_ctx.price_book(book)
    assert np.abs(got.astype(np.float64) - z["simd4_prices"]).max() <= 2e-4


def test_fp64_product_mode_device_pointers(gpu_ctx):
    torch = pytest.importorskip("torch")
    import oracle
    book = books.generate(100003, seed=17, dist="tails")
    wide = [torch.from_numpy(a).cuda() for a in oracle.widened(book)]
    ot = torch.from_numpy(book.otype).cuda()
    out = torch.empty(len(book), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()  # torch's copies and fills are done before the context's stream runs
    gpu_ctx.price_soa_f64(*wide, ot, out, n=len(book), device=True)
    torch.cuda.synchronize()
    want = oracle.price_fp64(book)
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("n", [2047, 2048, 2049, 4096 * 152 + 5, 1000003])
def test_bulk_staged_path_bits_and_tails(gpu_ctx, n):
    """The TMA bulk-staged kernel (load path 3): whole tiles through the
    shared-memory ring, the rest per option; sizes below one tile fall back to
    256-bit loads.  Same bits as the default path."""
    book = books.generate(n, seed=71)
    base = gpu_ctx.price_book(book)
    saved = gpu_ctx.get_tune()
    try:
        for lp in (3, 4, 5):
            for pdl in (0, 1):
                gpu_ctx.set_tune(1, 256, 0, lp, pdl)
                got = gpu_ctx.price_book(book, num_runs=5)
                assert np.array_equal(got.view(np.uint32), base.view(np.uint32)), (lp, pdl)
    finally:
        gpu_ctx.set_tune(**saved)


def test_concurrent_threads_share_a_context_and_own_contexts(gpu_ctx):
    """Calls on one context are serialised by its lock; separate contexts run
    side by side.  Every thread gets the bits a lone call gets."""
    import threading
    from p3arsec_gb300 import Context
    book = books.generate(200003, seed=91)
    want = gpu_ctx.price_book(book)
    errors = []

    def worker(ctx):
        try:
            for _ in range(5):
                got = ctx.price_book(book, num_runs=2)
                if not np.array_equal(got.view(np.uint32), want.view(np.uint32)):
                    errors.append("mismatch")
        except Exception as e:  # noqa: BLE001
            errors.append(repr(e))

    own = [Context(0, 1 << 18) for _ in range(2)]
    threads = [threading.Thread(target=worker, args=(c,)) for c in [gpu_ctx] * 3 + own]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for c in own:
        c.close()
    assert not errors, errors


def test_unknown_flag_bits_are_rejected(gpu_ctx):
    book = books.generate(100, seed=92)
    out = np.zeros(100, dtype=np.float32)
    st = gpu_ctx.lib.bsg_price_soa(gpu_ctx.h, *[a.ctypes.data for a in book.arrays()],
                                   out.ctypes.data, 100, 1, 0x8000)
    assert st == -1


def test_pipelined_host_calls_equal_synchronous_calls(gpu_ctx):
    """BSG_ASYNC with host pointers: calls alternate between two resident sets
    and overlap copies with passes; every result equals a lone call's."""
    torch = pytest.importorskip("torch")
    bks = [books.generate(n, seed=100 + i) for i, n in enumerate((300001, 4, 1 << 20, 77777, 1))]
    want = [gpu_ctx.price_book(b) for b in bks]
    pinned = [[torch.from_numpy(a).pin_memory().numpy() for a in b.arrays()] for b in bks]
    outs = [torch.zeros(len(b), dtype=torch.float32).pin_memory().numpy() for b in bks]
    for rep in range(2):
        for arrs, out in zip(pinned, outs):
            gpu_ctx.price_soa(*arrs, out, n=len(out), num_runs=3, asynchronous=True)
        gpu_ctx.synchronize()
        for w, o in zip(want, outs):
            assert np.array_equal(o.view(np.uint32), w.view(np.uint32)), rep
    # a synchronous call after pipelined ones drains them first
    gpu_ctx.price_soa(*pinned[0], outs[0], n=len(outs[0]), num_runs=1, asynchronous=True)
    again = gpu_ctx.price_book(bks[2])
    assert np.array_equal(again.view(np.uint32), want[2].view(np.uint32))
    gpu_ctx.synchronize()
    assert np.array_equal(outs[0].view(np.uint32), want[0].view(np.uint32))


@pytest.mark.parametrize("mode", ["fast", "sfu_ref", "libm_ref"])
def test_degenerate_inputs_follow_the_reference(gpu_ctx, mode):
    """Expiry (t = 0), zero and extreme volatility, zero prices, underflowing
    discount, overflowing S/K, negative t and NaN inputs: NaN exactly where
    the reference's own prices (tests/golden/degenerate.npz) are NaN, and the
    finite prices within 1e-4 + 1e-6 |price|, at every vector-lane offset."""
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "degenerate.npz"))
    book = books.Book(d["sptprice"], d["strike"], d["rate"], d["volatility"], d["otime"],
                      d["otype"])
    ref = d["ref_prices"].astype(np.float64)
    for shift in range(8):
        b = books.Book(*(np.roll(x, shift) for x in book.arrays()))
        got = np.roll(gpu_ctx.price_book(b, mode=mode).astype(np.float64), -shift)
        assert np.array_equal(np.isnan(got), np.isnan(ref)), (mode, shift, got, ref)
        fin = ~np.isnan(ref)
        tol = 1e-4 + 1e-6 * np.abs(ref[fin])
        assert np.all(np.abs(got[fin] - ref[fin]) <= tol), (mode, shift, got[fin] - ref[fin])
