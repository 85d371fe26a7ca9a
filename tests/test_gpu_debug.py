"""Debug guards (BSG_DEBUG): every resident array of a context is followed by
guard words that each synchronous call checks.  Clean calls of every size and
path leave them intact (no kernel or copy writes past n, ragged tails
included) and give bit-identical prices to a context without guards; a planted
overwrite, made inside the context's own allocation by the self-test, is
reported as BSG_ERR_STATE and the context stays usable."""
import numpy as np
import pytest

import oracle
from p3arsec_gb300 import abi, books

pytestmark = pytest.mark.gpu

CAP = 10007  # not a multiple of 4, 8 or 64


@pytest.fixture
def debug_ctx(monkeypatch):
    monkeypatch.setenv("BSG_DEBUG", "1")
    ctx = abi.Context(0, CAP)
    monkeypatch.delenv("BSG_DEBUG")
    yield ctx
    ctx.close()


@pytest.fixture(scope="module")
def plain_ctx():
    ctx = abi.Context(0, CAP)
    yield ctx
    ctx.close()


@pytest.mark.parametrize("mode", ["fast", "sfu_ref", "libm_ref"])
def test_guards_stay_intact_on_every_size(debug_ctx, plain_ctx, mode):
    book = books.generate(CAP, seed=91, dist="tails")
    for n in (1, 3, 4, 5, 7, 8, 9, 63, 64, 65, 1000, 4097, CAP - 1, CAP):
        sub = book.slice(0, n)
        got = debug_ctx.price_book(sub, num_runs=3, mode=mode)
        want = plain_ctx.price_book(sub, num_runs=3, mode=mode)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), n
    # a large call then a small one: the small call's check covers the
    # prices the large one left past its n
    debug_ctx.price_book(book, mode=mode)
    debug_ctx.price_book(book.slice(0, 5), mode=mode)


def test_guards_on_every_tune(debug_ctx):
    book = books.generate(CAP, seed=92)
    want = oracle.price_fp64(book)
    for tune in ((1, 256, 0, 0, 0), (2, 128, 2, 1, 1), (1, 256, 2, 2, 1),
                 (1, 256, 0, 3, 1), (1, 256, 0, 4, 1), (1, 256, 0, 5, 0),
                 (2, 128, 4, 6, 1)):
        debug_ctx.set_tune(*tune)
        for n in (CAP, 4099, 17):
            got = debug_ctx.price_book(book.slice(0, n), num_runs=2)
            assert np.abs(got.astype(np.float64) - want[:n]).max() <= 1e-4, (tune, n)


def test_guards_on_pipelined_and_fp64_calls(debug_ctx, plain_ctx):
    book = books.generate(CAP, seed=93)
    outs = []
    for n in (CAP, 777, 5000, 33):
        sub = book.slice(0, n)
        o = np.empty(n, dtype=np.float32)
        debug_ctx.price_soa(*sub.arrays(), o, n=n, num_runs=2, asynchronous=True)
        outs.append((sub, o))
    debug_ctx.synchronize()
    for sub, o in outs:
        assert np.array_equal(o, plain_ctx.price_book(sub, num_runs=2))
    d = np.empty(CAP, dtype=np.float64)
    debug_ctx.price_fp64(*book.arrays(), d)
    assert np.abs(d - oracle.price_fp64(book)).max() <= 1e-9


def test_planted_overwrite_is_reported(debug_ctx):
    st, msg = debug_ctx.selftest_guard()
    assert st == -11  # BSG_ERR_STATE
    assert "prices[" in msg and "guard" in msg
    # the self-test restored the word: ordinary calls pass again
    book = books.generate(1000, seed=94)
    got = debug_ctx.price_book(book)
    assert np.abs(got.astype(np.float64) - oracle.price_fp64(book)).max() <= 1e-4


def test_selftest_guard_needs_debug(plain_ctx):
    st, _ = plain_ctx.selftest_guard()
    assert st == -10  # BSG_ERR_NOT_SUPPORTED
