"""The CPU oracle against the reference's golden outputs (no GPU)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from p3arsec_gb300 import books

CASES = ["plain_4096", "tails_4096", "edge"]


@pytest.mark.parametrize("name", CASES)
def test_fp32_restatement_is_bit_identical_to_reference(oracle_lib, name):
    book, ref, _ = load_golden(name)
    got = oracle_lib.price_ref(book)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("name", CASES)
def test_fp64_oracle_matches_fixture(oracle_lib, name):
    book, _, fp64 = load_golden(name)
    got = oracle_lib.price_fp64(book)
    np.testing.assert_allclose(got, fp64, rtol=1e-12, atol=1e-12)


def test_cndf_bit_identical_to_reference(oracle_lib):
    z = np.load(os.path.join(GOLDEN, "cndf.npz"))
    got = oracle_lib.cndf_ref(z["x"])
    assert np.array_equal(got.view(np.uint32), z["ref"].view(np.uint32))


def test_reference_accuracy_recorded():
    """The reference's own FP32 error vs FP64 (what the GPU must not exceed)."""
    meta = json.load(open(os.path.join(GOLDEN, "golden.json")))
    assert meta["plain_4096"]["ref_vs_fp64_max_abs"] < 1e-4
    assert meta["plain_4096"]["err_chk_num_errors"] == 0
    # FastFlow / OpenMP / serial reference builds write identical files
    for name in CASES:
        cli = meta[name]["cli"]
        shas = {v for k, v in cli.items() if not k.endswith("matches_so")}
        assert len(shas) == 1
        assert all(v for k, v in cli.items() if k.endswith("matches_so"))


def test_known_answers(oracle_lib):
    L = oracle_lib.lib()
    assert L.bso_cndf_fp64(0.0) == pytest.approx(0.5, abs=1e-9)
    for x in (0.1, 0.7, 1.3, 2.9, 5.0):
        assert L.bso_cndf_fp64(x) + L.bso_cndf_fp64(-x) == pytest.approx(1.0, abs=1e-15)
    # put-call parity: C - P = S - K e^{-rT}
    for s, k, r, v, t in ((100, 100, 0.05, 0.2, 1.0), (50, 80, 0.01, 0.6, 0.3), (190, 95, 0.1, 0.05, 2.0)):
        c = L.bso_price_fp64(s, k, r, v, t, 0)
        p = L.bso_price_fp64(s, k, r, v, t, 1)
        assert c - p == pytest.approx(s - k * np.exp(-r * t), abs=1e-9)
    # monotone in S (call up, put down) and in K (call down)
    s = np.linspace(50, 150, 101)
    calls = [L.bso_price_fp64(x, 100, 0.03, 0.3, 1.0, 0) for x in s]
    puts = [L.bso_price_fp64(x, 100, 0.03, 0.3, 1.0, 1) for x in s]
    assert np.all(np.diff(calls) > 0) and np.all(np.diff(puts) < 0)


@pytest.mark.parametrize("n,nw", [(10, 3), (65536, 8), (7, 7), (5, 8), (1, 1), (100003, 16)])
def test_static_partition_matches_fastflow_rule(oracle_lib, n, nw):
    nw_eff = min(nw, n)
    b, e = oracle_lib.static_partition(n, nw_eff)
    sizes = e - b
    assert b[0] == 0 and e[-1] == n
    assert np.all(b[1:] == e[:-1])
    q, r = divmod(n, nw_eff)
    assert np.all(sizes[:r] == q + 1) and np.all(sizes[r:] == q)


@pytest.mark.parametrize("nthreads", [1, 3, 8])
def test_threaded_map_equals_serial(oracle_lib, nthreads):
    book = books.generate(10007, seed=5)
    serial = oracle_lib.price_ref(book)
    got, secs = oracle_lib.bs_map(book, nthreads, 3)
    assert secs >= 0
    assert np.array_equal(got.view(np.uint32), serial.view(np.uint32))


def test_parsec_flags_build_prices_like_the_checker(oracle_lib):
    """The timed CPU baseline is the same restatement built with PARSEC's
    flags and the compiler's default contraction: bit-identical to the
    checker on x86-64 (no fused multiply-add there), within the reference's
    1e-4 check (blackscholes.c:333-339) where the compiler fuses."""
    import platform
    book = books.generate(200003, seed=23)
    chk, _ = oracle_lib.bs_map(book, 4, 1)
    got, secs = oracle_lib.bs_map(book, 4, 2, parsec_flags=True)
    assert secs >= 0
    if platform.machine() in ("x86_64", "AMD64"):
        assert np.array_equal(got.view(np.uint32), chk.view(np.uint32))
    assert np.abs(got.astype(np.float64) - chk).max() <= 1e-4


def test_threaded_map_empty_and_more_threads_than_options(oracle_lib):
    book = books.generate(0, seed=1)
    out, secs = oracle_lib.bs_map(book, 4, 2)
    assert out.shape == (0,) and secs == 0.0
    book = books.generate(3, seed=1)
    out, _ = oracle_lib.bs_map(book, 16, 1)
    assert np.array_equal(out.view(np.uint32), oracle_lib.price_ref(book).view(np.uint32))


def test_compiled_reference_agrees_when_present(oracle_lib):
    """Where the reference source tree exists, its .so equals the restatement
    on a fresh seeded book (1M options, both distributions)."""
    if oracle_lib.ref_lib() is None:
        import oracle
        oracle.build(ref=True)
    if oracle_lib.ref_lib() is None:
        pytest.skip("reference source tree not present on this machine")
    for dist in ("plain", "tails"):
        book = books.generate(1 << 20, seed=99, dist=dist)
        a = oracle_lib.price_reference(book)
        b = oracle_lib.price_ref(book)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("name", CASES)
def test_fp64_oracle_is_bit_identical_to_reference_simd_double(oracle_lib, name):
    """The reference's SIMD variant built with NCO = 2 computes the formula in
    double (blackscholes.simd.c:68-81); the FP64 oracle reproduces it."""
    import numpy as np
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    book, _, _ = load_golden(name)
    got = oracle_lib.price_fp64_d(*oracle_lib.widened(book), book.otype)
    assert np.array_equal(got.view(np.uint64), z["simd2_prices"].view(np.uint64))


def test_reference_simd_variants_agree_when_present(oracle_lib):
    if oracle_lib.price_reference_simd(books.generate(8, seed=1), 2) is None:
        pytest.skip("the SIMD variant is built only on x86-64 with the reference tree")
    book = books.generate(1 << 19, seed=98, dist="tails")
    s2 = oracle_lib.price_reference_simd(book, 2)
    assert np.array_equal(s2.view(np.uint64), oracle_lib.price_fp64(book).view(np.uint64))
    s4 = oracle_lib.price_reference_simd(book, 4)
    assert np.abs(s4.astype(np.float64) - s2).max() < 1e-3


def test_restatement_on_degenerate_inputs(oracle_lib):
    """Expiry, zero volatility, zero prices, overflow, negative t and NaN
    inputs: the restatement gives the compiled reference's prices bit for
    bit, NaN where it is NaN (tests/golden/degenerate.npz)."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "degenerate.npz"))
    book = books.Book(d["sptprice"], d["strike"], d["rate"], d["volatility"], d["otime"],
                      d["otype"])
    got = oracle_lib.price_ref(book)
    ref = d["ref_prices"]
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    fin = ~np.isnan(ref)
    assert np.array_equal(got[fin].view(np.uint32), ref[fin].view(np.uint32))
