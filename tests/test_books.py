"""Seeded books and the PARSEC text formats (no GPU)."""
import numpy as np
import pytest

from p3arsec_gb300 import books


def test_generate_deterministic_and_in_range():
    a = books.generate(50000, seed=3)
    b = books.generate(50000, seed=3)
    for x, y in zip(a.arrays(), b.arrays()):
        assert np.array_equal(x, y)
    assert a.sptprice.dtype == np.float32 and a.otype.dtype == np.int32
    assert 10 <= a.sptprice.min() and a.sptprice.max() <= 200
    ratio = a.strike.astype(np.float64) / a.sptprice
    assert 0.5 - 1e-6 <= ratio.min() and ratio.max() <= 1.5 + 1e-6
    assert 0.01 <= a.rate.min() and a.rate.max() <= 0.10
    assert 0.05 <= a.volatility.min() and a.volatility.max() <= 0.65
    assert 0.05 <= a.otime.min() and a.otime.max() <= 2.0
    assert 0.45 < a.otype.mean() < 0.55


def test_tails_distribution():
    a = books.generate(50000, seed=4, dist="tails")
    ratio = a.strike.astype(np.float64) / a.sptprice
    assert ratio.min() < 0.1 and ratio.max() > 15
    assert a.otime.min() < 0.01 and a.otime.max() > 4.9


def test_parsec_text_round_trip(tmp_path):
    a = books.generate(1000, seed=8)
    ref = np.linspace(0, 50, 1000)
    p = tmp_path / "in.txt"
    books.write_parsec_input(p, a, dgrefval=ref)
    b, dg = books.read_parsec_input(p)
    for x, y in zip(a.arrays(), b.arrays()):
        assert np.array_equal(x, y)
    np.testing.assert_allclose(dg, ref.astype(np.float32), rtol=1e-7)


def test_parsec_output_round_trip(tmp_path):
    p = tmp_path / "out.txt"
    prices = np.array([1.5, 0.0, 123.456789, 1e-3], dtype=np.float32)
    books.write_parsec_output(p, prices)
    text = p.read_text().splitlines()
    assert text[0] == "4" and text[1] == "1.500000000000000000"
    assert np.array_equal(books.read_parsec_output(p), prices)


def test_truncated_input_raises(tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("3\n1 2 3 0 0.2 1 C 0 0\n")
    with pytest.raises(ValueError):
        books.read_parsec_input(p)
