"""The reference's file formats through libbsgpu.so's host I/O (no GPU).

Parity bar: byte-identical output files (the SHA-256 of the reference CLI's
own output for the golden cases) and bit-identical parsed arrays."""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from p3arsec_gb300 import abi, books

CASES = ["plain_4096", "tails_4096", "edge"]

_libc = ctypes.CDLL(None)


def c_f18(x: np.float32) -> bytes:
    buf = ctypes.create_string_buffer(128)
    _libc.snprintf(buf, 128, b"%.18f", ctypes.c_double(float(x)))
    return buf.value


@pytest.fixture(scope="module", autouse=True)
def built():
    from p3arsec_gb300 import build
    build.build()


@pytest.mark.parametrize("name", CASES)
def test_output_file_is_byte_identical_to_reference(name):
    _, ref, _ = load_golden(name)
    meta = json.load(open(os.path.join(GOLDEN, "golden.json")))
    want = meta[name]["cli"]["blackscholes_serial:1"]
    got = hashlib.sha256(abi.format_prices(ref)).hexdigest()
    assert got == want


def test_f18_matches_libc_on_random_and_edge_floats():
    rng = np.random.default_rng(0)
    bits = rng.integers(0, 2**32, 2_000_000, dtype=np.uint64).astype(np.uint32)
    x = bits.view(np.float32)
    x = x[np.isfinite(x) & (np.abs(x) < 1e12)]
    mags = np.concatenate([
        rng.uniform(0, 4000, 200_000), rng.uniform(0, 1e-6, 50_000),
        np.exp(rng.uniform(-60, 30, 200_000))]).astype(np.float32)
    ties = np.array([2.0 ** -k for k in range(15, 40)] + [3 * 2.0 ** -19, 5 * 2.0 ** -20],
                    dtype=np.float32)
    special = np.array([0.0, -0.0, 1.0, -1.0, 1e-45, -1e-45, 1.17549435e-38, 2.0 ** 40,
                        2.0 ** 40 - 65536, 3.4e38, -3.4e38, np.inf, -np.inf, np.nan, 0.5e-18,
                        1.5e-18, 5e-19, 123.456789, 0.1, 0.3], dtype=np.float32)
    allx = np.concatenate([x, mags, -mags[:1000], ties, special]).astype(np.float32)
    text = abi.format_prices(allx, nthreads=4).split(b"\n")
    assert text[0] == str(len(allx)).encode()
    lines = text[1:-1]
    assert len(lines) == len(allx)
    # check every special/tie value and a large sample of the rest against libc
    idx = np.concatenate([np.arange(len(allx) - len(ties) - len(special), len(allx)),
                          rng.choice(len(allx), 60_000, replace=False)])
    for i in idx:
        assert lines[i] == c_f18(allx[i]), (allx[i], lines[i], c_f18(allx[i]))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("threads", [1, 7])
def test_parse_is_bit_identical(tmp_path, name, threads):
    book, _, fp64 = load_golden(name)
    p = tmp_path / "in.txt"
    books.write_parsec_input(p, book, dgrefval=fp64)
    got, dg = abi.read_parsec(p, nthreads=threads)
    for a, b in zip(got.arrays(), book.arrays()):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    _, dg_py = books.read_parsec_input(p)
    assert np.array_equal(dg.view(np.uint32), dg_py.view(np.uint32))


def test_parse_odd_layouts():
    text = (b"0x3\n"                                   # %i: hex count
            b"  100 100 0.05 0 0.2 1.0 P 0 10.5\r\n"   # CRLF, leading spaces
            b"1.5e2\t9e1 5e-2 0 2.5E-1 0.5 C 0 1\n"    # tabs, exponents
            b"90 95 0.01 0 0.3 2 X 0\n 7\n"            # record over two lines, other type
            b"trailing garbage is ignored\n")
    for threads in (1, 4):
        book, dg = abi.parse_parsec(text, nthreads=threads)
        assert len(book) == 3
        np.testing.assert_array_equal(book.sptprice, np.float32([100, 150, 90]))
        np.testing.assert_array_equal(book.otype, np.int32([1, 0, 0]))
        np.testing.assert_array_equal(dg, np.float32([10.5, 1, 7]))
        assert book.volatility[1] == np.float32(0.25)


@pytest.mark.parametrize("text", [b"", b"abc", b"2\n1 2 3 0 0.2 1 C 0 0\n", b"1\n1 2 3 0 0.2 1\n"])
def test_parse_errors(text):
    with pytest.raises(abi.BsgError):
        abi.parse_parsec(text)


def test_empty_book_and_octal_count():
    book, _ = abi.parse_parsec(b"0\n")
    assert len(book) == 0
    book, _ = abi.parse_parsec(b"010\n" + b"1 1 0.01 0 0.1 1 C 0 0\n" * 8)
    assert len(book) == 8  # "%i" reads a leading 0 as octal


def test_soa_round_trip(tmp_path):
    book = books.generate(100003, seed=9)
    dg = np.arange(len(book), dtype=np.float32)
    p = tmp_path / "b.soa"
    abi.write_soa(p, book, dg)
    got, gdg = abi.read_soa(p)
    for a, b in zip(got.arrays(), book.arrays()):
        assert np.array_equal(a, b)
    assert np.array_equal(gdg, dg)
    with pytest.raises(abi.BsgError):
        abi.read_soa(tmp_path / "missing.soa")


def test_write_file(tmp_path):
    _, ref, _ = load_golden("edge")
    p = tmp_path / "out.txt"
    abi.write_parsec_prices(p, ref, nthreads=3)
    assert p.read_bytes() == abi.format_prices(ref, nthreads=1)
    assert np.array_equal(books.read_parsec_output(p), np.array(
        [float(x) for x in p.read_text().split()[1:]], dtype=np.float32))


def test_input_writer_round_trips(tmp_path):
    book = books.generate(50001, seed=12, dist="tails")
    dg = np.linspace(0, 3000, len(book)).astype(np.float32)
    p = tmp_path / "in.txt"
    abi.write_parsec_input(p, book, dg, nthreads=5)
    got, gdg = abi.read_parsec(p)
    for a, b in zip(got.arrays(), book.arrays()):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(gdg.view(np.uint32), dg.view(np.uint32))
    # and the Python reader (the reference's field layout) agrees
    pyb, _ = books.read_parsec_input(p)
    assert np.array_equal(pyb.strike.view(np.uint32), book.strike.view(np.uint32))


def test_parallel_io_equals_the_reference_sequential_io(tmp_path, oracle_lib):
    book = books.generate(20011, seed=13)
    fp64 = oracle_lib.price_fp64(book)
    p = tmp_path / "in.txt"
    abi.write_parsec_input(p, book, fp64)
    a, adg = abi.read_parsec(p, nthreads=4)
    b, bdg = oracle_lib.read_parsec_fscanf(p, len(book))
    for x, y in zip(a.arrays(), b.arrays()):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    assert np.array_equal(adg.view(np.uint32), bdg.view(np.uint32))
    prices = oracle_lib.price_ref(book)
    o1, o2 = tmp_path / "o1.txt", tmp_path / "o2.txt"
    abi.write_parsec_prices(o1, prices, nthreads=4)
    oracle_lib.write_prices_fprintf(o2, prices)
    assert o1.read_bytes() == o2.read_bytes()


def _tokens(rng, count):
    """Decimal tokens of every shape the parser's fast path handles or must
    hand to strtof: random floats and doubles at 1-20 significant digits,
    float midpoints (ties in double, not always in decimal), integers, tiny
    and huge magnitudes, signs, leading zeros, exponent forms."""
    out = []
    f = rng.standard_normal(count).astype(np.float32) * np.float32(10.0) ** rng.integers(-12, 12, count)
    for i, x in enumerate(f):
        prec = int(rng.integers(1, 21))
        out.append(("%." + str(prec) + ("g" if i % 3 else "e")) % float(x))
    # midpoints between adjacent floats, printed with enough digits to be exact
    # in double and with digits that break the tie either way
    base = (rng.random(count // 4) * 1e4).astype(np.float32)
    nxt = np.nextafter(base, np.float32(np.inf))
    mids = (base.astype(np.float64) + nxt.astype(np.float64)) / 2
    for m in mids:
        out += ["%.17g" % m, "%.25g" % m, "%.9g" % m, repr(float(m)) + "1", repr(float(m))[:-1]]
    out += ["0", "-0", "-0.0", "000123.4500", "+7", ".5", "5.", "1e5", "1E-5", "2.5e+03",
            "123456789012345678901", "0.000000000000000000012345", "3.4028235e38", "1e39",
            "1.17549435e-38", "1e-45", "9007199254740993", "16777217", "0.1", "0.30000001"]
    return out


@pytest.mark.parametrize("threads", [1, 5])
def test_parse_every_float_shape_like_strtof(threads):
    rng = np.random.default_rng(77)
    toks = _tokens(rng, 24000)
    _libc.strtof.restype = ctypes.c_float
    _libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    want = np.array([_libc.strtof(t.encode(), None) for t in toks], dtype=np.float32)
    # pack the tokens into records: 8 float fields (plus the type letter) per line
    per = 8
    n = len(toks) // per
    lines = [str(n)]
    for r in range(n):
        t = toks[r * per:(r + 1) * per]
        lines.append(" ".join(t[:6] + ["C"] + t[6:]))
    book, dg = abi.parse_parsec(("\n".join(lines) + "\n").encode(), nthreads=threads)
    got = np.stack([book.sptprice, book.strike, book.rate, np.zeros(n, np.float32),
                    book.volatility, book.otime], axis=1)
    ref = want[:n * per].reshape(n, per)
    cols = [0, 1, 2, 4, 5]  # the fields the book keeps (divq is read and dropped)
    assert np.array_equal(got[:, cols].view(np.uint32), ref[:, cols].view(np.uint32))
    assert np.array_equal(dg.view(np.uint32), ref[:, 7].view(np.uint32))
