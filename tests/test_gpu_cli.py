"""The drop-in CLI: reference argv and file formats, priced on the GPU."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from p3arsec_gb300 import books, build

pytestmark = pytest.mark.gpu


def test_cli_round_trip(tmp_path):
    build.build()
    book = books.generate(20000, seed=31)
    fp64 = oracle.price_fp64(book)
    inp = tmp_path / "in.txt"
    out = tmp_path / "out.txt"
    books.write_parsec_input(inp, book, dgrefval=fp64)
    env = dict(os.environ, BSG_ERR_CHK="1", BSG_NUM_RUNS="5")
    r = subprocess.run([build.CLI, "8", str(inp), str(out)], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stdout
    assert "Num of Options: 20000" in r.stdout and "Num of Runs: 5" in r.stdout
    assert "roi.time|" in r.stdout
    assert "Num Errors: 0" in r.stdout
    got = books.read_parsec_output(out)
    assert np.abs(got.astype(np.float64) - fp64).max() <= 1e-4


def test_cli_bad_input_exits_1(tmp_path):
    build.build()
    bad = tmp_path / "bad.txt"
    bad.write_text("5\n1 2\n")
    r = subprocess.run([build.CLI, "1", str(bad), str(tmp_path / "o.txt")],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=60)
    assert r.returncode == 1 and "ERROR" in r.stdout


# ------------------------------------------------------------ swaptions CLI
def _swaptions_cli(*args, timeout=120):
    build.build()
    return subprocess.run([build.SWAPTIONS_CLI, *args], stdout=subprocess.PIPE,
                          stderr=subprocess.PIPE, text=True, timeout=timeout)


def test_swaptions_cli_prices_like_the_oracle():
    """The swaptions drop-in (HJM_Securities.cpp's main): reference options and
    output lines; every printed price and standard error equals the CPU
    oracle's on the same swaption set and paths (to the 10 decimals printed
    and the oracle's tolerance)."""
    from p3arsec_gb300 import swaptions as S
    r = _swaptions_cli("-ns", "6", "-sm", "20000", "-nt", "2", "-sd", "7")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Number of Simulations: 20000,  Number of threads: 2 Number of swaptions: 6" in r.stdout
    assert "roi.time|" in r.stdout
    lines = [l for l in r.stderr.splitlines() if l.startswith("Swaption ")]
    assert len(lines) == 6
    got = np.array([[float(x) for x in l.split("SwaptionPrice: ")[1].split(" StdError: ")[0:1]]
                    + [float(l.split("StdError: ")[1].rstrip("] "))] for l in lines])
    want, want_err, _ = oracle.swaptions_all(S.generate_cli(6, seed=7), 20000, 4)
    assert np.allclose(got[:, 0], want, rtol=1e-10, atol=1e-9)
    assert np.allclose(got[:, 1], want_err, rtol=1e-6, atol=1e-9)


def test_cli_at_two_million_options(tmp_path):
    """The drop-in at scale: a 2M-option PARSEC file (~150 MB, split across
    the parser's threads) through the CLI with the reference's ERR_CHK
    against FP64 DGrefval, and the printed prices against the FP64 oracle."""
    build.build()
    n = 1 << 21
    book = books.generate(n, seed=37)
    fp64 = oracle.price_fp64(book)
    inp = tmp_path / "in.txt"
    out = tmp_path / "out.txt"
    books.write_parsec_input(inp, book, dgrefval=fp64)
    env = dict(os.environ, BSG_ERR_CHK="1", BSG_NUM_RUNS="3")
    r = subprocess.run([build.CLI, "16", str(inp), str(out)], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stdout
    assert f"Num of Options: {n}" in r.stdout and "Num Errors: 0" in r.stdout
    got = books.read_parsec_output(out)
    assert got.shape == (n,)
    assert np.abs(got.astype(np.float64) - fp64).max() <= 1e-4
