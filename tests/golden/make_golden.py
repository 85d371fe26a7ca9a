"""Generate the golden fixtures from the reference's own blackscholes.

Run in a checkout where the reference source tree is present (it is compiled
by oracle/Makefile into oracle/_ref/):

    python tests/golden/make_golden.py

For each seeded case it stores the float32 inputs, the prices of the
reference's own BlkSchlsEqEuroNoDiv (bits), and the FP64 same-formula oracle,
and it runs the reference CLI (serial, FastFlow, OpenMP and SkePU2-OpenMP
builds) on the PARSEC
text file and records the SHA-256 of each output file and the ERR_CHK count
against an FP64-filled DGrefval column.  Fixtures are small (.npz + .json).
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from p3arsec_gb300 import books  # noqa: E402

import oracle  # noqa: E402

REF_DIR = os.path.join(ROOT, "oracle", "_ref")


def edge_book() -> books.Book:
    """Hand-picked options: at the money, deep in/out of the money, tiny and
    long maturities, tiny and large volatility, zero rate, both types."""
    rows = []
    for ot in (0, 1):
        for s, k in ((100, 100), (100, 50), (100, 150), (10, 200), (200, 10), (100, 99.99),
                     (50.5, 50.5), (199.9, 100.1)):
            for r in (0.0, 0.01, 0.1):
                for v in (0.01, 0.05, 0.3, 0.65, 1.5):
                    for t in (0.001, 0.05, 0.5, 2.0, 5.0):
                        rows.append((s, k, r, v, t, ot))
    a = np.array(rows, dtype=np.float64)
    f = np.float32
    return books.Book(a[:, 0].astype(f), a[:, 1].astype(f), a[:, 2].astype(f),
                      a[:, 3].astype(f), a[:, 4].astype(f), a[:, 5].astype(np.int32))


# Degenerate but finite inputs the reference prices without faulting:
# expiry (t = 0), zero and extreme volatility, zero rate and price, tiny t,
# a discount factor that underflows, S/K overflowing float, and negative t
# or NaN inputs (the reference returns NaN).  Rows: S, K, r, v, t, otype.
DEGENERATE = [
    (100, 100, 0.05, 0.3, 0.0, 0), (100, 100, 0.05, 0.3, 0.0, 1),
    (100, 90, 0.05, 0.3, 0.0, 0), (100, 110, 0.05, 0.3, 0.0, 1),
    (90, 100, 0.05, 0.3, 0.0, 0), (110, 100, 0.05, 0.3, 0.0, 1),
    (100, 100, 0.05, 0.0, 1.0, 0), (100, 90, 0.05, 0.0, 1.0, 0),
    (100, 110, 0.05, 0.0, 1.0, 1), (100, 100, 0.0, 0.3, 1.0, 0),
    (100, 100, 0.05, 0.3, -1.0, 0), (float("nan"), 100, 0.05, 0.3, 1, 0),
    (100, 100, 0.05, float("nan"), 1, 1), (100, float("nan"), 0.05, 0.3, 1, 0),
    (0.0, 100, 0.05, 0.3, 1, 0), (0.0, 100, 0.05, 0.3, 1, 1),
    (100, 0.0, 0.05, 0.3, 1, 1), (100, 100, 0.05, 0.3, 1e-30, 0),
    (100, 100, 0.05, 1e-20, 1.0, 0), (100, 100, 0.05, 50.0, 1.0, 0),
    (100, 100, 0.05, 50.0, 1.0, 1), (100, 100, 5.0, 0.3, 100.0, 0),
    (100, 100, 5.0, 0.3, 100.0, 1), (1e30, 1e-30, 0.05, 0.3, 1, 0),
    (1e-30, 1e30, 0.05, 0.3, 1, 1),
]


def degenerate_book() -> books.Book:
    a = np.array(DEGENERATE, dtype=np.float64)
    f = np.float32
    return books.Book(a[:, 0].astype(f), a[:, 1].astype(f), a[:, 2].astype(f),
                      a[:, 3].astype(f), a[:, 4].astype(f), a[:, 5].astype(np.int32))


CASES = {
    "plain_4096": lambda: books.generate(4096, seed=20240101, dist="plain"),
    "tails_4096": lambda: books.generate(4096, seed=20240102, dist="tails"),
    "edge": edge_book,
}


def sha256(path):
    h = hashlib.sha256()
    with open(path, "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def run_cli(binary, nthreads, inp, out):
    r = subprocess.run([os.path.join(REF_DIR, binary), str(nthreads), inp, out],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, check=True)
    return r.stdout


def main():
    oracle.build(ref=True)
    if oracle.ref_lib() is None or oracle.price_reference_simd(CASES["edge"](), 2) is None:
        raise SystemExit("the reference could not be built (source tree absent, or not x86-64)")
    meta = {}
    for name, make in CASES.items():
        book = make()
        ref = oracle.price_reference(book)
        fp64 = oracle.price_fp64(book)
        # the reference's SIMD variant (blackscholes.simd.c): NCO = 4 (SSE
        # float) and NCO = 2 (SSE2 double, inputs widened to double)
        simd4 = oracle.price_reference_simd(book, 4)
        simd2 = oracle.price_reference_simd(book, 2)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"),
                            sptprice=book.sptprice, strike=book.strike, rate=book.rate,
                            volatility=book.volatility, otime=book.otime, otype=book.otype,
                            ref_prices=ref, fp64_prices=fp64, simd4_prices=simd4,
                            simd2_prices=simd2)
        info = {"n": len(book), "cli": {},
                "simd2_equals_fp64_oracle_bitwise": bool(np.array_equal(
                    simd2.view(np.uint64), fp64.view(np.uint64))),
                "simd4_vs_scalar_max_abs": float(np.abs(simd4.astype(np.float64) - ref).max())}
        with tempfile.TemporaryDirectory() as td:
            inp = os.path.join(td, "in.txt")
            books.write_parsec_input(inp, book, dgrefval=fp64)
            for binary, nthr in (("blackscholes_serial", 1), ("blackscholes_ff", 4),
                                 ("blackscholes_omp", 4), ("blackscholes_skepu_omp", 4)):
                out = os.path.join(td, f"{binary}.txt")
                run_cli(binary, nthr, inp, out)
                info["cli"][f"{binary}:{nthr}"] = sha256(out)
                got = books.read_parsec_output(out)
                # the CLI (text in, %.18f out) agrees with the .so on the same floats
                same = np.array_equal(np.char.mod("%.18f", got.astype(np.float64)),
                                      np.char.mod("%.18f", ref.astype(np.float64)))
                info["cli"][f"{binary}:{nthr}:matches_so"] = bool(same)
            log = run_cli("blackscholes_serial_chk", 1, inp, os.path.join(td, "chk.txt"))
            line = [x for x in log.splitlines() if x.startswith("Num Errors:")]
            info["err_chk_num_errors"] = int(line[0].split(":")[1]) if line else None
        info["ref_vs_fp64_max_abs"] = float(np.max(np.abs(ref.astype(np.float64) - fp64)))
        meta[name] = info
        print(name, json.dumps(info))
    # degenerate inputs: the compiled reference's prices only (no CLI run)
    book = degenerate_book()
    np.savez_compressed(os.path.join(HERE, "degenerate.npz"),
                        sptprice=book.sptprice, strike=book.strike, rate=book.rate,
                        volatility=book.volatility, otime=book.otime, otype=book.otype,
                        ref_prices=oracle.price_reference(book))
    x = np.linspace(-8.0, 8.0, 4097, dtype=np.float32)
    x = np.concatenate([x, np.array([0.0, -0.0, 1e-8, -1e-8, 30.0, -30.0], dtype=np.float32)])
    R = oracle.ref_lib()
    y = np.empty_like(x)
    R.bsref_cndf(len(x), x.ctypes.data_as(oracle.oracle._P), y.ctypes.data_as(oracle.oracle._P))
    np.savez_compressed(os.path.join(HERE, "cndf.npz"), x=x, ref=y)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
