"""Seeded synthetic option books and the PARSEC blackscholes text format.

The PARSEC input sets (``in_*.txt``) are not distributed with the reference, so
every workload here is a seeded synthetic book with the field distributions
of the benchmark configurations:

* ``plain``  -- S~U[10,200], K=S*U[0.5,1.5], r~U[0.01,0.10], v~U[0.05,0.65],
  t~U[0.05,2.0], otype~Bernoulli(0.5) (65,536 and 10,000,000-option maps,
  the batched books and the serving requests);
* ``tails``  -- as ``plain`` but K=S*U[0.05,20] and t~U[0.001,5]: deep
  in/out-of-the-money options whose |d1| reaches the CNDF tails (the 2^28
  precision sweep).

Every field is drawn in float64 and rounded once to float32, the storage
type of the reference (``fptype float``, blackscholes.c:85).

Text format (blackscholes.c:695-739): a first line with the option count,
then one line per option ``s strike r divq v t OptionType divs DGrefval``
(``%f %f %f %f %f %f %c %f %f``).  ``otype`` is 1 for 'P' and 0 otherwise
(blackscholes.c:760).  Output files are the count then ``%.18f`` per price
(blackscholes.c:929-942).
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

FIELDS = ("sptprice", "strike", "rate", "volatility", "otime")


@dataclasses.dataclass
class Book:
    """One option book in the reference's SoA layout (blackscholes.c:747-767)."""

    sptprice: np.ndarray
    strike: np.ndarray
    rate: np.ndarray
    volatility: np.ndarray
    otime: np.ndarray
    otype: np.ndarray  # int32, 1 = put, 0 = call

    def __len__(self) -> int:
        return int(self.sptprice.shape[0])

    def arrays(self):
        return (self.sptprice, self.strike, self.rate, self.volatility,
                self.otime, self.otype)

    def slice(self, a: int, b: int) -> "Book":
        return Book(*(x[a:b] for x in self.arrays()))


def generate(n: int, seed: int, dist: str = "plain") -> Book:
    """Seeded book of ``n`` options (PCG64 stream ``seed``)."""
    if n < 0:
        raise ValueError("n must be >= 0")
    if dist not in ("plain", "tails"):
        raise ValueError(f"unknown distribution {dist!r}")
    rng = np.random.Generator(np.random.PCG64(seed))
    f32 = np.float32
    s = rng.uniform(10.0, 200.0, n)
    if dist == "plain":
        k = s * rng.uniform(0.5, 1.5, n)
        t = rng.uniform(0.05, 2.0, n)
    else:
        k = s * rng.uniform(0.05, 20.0, n)
        t = rng.uniform(0.001, 5.0, n)
    r = rng.uniform(0.01, 0.10, n)
    v = rng.uniform(0.05, 0.65, n)
    otype = (rng.random(n) < 0.5).astype(np.int32)
    return Book(s.astype(f32), k.astype(f32), r.astype(f32), v.astype(f32),
                t.astype(f32), otype)


def generate_device(n: int, seed: int, dist: str = "plain", device: str = "cuda:0",
                    chunk: int = 1 << 26):
    """Seeded book of ``n`` options drawn on the GPU (torch's Philox stream
    ``seed``), for books too large to draw on the host in reasonable time
    (2^28 options: seconds here against minutes with numpy).  Same field
    distributions and float64-then-float32 rounding as :func:`generate`, a
    different random stream.  Returns six device tensors in ``Book.arrays()``
    order."""
    import torch
    if dist not in ("plain", "tails"):
        raise ValueError(f"unknown distribution {dist!r}")
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    out = [torch.empty(n, dtype=torch.float32, device=device) for _ in range(5)]
    ot = torch.empty(n, dtype=torch.int32, device=device)

    def u(m, lo, hi):
        return torch.rand(m, dtype=torch.float64, device=device, generator=g) * (hi - lo) + lo

    for a in range(0, n, chunk):
        m = min(chunk, n - a)
        s = u(m, 10.0, 200.0)
        if dist == "plain":
            k = s * u(m, 0.5, 1.5)
            t = u(m, 0.05, 2.0)
        else:
            k = s * u(m, 0.05, 20.0)
            t = u(m, 0.001, 5.0)
        out[0][a:a + m] = s.float()
        out[1][a:a + m] = k.float()
        out[4][a:a + m] = t.float()
        del s, k, t
        out[2][a:a + m] = u(m, 0.01, 0.10).float()
        out[3][a:a + m] = u(m, 0.05, 0.65).float()
        ot[a:a + m] = (torch.rand(m, device=device, generator=g) < 0.5).int()
    return out + [ot]


def concat(books) -> Book:
    books = list(books)
    return Book(*(np.concatenate([b.arrays()[i] for b in books]) for i in range(6)))


# ---------------------------------------------------------------- text format

def write_parsec_input(path: str | os.PathLike, book: Book,
                       dgrefval: np.ndarray | None = None) -> None:
    """Write ``book`` in the PARSEC blackscholes input format.

    Floats are printed with 9 significant digits, which round-trips every
    float32 exactly through the reference's ``fscanf("%f")``.  ``divq`` and
    ``divs`` are 0 (the pricing formula does not use them).  ``dgrefval`` is
    the reference price column that the reference's ERR_CHK build compares
    against (blackscholes.c:333-339); 0 when absent.
    """
    n = len(book)
    ref = np.zeros(n) if dgrefval is None else np.asarray(dgrefval, dtype=np.float64)
    typ = np.where(book.otype == 1, "P", "C")
    with open(path, "w") as f:
        f.write(f"{n}\n")
        cols = [book.sptprice, book.strike, book.rate, book.volatility, book.otime]
        for i in range(n):
            s, k, r, v, t = (float(c[i]) for c in cols)
            f.write(f"{s:.9g} {k:.9g} {r:.9g} 0 {v:.9g} {t:.9g} {typ[i]} 0 {ref[i]:.17g}\n")


def read_parsec_input(path: str | os.PathLike):
    """Parse a PARSEC input file; returns ``(Book, dgrefval float32)``.

    Mirrors blackscholes.c:695-739: the count, then 9 whitespace-separated
    fields per option.  Raises ``ValueError`` where the reference prints an
    error and exits.
    """
    with open(path) as f:
        head = f.readline().split()
        if not head:
            raise ValueError(f"unable to read from file {path!s}")
        n = int(head[0])
        rows = f.read().split()
    if len(rows) < 9 * n:
        raise ValueError(f"unable to read from file {path!s}")
    rows = np.array(rows[: 9 * n], dtype=object).reshape(n, 9) if n else np.zeros((0, 9), dtype=object)
    col = lambda j: rows[:, j].astype(np.float64).astype(np.float32)  # noqa: E731
    otype = (rows[:, 6] == "P").astype(np.int32)
    book = Book(col(0), col(1), col(2), col(4), col(5), otype)
    return book, col(8)


def write_parsec_output(path: str | os.PathLike, prices: np.ndarray) -> None:
    """``%i`` count then ``%.18f`` per price (blackscholes.c:929-942)."""
    p = np.asarray(prices, dtype=np.float32)
    with open(path, "w") as f:
        f.write(f"{p.shape[0]}\n")
        for x in p:
            f.write("%.18f\n" % float(x))


def read_parsec_output(path: str | os.PathLike) -> np.ndarray:
    with open(path) as f:
        n = int(f.readline())
        vals = np.array(f.read().split()[:n], dtype=np.float64)
    return vals.astype(np.float32)
