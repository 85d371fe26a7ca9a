"""p3arsec_gb300 -- GB300 (sm_103a) Black-Scholes map, a drop-in for the hot
path of P3ARSEC's blackscholes benchmark.

The product is libbsgpu.so (CUDA kernels + C ABI, include/bsg.h); this
package is its Python host side: the ctypes binding (``abi``), seeded option
books and the PARSEC text format (``books``), the reference-shaped driver
(``blackscholes``), and the in-tree build (``build``).
"""
from . import books  # noqa: F401
from .abi import (BlkSchlsEqEuroNoDiv, BsgError, Context, NUM_RUNS,  # noqa: F401
                  load)

__all__ = ["books", "BlkSchlsEqEuroNoDiv", "BsgError", "Context", "NUM_RUNS", "load"]
