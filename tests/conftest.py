import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built libbsgpu.so")


def load_golden(name):
    """(Book, reference prices float32, FP64 oracle prices) of a fixture."""
    from p3arsec_gb300 import books
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    book = books.Book(z["sptprice"], z["strike"], z["rate"], z["volatility"], z["otime"],
                      z["otype"])
    return book, z["ref_prices"], z["fp64_prices"]


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build(ref=False)
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx():
    """A context on cuda:0; fails (not skips) when the library or GPU is missing."""
    from p3arsec_gb300 import build as b
    b.build()
    from p3arsec_gb300 import Context
    ctx = Context(0, 1 << 22)
    yield ctx
    ctx.close()
