"""Device-side failure detection without a GPU fault: the staged kernel's
mbarrier waits are bounded by GPU time; the self-test makes every wait run
out (barriers expecting more bytes than their copies deliver — nothing ever
completes them), and the host reads BSG_ERR_TIMEOUT.  The context stays
usable.  Host-side failures of the serving loop are in test_gpu_serve.py."""
import numpy as np
import pytest

import oracle
from p3arsec_gb300 import books

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_context_survives(gpu_ctx):
    st, secs = gpu_ctx.selftest_wait_timeout(0.05)
    assert st == -7  # BSG_ERR_TIMEOUT
    assert 0.05 <= secs < 5.0
    # the same context prices correctly afterwards, on every path
    book = books.generate(20011, seed=81)
    fp64 = oracle.price_fp64(book)
    saved = gpu_ctx.get_tune()
    try:
        for tune in ((1, 256, 2, 2, 1), (1, 256, 0, 4, 1)):
            gpu_ctx.set_tune(*tune)
            got = gpu_ctx.price_book(book, num_runs=3)
            assert np.abs(got.astype(np.float64) - fp64).max() <= 1e-4
    finally:
        gpu_ctx.set_tune(**saved)
    st2, _ = gpu_ctx.selftest_wait_timeout(0.02)
    assert st2 == -7
