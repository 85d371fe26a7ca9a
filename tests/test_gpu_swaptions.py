"""The swaption Monte Carlo on the GPU, called through the C ABI, against the
CPU oracle (oracle/swpt_oracle.c).

Both draw every path's normal variates from the same counter-based stream,
so they simulate the same paths; the GPU stops each path at the swaption's
maturity (later rows never reach the payoff) while the oracle simulates the
whole path matrix as the reference does.  They differ only in rounding (CUDA's
double log/sincos/exp vs glibc's, fused multiply-adds, summation order):
  * price: relative 1e-10 (absolute 1e-12 for prices near zero);
  * standard error: relative 1e-6 (the reference's formula subtracts two
    nearly equal sums).
Parity with the reference itself is unpinned (its model core is not in the
reference tree); the oracle's own checks are in test_swaptions_oracle.py.
"""
import numpy as np
import pytest

from p3arsec_gb300 import abi
from p3arsec_gb300 import swaptions as S

pytestmark = pytest.mark.gpu


def check(got, err, want, want_err):
    assert np.allclose(got, want, rtol=1e-10, atol=1e-12), np.max(np.abs(got - want))
    assert np.allclose(err, want_err, rtol=1e-6, atol=1e-14)


@pytest.mark.parametrize("trials", [20_000, 100_003])
def test_reference_workload_against_oracle(gpu_ctx, oracle_lib, trials):
    sw = S.generate(16, seed=1979)
    got, err = gpu_ctx.price_swaptions(sw, trials)
    want, want_err, _ = oracle_lib.swaptions_all(sw, trials, 8)
    check(got, err, want, want_err)


def test_longer_grids_and_other_factor_counts(gpu_ctx, oracle_lib):
    """Grids longer than 12 points (the kernel's second shape), one and five
    factors, compounded strikes, semi-annual payments."""
    rng = np.random.default_rng(4)
    sw = []
    for i, (n, nf) in enumerate([(20, 1), (32, 5), (12, 3), (7, 2), (25, 8)]):
        sw.append(S.Swaption(strike=0.05 + 0.02 * i, years=0.5 * n, compounding=0.5 if i % 2 else 0.0,
                             maturity=1.0, tenor=2.0, payment_interval=0.5 if n >= 20 else 1.0,
                             yield_curve=0.03 + 0.002 * np.arange(n),
                             factors=rng.uniform(-0.004, 0.012, (nf, n - 1)), seed=77 + i))
    got, err = gpu_ctx.price_swaptions(sw, 30_000)
    for i, w in enumerate(sw):
        p, e = oracle_lib.swaption_price(w, 30_000)
        check(got[i:i + 1], err[i:i + 1], np.array([p]), np.array([e]))


def _shaped(n, years, maturity, tenor, pay, i, nf=3):
    rng = np.random.default_rng(100 + i)
    return S.Swaption(strike=0.04 + 0.01 * i, years=years, maturity=maturity, tenor=tenor,
                      payment_interval=pay, yield_curve=0.03 + 0.001 * np.arange(n),
                      factors=rng.uniform(-0.003, 0.01, (nf, n - 1)), seed=900 + i)


@pytest.mark.parametrize("shapes", [
    # 11- and 12-point grids (the 12-point kernel): rows of every length the
    # payoff can read there, swap_points + start - 1 = 1..10
    [(11, 11, 1, 1, 1), (11, 11, 1, 2, 1), (11, 11, 2, 2, 1), (11, 11, 2, 3, 1), (11, 11, 3, 3, 1),
     (11, 11, 3, 4, 1), (11, 11, 4, 4, 1), (11, 11, 4, 5, 1), (12, 6, 2, 3, 0.5), (12, 12, 1, 10, 1),
     (11, 5.5, 4.5, 0.5, 0.5)],
    # with 32-point grids (the 32-point kernel): short rows, and rows longer
    # than 10 that take the untrimmed body
    [(32, 16, 0.5, 1, 0.5), (20, 10, 2, 3, 0.5), (32, 8, 2, 3, 0.25), (32, 32, 5, 20, 1)],
], ids=["12-point", "32-point"])
def test_every_row_length_against_oracle(gpu_ctx, oracle_lib, shapes):
    """The kernel cuts each path row to the entries the payoff reads, with
    one instantiation per row length: every length prices as the oracle's
    full-matrix simulation of the same paths."""
    sw = [_shaped(*sh, i) for i, sh in enumerate(shapes)]
    got, err = gpu_ctx.price_swaptions(sw, 20_000)
    for i, w in enumerate(sw):
        p, e = oracle_lib.swaption_price(w, 20_000)
        check(got[i:i + 1], err[i:i + 1], np.array([p]), np.array([e]))


def test_zero_volatility_is_deterministic(gpu_ctx, oracle_lib):
    sw = [S.Swaption(strike=k, years=y, factors=np.zeros((3, 10)), seed=5)
          for k, y in ((0.1, 5.0), (1.7, 12.25), (4.9, 19.75))]
    got, _ = gpu_ctx.price_swaptions(sw, 4096)
    for i, w in enumerate(sw):
        p, _ = oracle_lib.swaption_price(w, 64)
        assert got[i] == pytest.approx(p, rel=1e-13, abs=1e-15)


def test_two_runs_give_the_same_bits(gpu_ctx):
    sw = S.generate(8, seed=2)
    a, ea = gpu_ctx.price_swaptions(sw, 50_000)
    b, eb = gpu_ctx.price_swaptions(sw, 50_000)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    assert np.array_equal(ea.view(np.uint64), eb.view(np.uint64))


def test_reference_signature_equals_the_batched_call(gpu_ctx):
    sw = S.generate(3, seed=5)
    got, err = gpu_ctx.price_swaptions(sw, 10_000)
    for i, w in enumerate(sw):
        st, p, e = abi.HJM_Swaption_Blocking(w, 10_000)
        assert st == 1
        assert p == got[i] and e == err[i]


def test_invalid_swaptions_are_refused(gpu_ctx):
    from p3arsec_gb300.abi import BsgError
    good = S.generate(2, seed=3)
    bad_tenor = S.Swaption(strike=0.1, years=5.0, tenor=10.0)  # past the grid
    with pytest.raises(BsgError, match="swaption 2"):
        gpu_ctx.price_swaptions(good + [bad_tenor], 1000)
    with pytest.raises(BsgError):
        gpu_ctx.price_swaptions(good, 1)  # the standard error needs two trials
    short = S.Swaption(strike=0.1, years=5.0, yield_curve=np.array([0.1]), factors=np.zeros((3, 0)))
    with pytest.raises(BsgError):
        gpu_ctx.price_swaptions([short], 1000)
    # the context still prices afterwards
    p, _ = gpu_ctx.price_swaptions(good, 1000)
    assert np.all(np.isfinite(p))


def test_the_most_swaptions_one_call_takes(gpu_ctx, oracle_lib):
    """65,535 swaptions (the grid's y extent) in one call at the fewest
    trials (2), a few of them checked against the oracle; one more is
    refused with BSG_ERR_CAPACITY before anything runs."""
    from p3arsec_gb300.abi import BsgError
    sw = S.generate(65535, seed=8)
    got, err = gpu_ctx.price_swaptions(sw, 2)
    assert got.shape == (65535,) and np.all(np.isfinite(got)) and np.all(np.isfinite(err))
    for i in (0, 1, 32767, 65534):
        p, e = oracle_lib.swaption_price(sw[i], 2)
        check(got[i:i + 1], err[i:i + 1], np.array([p]), np.array([e]))
    with pytest.raises(BsgError) as e:
        gpu_ctx.price_swaptions(sw + sw[:1], 2)
    assert e.value.status == -5  # BSG_ERR_CAPACITY
