"""The swaption oracle (oracle/swpt_oracle.c) on the CPU.

The reference tree holds the swaptions driver but not its HJM model core,
so these checks pin the restatement against what the mathematics requires
instead of against reference outputs (parity with the reference: unpinned):
  * with every factor volatility zero the model is deterministic and the
    price is the driver's payoff on the initial curve, computed here
    independently (HJM_Swaption_Blocking.cpp:116-140, 191-198);
  * the drift makes discounted bond prices martingales, so the unfloored
    payoff's expectation is the initial curve's value of the fixed leg minus
    the zero-coupon bond to maturity: the Monte Carlo mean must land within
    a few standard errors of it;
  * the normal variates have mean 0, variance 1 and uncorrelated pairs;
  * the forward curve averages back to the yield curve;
  * the threaded driver gives each swaption the bits of pricing it alone.
"""
import math

import numpy as np
import pytest

from p3arsec_gb300 import swaptions as S


def driver_constants(sw):
    """The driver's per-swaption indices and payments, restated in numpy."""
    n = sw.n_steps
    h = sw.years / n
    freq = int(sw.payment_interval / h + 0.5)
    k = sw.strike if sw.compounding == 0 else math.log(1 + sw.strike * sw.compounding) / sw.compounding
    swap_len = int(n - sw.maturity / h + 0.5)
    start = int(sw.maturity / h + 0.5)
    points = int(sw.tenor / h + 0.5)
    pay = np.zeros(swap_len)
    for i in range(freq, points + 1, freq):
        pay[i] = math.exp(k * sw.payment_interval) - (0 if i == points else 1)
    return h, start, pay


def initial_bonds(sw, oracle_lib):
    h, start, pay = driver_constants(sw)
    f = oracle_lib.yield_to_forward(sw.yield_curve)
    p0 = np.exp(-h * np.concatenate([[0.0], np.cumsum(f)]))  # P(0, t_j), j = 0..n
    return h, start, pay, p0


@pytest.mark.parametrize("years,strike", [(5.0, 0.1), (5.0, 4.9), (12.25, 1.7), (19.75, 0.3)])
def test_zero_volatility_is_the_deterministic_payoff(oracle_lib, years, strike):
    sw = S.Swaption(strike=strike, years=years, factors=np.zeros((3, 10)), seed=5)
    h, start, pay, p0 = initial_bonds(sw, oracle_lib)
    fixed = sum(pay[l] * p0[start + l] / p0[start] for l in range(len(pay)))
    want = max(fixed - 1.0, 0.0) * p0[start]
    price, err = oracle_lib.swaption_price(sw, 64)
    assert price == pytest.approx(want, rel=1e-13, abs=1e-15)
    # zero up to the rounding of the reference's formula, sqrt((sum_sq -
    # sum^2 / M) / (M - 1)) / sqrt(M), which cancels (or NaN when the
    # rounding leaves the difference below zero)
    assert not (err > 1e-7 * max(1.0, want))


@pytest.mark.parametrize("years", [5.0, 9.5, 19.75])
def test_discounted_bonds_are_martingales(oracle_lib, years):
    # a strike near the money, so that the unfloored payoff's spread is modest
    sw = S.Swaption(strike=0.12, years=years, seed=11)
    h, start, pay, p0 = initial_bonds(sw, oracle_lib)
    want = sum(pay[l] * p0[start + l] for l in range(len(pay))) - p0[start]
    mean, err = oracle_lib.swaption_price(sw, 200_000, unfloored=True)
    assert abs(mean - want) <= 4.0 * err, (mean, want, err)
    # and with the floor the price is at least the unfloored one
    floored, _ = oracle_lib.swaption_price(sw, 200_000)
    assert floored >= mean


def test_martingale_check_sees_the_drift(oracle_lib):
    """At four times the reference's volatilities the drift moves the
    expected payoff by many standard errors, so the martingale check would
    fail without it; with it the Monte Carlo mean still lands on the
    initial curve's value."""
    sw = S.Swaption(strike=0.12, years=19.75, factors=S.FACTORS * 4.0, seed=13)
    h, start, pay, p0 = initial_bonds(sw, oracle_lib)
    mu = oracle_lib.hjm_drift(sw.factors, h)
    want = sum(pay[l] * p0[start + l] for l in range(len(pay))) - p0[start]
    mean, err = oracle_lib.swaption_price(sw, 200_000, unfloored=True)
    assert abs(mean - want) <= 4.0 * err
    # without the drift, the forwards at maturity would sit lower by about
    # start steps of it, and the swap's bonds higher by that much
    shift = start * h * np.concatenate([[0.0], np.cumsum(mu)])[: len(pay)]
    effect = sum(pay[l] * p0[start + l] * (math.exp(h * shift[l]) - 1.0) for l in range(len(pay)))
    assert abs(effect) > 8.0 * err, (effect, err)


def test_normals(oracle_lib):
    z = np.array([oracle_lib.normal_pair(7, t, j) for t in range(20_000) for j in range(3)])
    assert abs(z.mean()) < 0.02
    assert abs(z.var() - 1.0) < 0.03
    assert abs(np.corrcoef(z[:, 0], z[:, 1])[0, 1]) < 0.02
    # depends on the seed, the trial and the index
    assert oracle_lib.normal_pair(7, 0, 0) != oracle_lib.normal_pair(8, 0, 0)
    assert oracle_lib.normal_pair(7, 1, 0) != oracle_lib.normal_pair(7, 0, 0)
    assert oracle_lib.normal_pair(7, 0, 1) != oracle_lib.normal_pair(7, 0, 0)


def test_forward_curve_averages_to_the_yields(oracle_lib):
    y = 0.1 + 0.005 * np.arange(11)
    f = oracle_lib.yield_to_forward(y)
    assert np.allclose(np.cumsum(f) / np.arange(1, 12), y, rtol=0, atol=1e-15)


def test_drift_formula(oracle_lib):
    h = 0.5
    mu = oracle_lib.hjm_drift(S.FACTORS, h)
    s = np.cumsum(S.FACTORS, axis=1)
    s_prev = np.concatenate([np.zeros((3, 1)), s[:, :-1]], axis=1)
    assert np.allclose(mu, 0.5 * h * (s * s - s_prev * s_prev).sum(axis=0), rtol=1e-12, atol=0)


def test_threaded_driver_equals_one_at_a_time(oracle_lib):
    sw = S.generate(7, seed=3)
    price, err, secs = oracle_lib.swaptions_all(sw, 2000, 3)
    for i, s in enumerate(sw):
        p, e = oracle_lib.swaption_price(s, 2000)
        assert price[i] == p and err[i] == e
    assert secs >= 0


def test_out_of_range_parameters_are_refused(oracle_lib):
    # a tenor reaching past the path: the reference would write past its
    # payment vector (HJM_Swaption_Blocking.cpp:122, 134-140)
    with pytest.raises(ValueError):
        oracle_lib.swaption_price(S.Swaption(strike=0.1, years=5.0, tenor=10.0), 100)
