"""Swaption books for the HJM Monte-Carlo pricer (the swaptions application).

The reference's driver builds its swaptions in code
(parsec-ff/pkgs/apps/swaptions/src/HJM_Securities.cpp:231-296): an 11-point
HJM grid, three volatility factors from a fixed table, a yield curve rising
from 10 % in steps of 0.5 %, maturity 1 year, tenor 2 years, annual
payments, continuously compounded strikes, and per swaption a horizon of
5 to 19.75 years in quarter-year steps and a strike of 0.1 to 4.9 in steps
of 0.1 -- both drawn with the reference's RanUnif, which is not in the
reference tree, so a seeded numpy stream draws them here.  Swaption i's
paths use seed base + i, as the reference passes swaption_seed + i
(HJM_Securities.cpp:198, 319).
"""
from __future__ import annotations

import dataclasses

import numpy as np

N_STEPS = 11  # iN, HJM_Securities.cpp:56
N_FACTORS = 3  # iFactors, HJM_Securities.cpp:58

# The factor volatilities, HJM_Securities.cpp:231-264: factor k's vol for the
# forward rate m + 1 steps from maturity.
FACTORS = np.array([
    [.01] * 10,
    [.009048, .008187, .007408, .006703, .006065, .005488, .004966, .004493, .004066, .003679],
    [.001000, .000750, .000500, .000250, .000000, -.000250, -.000500, -.000750, -.001000, -.001250],
], dtype=np.float64)


def reference_yields(n: int = N_STEPS) -> np.ndarray:
    """The yield curve as the reference builds it: 0.1, then each point the
    previous one plus 0.005 (HJM_Securities.cpp:288-290)."""
    y = np.empty(n, dtype=np.float64)
    y[0] = .1
    for j in range(1, n):
        y[j] = y[j - 1] + .005
    return y


@dataclasses.dataclass
class Swaption:
    """One swaption: the reference's parm fields (HJM_Securities.cpp:276-296)."""

    strike: float
    years: float
    compounding: float = 0.0
    maturity: float = 1.0
    tenor: float = 2.0
    payment_interval: float = 1.0
    yield_curve: np.ndarray = dataclasses.field(default_factory=lambda: reference_yields())
    factors: np.ndarray = dataclasses.field(default_factory=lambda: FACTORS.copy())
    seed: int = 0

    @property
    def n_steps(self) -> int:
        return int(self.yield_curve.shape[0])

    @property
    def n_factors(self) -> int:
        return int(self.factors.shape[0])


class SplitMix64:
    """The CLI's parameter stream (host/swaptions_gpu.cpp): splitmix64,
    u = top 53 bits / 2^53."""

    def __init__(self, seed: int):
        self.s = seed & (2**64 - 1)

    def unit(self) -> float:
        m = 2**64 - 1
        self.s = (self.s + 0x9E3779B97F4A7C15) & m
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
        z ^= z >> 31
        return (z >> 11) * (1.0 / 9007199254740992.0)


def generate_cli(n: int, seed: int = 1979) -> list[Swaption]:
    """The swaption set the drop-in CLI builds for `-ns n -sd seed`."""
    rng = SplitMix64(seed)
    base = int(2147483647 * rng.unit())
    out = []
    for i in range(n):
        years = 5.0 + int(60 * rng.unit()) * 0.25
        strike = 0.1 + int(49 * rng.unit()) * 0.1
        out.append(Swaption(strike=strike, years=years, seed=base + i))
    return out


def generate(n: int, seed: int = 1979) -> list[Swaption]:
    """n swaptions of the reference's workload (seeded)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    base = int(rng.integers(1, 2**31 - 1))
    out = []
    for i in range(n):
        years = 5.0 + int(60 * rng.random()) * 0.25     # HJM_Securities.cpp:279
        strike = 0.1 + int(49 * rng.random()) * 0.1     # HJM_Securities.cpp:281
        out.append(Swaption(strike=strike, years=years, seed=base + i))
    return out
