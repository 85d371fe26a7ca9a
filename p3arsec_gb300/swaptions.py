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


@dataclasses.dataclass
class Swaption:
    """One swaption: the reference's parm fields (HJM_Securities.cpp:276-296)."""

    strike: float
    years: float
    compounding: float = 0.0
    maturity: float = 1.0
    tenor: float = 2.0
    payment_interval: float = 1.0
    yield_curve: np.ndarray = dataclasses.field(
        default_factory=lambda: 0.1 + 0.005 * np.arange(N_STEPS, dtype=np.float64))
    factors: np.ndarray = dataclasses.field(default_factory=lambda: FACTORS.copy())
    seed: int = 0

    @property
    def n_steps(self) -> int:
        return int(self.yield_curve.shape[0])

    @property
    def n_factors(self) -> int:
        return int(self.factors.shape[0])


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
