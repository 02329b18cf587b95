"""Market and product inputs for the HJM exposure path.

The reference hard-codes a Bank of England forward curve, a three-factor PCA
volatility table and a pre-computed drift table (simulation_gpu_testing.cpp:
36-123) and a swap whose schedules are never read (product.h:4-18).  This
module builds the same kinds of arrays, in the same layouts, from closed
forms:

* tenor grid ``tau_i = dtau * i`` (51 points for 0..25y, 61 for 0..30y);
* Nelson-Siegel forward curve ``f(T) = 0.03 - 0.01 e^{-T/2} + 0.01 (T/2) e^{-T/2}``;
* three polynomial volatility factors, ``sigma_k(T) = sum_d c[k, d] T^d``
  (defaults: 0.0064; -0.0036 + 0.0004 T; 0.0020 - 0.0006 T + 0.00002 T^2),
  stored factor-major ``vol[k * n_tenor + t]`` like simulation_gpu_testing.cpp:47-63;
* the Musiela no-arbitrage drift by the trapezoid rule (the reference passes a
  drift table that this rule reproduces to the table's 7 printed decimals);
* a payer interest-rate swap with accrual ``alpha_i = dtau`` on periods
  ``1..n_periods`` and zero elsewhere.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

N_FACTOR = 3
POLY_DEGREE = 2  # each factor is a polynomial of degree <= 2 in T: 9 coefficients
DEFAULT_VOL_COEFFS = np.array(
    [
        [0.0064, 0.0, 0.0],
        [-0.0036, 0.0004, 0.0],
        [0.0020, -0.0006, 0.00002],
    ],
    dtype=np.float64,
)


def tenor_grid(n_tenor: int = 51, dtau: float = 0.5) -> np.ndarray:
    return dtau * np.arange(n_tenor, dtype=np.float64)


def nelson_siegel_curve(tau: np.ndarray) -> np.ndarray:
    e = np.exp(-tau / 2.0)
    return 0.03 - 0.01 * e + 0.01 * (tau / 2.0) * e


def poly_vols(tau: np.ndarray, coeffs: np.ndarray = DEFAULT_VOL_COEFFS) -> np.ndarray:
    """Factor-major volatility table ``[N_FACTOR][n_tenor]`` from polynomial coefficients."""
    coeffs = np.asarray(coeffs, dtype=np.float64).reshape(N_FACTOR, POLY_DEGREE + 1)
    powers = np.stack([tau**d for d in range(POLY_DEGREE + 1)])  # [3][n_tenor]
    return coeffs @ powers


def trapezoid_drift(vol: np.ndarray, dtau: float) -> np.ndarray:
    """mu_i = sum_k sigma_k(tau_i) * sum_{j<=i} (sigma_k(tau_j) + sigma_k(tau_{j-1})) / 2 * dtau."""
    vol = np.asarray(vol, dtype=np.float64)
    seg = 0.5 * (vol[:, 1:] + vol[:, :-1]) * dtau
    integral = np.concatenate([np.zeros((vol.shape[0], 1)), np.cumsum(seg, axis=1)], axis=1)
    return np.sum(vol * integral, axis=0)


def swap_accrual(n_tenor: int, n_periods: int, dtau: float = 0.5) -> np.ndarray:
    a = np.zeros(n_tenor, dtype=np.float64)
    a[1 : n_periods + 1] = dtau
    return a


@dataclass
class Market:
    """Inputs of one run, in the reference's array layouts."""

    n_tenor: int = 51
    dtau: float = 0.5
    vol_coeffs: np.ndarray = field(default_factory=lambda: DEFAULT_VOL_COEFFS.copy())
    spot: np.ndarray | None = None
    vol: np.ndarray | None = None
    drift: np.ndarray | None = None

    def __post_init__(self) -> None:
        tau = tenor_grid(self.n_tenor, self.dtau)
        if self.spot is None:
            self.spot = nelson_siegel_curve(tau)
        if self.vol is None:
            self.vol = poly_vols(tau, self.vol_coeffs)
        if self.drift is None:
            self.drift = trapezoid_drift(self.vol, self.dtau)
        self.spot = np.ascontiguousarray(self.spot, dtype=np.float64)
        self.vol = np.ascontiguousarray(self.vol, dtype=np.float64).reshape(N_FACTOR, self.n_tenor)
        self.drift = np.ascontiguousarray(self.drift, dtype=np.float64)

    @property
    def tau(self) -> np.ndarray:
        return tenor_grid(self.n_tenor, self.dtau)


@dataclass
class Swap:
    """One interest-rate swap leg pair on the tenor grid (payer: receives float, pays fixed)."""

    notional: float = 1.0e6
    strike: float = 0.025
    n_periods: int = 20
    payer: bool = True
    n_tenor: int = 51
    dtau: float = 0.5
    accrual: np.ndarray | None = None

    def __post_init__(self) -> None:
        if self.accrual is None:
            self.accrual = swap_accrual(self.n_tenor, self.n_periods, self.dtau)
        self.accrual = np.ascontiguousarray(self.accrual, dtype=np.float64)

    @property
    def sign(self) -> float:
        return 1.0 if self.payer else -1.0


@dataclass
class RunConfig:
    n_paths: int = 5000
    n_steps: int = 1000
    dt: float = 0.01
    seed: int = 1234
    hazard: float = 0.02
    recovery: float = 0.4
    pfe_quantile: float = 0.975
    path_offset: int = 0


@dataclass
class NettingSet:
    """Swaps on the tenor grid, netted before max(., 0): swap s pays (payer) or
    receives fixed_rate[s] on notional[s], accruing dtau on periods 1..n_periods[s]."""

    notional: np.ndarray
    fixed_rate: np.ndarray
    n_periods: np.ndarray
    payer: np.ndarray

    def __len__(self) -> int:
        return len(self.notional)

    def payoff_vectors(self, n_tenor: int, dtau: float = 0.5) -> tuple[np.ndarray, np.ndarray]:
        """Per-date (payA, payB): the netted cash flow of date i is D_i (payA_i L_i - payB_i)."""
        a, b = np.zeros(n_tenor), np.zeros(n_tenor)
        for n, k, m, p in zip(self.notional, self.fixed_rate, self.n_periods, self.payer):
            sgn = 1.0 if p else -1.0
            a[1 : m + 1] += sgn * n * dtau
            b[1 : m + 1] += sgn * n * dtau * k
        return a, b


def random_netting_set(n_swaps: int = 64, seed: int = 20261203, max_years: float = 30.0,
                       dtau: float = 0.5) -> NettingSet:
    """Maturities uniform on [1, max_years] snapped to the dtau grid, notionals
    log-uniform on [1e5, 1e7], fixed rates uniform on [1 %, 4 %], payer/receiver
    50/50, from a fixed seed."""
    rng = np.random.default_rng(seed)
    mat = rng.uniform(1.0, max_years, n_swaps)
    n_periods = np.clip(np.rint(mat / dtau).astype(np.int32), 1, int(round(max_years / dtau)))
    notional = np.exp(rng.uniform(np.log(1e5), np.log(1e7), n_swaps))
    fixed = rng.uniform(0.01, 0.04, n_swaps)
    payer = (rng.uniform(size=n_swaps) < 0.5).astype(np.int32)
    return NettingSet(notional, fixed, n_periods, payer)


def quantile_rank(q: float, n: int) -> int:
    """1-based rank of the q-quantile under the inverted-CDF definition."""
    k = int(np.ceil(q * n - 1e-7))
    return min(max(k, 1), n)
