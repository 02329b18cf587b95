"""Host-side inputs: the synthetic market, the trapezoid drift, quantile ranks."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from conftest import load_golden
from cva_hjm_cuda_gb300.market import Market, Swap, nelson_siegel_curve, poly_vols, quantile_rank, trapezoid_drift


def test_market_shapes_and_forms():
    mk = Market(n_tenor=51)
    assert mk.spot.shape == (51,) and mk.vol.shape == (3, 51) and mk.drift.shape == (51,)
    tau = mk.tau
    assert tau[-1] == 25.0
    np.testing.assert_allclose(mk.spot, 0.03 - 0.01 * np.exp(-tau / 2) + 0.01 * (tau / 2) * np.exp(-tau / 2))
    np.testing.assert_allclose(mk.vol[0], 0.0064)
    np.testing.assert_allclose(mk.vol[1], -0.0036 + 0.0004 * tau, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(mk.vol[2], 0.0020 - 0.0006 * tau + 0.00002 * tau**2, rtol=1e-12, atol=1e-15)
    mk61 = Market(n_tenor=61)
    assert mk61.tau[-1] == 30.0


def test_drift_matches_oracle_trapezoid():
    mk = Market()
    np.testing.assert_allclose(trapezoid_drift(mk.vol, 0.5), O.trapezoid_drift(mk.vol, 0.5), rtol=1e-14, atol=1e-20)


def test_trapezoid_drift_reproduces_reference_drift_table():
    """The reference passes a pre-computed drift (simulation_gpu_testing.cpp:66-71) for its
    PCA volatility table (:47-63), both stored verbatim in the driver's golden fixture; the
    trapezoid rule reproduces it to the table's printed precision (7 decimals)."""
    g = load_golden("ref_driver_own_market.json")
    vol = np.array(g["vol"]).reshape(3, 51)
    drift = np.array(g["drift"])
    mine = trapezoid_drift(vol, 0.5)
    assert np.max(np.abs(mine - drift)) < 2e-7


def test_swap_accrual():
    sw = Swap(n_periods=20)
    assert sw.accrual[0] == 0.0 and np.all(sw.accrual[1:21] == 0.5) and np.all(sw.accrual[21:] == 0.0)
    assert Swap(payer=False).sign == -1.0


@pytest.mark.parametrize("q,n", [(0.975, 5000), (0.975, 1048576), (0.975, 4194304), (0.5, 7), (0.999, 10), (0.01, 3)])
def test_quantile_rank_matches_oracle(q, n):
    assert quantile_rank(q, n) == O.oracle().oracle_quantile_rank(q, n)
    k = quantile_rank(q, n)
    assert 1 <= k <= n and k >= q * n - 1e-6 and k - 1 < q * n + 1e-6


def test_pfe_and_cva_oracle_properties():
    rng = np.random.default_rng(0)
    x = np.maximum(rng.normal(size=(1000, 51)), 0.0)
    x[:, 21:] = 0
    pfe = O.pfe(x, 21, 0.975)
    k = quantile_rank(0.975, 1000)
    np.testing.assert_array_equal(pfe, np.sort(x[:, :21], axis=0)[k - 1])
    ee = O.expected_exposure(x)
    cva, dcva = O.cva(ee, 21, 0.5, 0.02, 0.4)
    c = O.cva_paths(x, 21, 0.5, 0.02, 0.4)
    assert abs(c.mean() - cva) < 1e-12 * abs(cva)
    h = 1e-6
    fd = (O.cva(ee, 21, 0.5, 0.02 + h, 0.4)[0] - O.cva(ee, 21, 0.5, 0.02 - h, 0.4)[0]) / (2 * h)
    assert abs(fd - dcva) < 1e-6 * abs(dcva)
