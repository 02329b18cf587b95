"""The oracle against the reference: golden vectors made by the reference's
own CPU code (tests/golden/make_golden.py) and, where the reference tree is
present, the reference compiled from its sources (oracle/_ref)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from conftest import market_from_golden


def _curand_normals(g):
    return O.curand_normals_double(g["normals"]["count"], seed=g["normals"]["seed"]).reshape(g["n_paths"], g["n_steps"], 3)


def test_oracle_matches_reference_driver_25y(golden_25y):
    """The reference's whole calculateExposureCPU<double> (simulation_cpu.h:350)."""
    g = golden_25y
    mk, sw = market_from_golden(g)
    x = O.exposure_paths(mk, sw, g["n_steps"], g["dt"], _curand_normals(g))
    ee = O.expected_exposure(x)
    ref = np.array(g["ee"])
    np.testing.assert_allclose(ee, ref, rtol=1e-13, atol=0)


def test_oracle_matches_reference_driver_own_market(golden_own):
    """The reference driver's own run (simulation_gpu_testing.cpp -cpu -scenarios 5000): its BoE
    curve, cubic PCA volatility table, hard-coded drift table, irregular accruals, N = 10,
    K = 6.7%, 25y; EE from the unmodified calculateExposureCPU<double>."""
    g = golden_own
    mk, sw = market_from_golden(g)
    normals = _curand_normals(g)
    x = O.exposure_paths(mk, sw, g["n_steps"], g["dt"], normals)
    np.testing.assert_array_equal(x[:16], np.array(g["exposures_first_paths"]))
    ee, ref = O.expected_exposure(x), np.array(g["ee"])
    np.testing.assert_allclose(ee, ref, rtol=1e-13, atol=0)
    assert abs(ref[0] - 0.122920) < 5e-7  # the driver's printed first EE value
    assert ref[50] == 0.0 and np.all(ref[:50] > 0.0)  # the 25y swap's last date has no cash flow left


def test_oracle_matches_reference_blocks_10y(golden_10y):
    """The reference's per-path functions over a 10y swap (zeroed numeraires)."""
    g = golden_10y
    mk, sw = market_from_golden(g)
    x = O.exposure_paths(mk, sw, g["n_steps"], g["dt"], _curand_normals(g))
    np.testing.assert_allclose(x[:16], np.array(g["exposures_first_paths"]), rtol=1e-14, atol=0)
    np.testing.assert_allclose(O.expected_exposure(x), np.array(g["ee"]), rtol=1e-13, atol=0)
    # 20 sampled dates: exposure is zero from date 20 on (no cash flows after the swap)
    assert np.all(x[:, 20:] == 0.0)


@pytest.mark.skipif(not O.ref_available(), reason="reference tree not present")
@pytest.mark.parametrize("seed,n_paths", [(7, 32), (99, 9)])
def test_oracle_bitwise_vs_compiled_reference(seed, n_paths):
    """Restatement vs the reference compiled from its own sources, same normals."""
    from cva_hjm_cuda_gb300.market import Market, Swap

    mk = Market()
    mk.drift = O.trapezoid_drift(mk.vol, mk.dtau)
    sw = Swap()
    n_steps = 1000
    normals = O.host_normals(seed, 0, n_paths, n_steps)
    x_ref = np.zeros((n_paths, 51))
    ee_ref = np.zeros(51)
    rc = O.ref().ref_exposure_paths(n_steps, mk.spot, mk.vol.ravel(), mk.drift, sw.accrual, sw.notional, sw.strike,
                                    n_paths, normals.ravel(), x_ref.ravel(), ee_ref)
    assert rc == 0
    x = O.exposure_paths(mk, sw, n_steps, 0.01, normals)
    assert np.array_equal(x, x_ref)
    np.testing.assert_allclose(O.expected_exposure(x), ee_ref, rtol=1e-15, atol=0)


def test_oracle_rejects_bad_shapes():
    from cva_hjm_cuda_gb300.market import Market, Swap

    mk, sw = Market(), Swap()
    with pytest.raises(ValueError):
        O.exposure_paths(mk, sw, 1010, 0.01, np.zeros((2, 1010, 3)))  # not a multiple of 50 steps
    with pytest.raises(ValueError):
        O.exposure_paths(mk, sw, 2550, 0.01, np.zeros((1, 2550, 3)))  # 51 dates on a 51-tenor grid


def test_empty_path_set_has_zero_exposure():
    from cva_hjm_cuda_gb300.market import Market, Swap

    x = O.exposure_paths(Market(), Swap(), 1000, 0.01, np.zeros((0, 1000, 3)))
    assert x.shape == (0, 51)
