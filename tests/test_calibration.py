"""The market-input step (hjm_calibrate_pca), on CPU: it needs no GPU.

* against numpy: the annualised covariance of the curve changes, its three
  leading eigenpairs (numpy.linalg.eigh) and least-squares polynomial fits
  (numpy.polyfit) on the same synthetic history, to 1e-9 relative;
* against the model: on a long history simulated from the reference's own
  three factors (constant, linear, quadratic in T), the calibrated factors
  reproduce the model's covariance sum_k sigma_k sigma_k^T within the sampling
  error, and the round trip into the engine's polynomial market works;
* bad input is rejected.
"""
from __future__ import annotations

import numpy as np
import pytest

from cva_hjm_cuda_gb300 import _lib
from cva_hjm_cuda_gb300.engine import calibrate_pca
from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS, Market, nelson_siegel_curve, poly_vols, tenor_grid


def _history(n_obs: int, nt: int = 51, seed: int = 7, coeffs=DEFAULT_VOL_COEFFS, obs_per_year: float = 252.0):
    """Curves whose daily changes are sum_k sigma_k(T) sqrt(1/252) Z_k plus a small drift."""
    rng = np.random.default_rng(seed)
    tau = tenor_grid(nt, 0.5)
    vol = poly_vols(tau, coeffs)
    z = rng.standard_normal((n_obs - 1, 3))
    dx = z @ vol / np.sqrt(obs_per_year) + 1e-5
    return np.vstack([nelson_siegel_curve(tau), nelson_siegel_curve(tau) + np.cumsum(dx, axis=0)]), vol


def _numpy_pca(curves, dtau, obs_per_year):
    d = np.diff(curves, axis=0)
    cov = np.cov(d, rowvar=False) * obs_per_year
    w, v = np.linalg.eigh(cov)
    idx = np.argsort(w)[::-1][:3]
    vols = []
    for k in idx:
        e = v[:, k]
        e = e if e[np.argmax(np.abs(e))] > 0 else -e
        vols.append(np.sqrt(max(w[k], 0.0)) * e)
    return np.array(vols), w[idx], w[idx].sum() / np.trace(cov)


@pytest.fixture(scope="module")
def lib():
    if not _lib.LIB_PATH.exists():
        from cva_hjm_cuda_gb300 import build

        build.build()
    return _lib.load()


@pytest.mark.parametrize("nt,n_obs", [(51, 500), (61, 2000), (5, 40)])
def test_matches_numpy_pca_and_polyfit(lib, nt, n_obs):
    curves, _ = _history(n_obs, nt)
    cal = calibrate_pca(curves, 0.5, 252.0)
    vol, eig, expl = _numpy_pca(curves, 0.5, 252.0)
    np.testing.assert_allclose(cal.eigval, eig, rtol=1e-9)
    np.testing.assert_allclose(cal.vol, vol, rtol=1e-7, atol=1e-9 * np.max(np.abs(vol)))
    assert cal.explained == pytest.approx(expl, rel=1e-9)
    tau = tenor_grid(nt, 0.5)
    for k in range(3):
        deg = min(k, 2)
        ref = np.polyfit(tau, cal.vol[k], deg)[::-1]
        np.testing.assert_allclose(cal.vol_coeffs[k, : deg + 1], ref, rtol=1e-8, atol=1e-12)
        assert np.all(cal.vol_coeffs[k, deg + 1:] == 0.0)


def test_recovers_the_model_covariance():
    curves, vol = _history(40000, 51, seed=11)
    cal = calibrate_pca(curves, 0.5, 252.0)
    model_cov = vol.T @ vol
    fit_cov = cal.vol.T @ cal.vol
    # three factors carry all the variance of a three-factor history
    assert cal.explained > 1 - 1e-12
    err = np.max(np.abs(fit_cov - model_cov)) / np.max(np.abs(model_cov))
    assert err < 0.03, err  # sampling error of 40,000 changes: ~1.5 %


def test_calibrated_market_round_trip():
    curves, _ = _history(3000, 51, seed=3)
    cal = calibrate_pca(curves)
    mk = cal.market(curves[-1])
    assert mk.vol.shape == (3, 51)
    np.testing.assert_allclose(mk.vol, poly_vols(tenor_grid(51, 0.5), cal.vol_coeffs))
    raw = cal.market(curves[-1], poly=False)
    np.testing.assert_array_equal(raw.vol, cal.vol)


def test_rejects_bad_input(lib):
    with pytest.raises(_lib.HJMError):
        calibrate_pca(np.zeros((2, 51)))  # fewer than 3 curves
    with pytest.raises(_lib.HJMError):
        calibrate_pca(np.zeros((10, 51)))  # no changes
    bad = np.ones((10, 51))
    bad[3, 4] = np.nan
    with pytest.raises(_lib.HJMError):
        calibrate_pca(bad)
    with pytest.raises(_lib.HJMError):
        calibrate_pca(np.ones((10, 70)))  # beyond the tenor capacity


@pytest.mark.gpu
def test_calibrated_market_valuation_vs_oracle(engine):
    """History -> factors -> valuation: the calibrated polynomial market runs
    the decomposed step and matches the oracle on the device's normals."""
    import oracle_lib as O
    from cva_hjm_cuda_gb300.market import RunConfig, Swap

    curves, _ = _history(2500, 51, seed=5)
    cal = calibrate_pca(curves)
    mk = cal.market(nelson_siegel_curve(tenor_grid(51, 0.5)))
    sw = Swap()
    engine.set_market_poly(51, 0.5, mk.spot, cal.vol_coeffs)
    engine.set_swap(sw)
    assert engine.vol_form() == "poly_tri"
    cfg = RunConfig(n_paths=3000, seed=17)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    ee = O.expected_exposure(O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals))
    v = engine.run(cfg, "fp64")
    np.testing.assert_allclose(v.ee[:20], ee[:20], rtol=1e-10)
