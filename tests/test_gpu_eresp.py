"""GPU parity of the generalised FP64 Euler response form (hjm_eresp.cu).

* The reference driver's own volatility table (simulation_gpu_testing.cpp:47-63,
  cubic factors to its 9-decimal rounding) runs the cubic decomposition with
  its residual table: per-path exposures, EE, PFE and CVA within 1e-10 of
  the oracle on the device's normals, and within 1e-11 of the convected table
  step on the same paths, at the 10y shape (one window) and at the driver's
  own 25y swap with its irregular accruals (50 dates: three windows).
* Runs of more than 24 dates in windows, for quadratic factors too: the 30y
  swap and the 64-swap netting set on 61 tenors (60 dates), ragged path
  counts, PFE (every window's exposure rows), strides 25 to 100 (beyond 112
  steps per block the cubic frame's coefficients are read through L1).
* External FP64 normals through the windows (the reference's own draws are in
  test_dropin.py).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from conftest import load_golden, market_from_golden
from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS, Market, RunConfig, Swap, random_netting_set

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
# Per-path exposures near zero have no relative accuracy: E_j sums up to 50
# cash flows of either sign.  Values below floor x the exposure scale are
# compared absolutely.  For runs of at most 24 dates 1e-13 holds (the response
# form's double-FP32 parts leave ~5e-14 of the scale); over 50 dates and 2,500
# steps the all-FP64 convected step itself is 1.1e-13 of the scale from the
# oracle (the two order their FP64 operations differently) and the response
# form ~2.4e-13, so longer runs take 5e-13.
LONG_RUN_FLOOR = 5e-13


def _floor(n_dates):
    return 1e-13 if n_dates <= 24 else LONG_RUN_FLOOR


def _assert_rel(actual, desired, rtol, what, floor=1e-13):
    actual, desired = np.asarray(actual), np.asarray(desired)
    scale = np.max(np.abs(desired)) if desired.size else 0.0
    err = np.abs(actual - desired)
    bad = (err > rtol * np.maximum(np.abs(desired), 1e-300)) & (err > floor * scale)
    assert not np.any(bad), f"{what}: max rel err {np.max(err / np.maximum(np.abs(desired), 1e-300)):.3e}"


@pytest.fixture
def remainder_form(engine):
    yield engine.set_remainder_form
    engine.set_remainder_form("auto")


def _own_market():
    g = load_golden("ref_driver_own_market.json")
    return market_from_golden(g)


def _run_and_oracle(engine, mk, sw, cfg, nd):
    engine.keep_exposures(True)
    try:
        v = engine.run(cfg, "fp64")
        x = engine.exposures()
    finally:
        engine.keep_exposures(False)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed, cfg.path_offset)
    xo = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(xo)
    cva, dcva = O.cva(ee, nd + 1, mk.dtau, cfg.hazard, cfg.recovery)
    pfe = O.pfe(xo, nd + 1, cfg.pfe_quantile)
    return v, x, xo, ee, cva, pfe


@pytest.mark.parametrize("shape", ["10y-synthetic-swap", "25y-driver-swap"])
def test_reference_table_cubic_form_vs_oracle(engine, remainder_form, shape):
    mk, drv = _own_market()
    if shape == "10y-synthetic-swap":
        sw, n_steps, n_paths = Swap(), 1000, 3000
    else:
        sw, n_steps, n_paths = drv, 2500, 1500  # N = 10, K = 6.7%, the driver's accruals
    engine.set_market(mk)
    engine.set_swap(sw)
    assert engine.vol_form() == "cubic_resid"
    nd = n_steps // 50
    cfg = RunConfig(n_paths=n_paths, n_steps=n_steps, dt=0.01, seed=2024, path_offset=1000)
    v, x, xo, ee, cva, pfe = _run_and_oracle(engine, mk, sw, cfg, nd)
    assert engine.remainder_form() == "response"
    _assert_rel(x, xo[:, :nd + 1].T, FP64_RTOL, "exposures", floor=_floor(nd))
    _assert_rel(v.ee[:nd + 1], ee[:nd + 1], FP64_RTOL, "EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")
    _assert_rel(v.pfe[:nd + 1], pfe, FP64_RTOL, "PFE", floor=_floor(nd))
    # the convected table step on the same paths (every operation of the curve in FP64)
    remainder_form("convect")
    engine.keep_exposures(True)
    try:
        vc = engine.run(cfg, "fp64")
        xc = engine.exposures()
    finally:
        engine.keep_exposures(False)
    assert engine.remainder_form() == "convect"
    _assert_rel(x, xc, 1e-11, "exposures response vs convected table step", floor=_floor(nd))
    _assert_rel(v.cva, vc.cva, 1e-12, "CVA response vs convected")


@pytest.mark.parametrize("n_paths", [1, 63, 257])
def test_windows_30y_quadratic_vs_oracle(engine, remainder_form, n_paths):
    mk = Market(n_tenor=61)
    engine.set_market_poly(61, mk.dtau, mk.spot, DEFAULT_VOL_COEFFS)
    sw = Swap(n_tenor=61, n_periods=60)
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=n_paths, n_steps=3000, dt=0.01, seed=11)
    v, x, xo, ee, cva, pfe = _run_and_oracle(engine, mk, sw, cfg, 60)
    assert engine.remainder_form() == "response"
    _assert_rel(x, xo[:, :61].T, FP64_RTOL, "exposures", floor=LONG_RUN_FLOOR)
    _assert_rel(v.ee[:61], ee[:61], FP64_RTOL, "EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")
    _assert_rel(v.pfe[:61], pfe, FP64_RTOL, "PFE", floor=LONG_RUN_FLOOR)
    if n_paths >= 63:
        remainder_form("convect")
        vc = engine.run(cfg, "fp64")
        _assert_rel(v.ee[:61], vc.ee[:61], 1e-12, "EE response vs convect")


def test_windows_netting_set_fp64_vs_oracle(engine):
    mk = Market(n_tenor=61)
    engine.set_market_poly(61, mk.dtau, mk.spot, DEFAULT_VOL_COEFFS)
    ns = random_netting_set(64, seed=20261203)
    engine.set_netting_set(ns)
    cfg = RunConfig(n_paths=400, n_steps=3000, dt=0.01, seed=3)
    v = engine.run(cfg, "fp64")
    assert engine.remainder_form() == "response"
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    payA, payB = ns.payoff_vectors(61, mk.dtau)
    xo = O.exposure_paths_netting(mk, payA, payB, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(xo)
    cva, _ = O.cva(ee, 61, mk.dtau, cfg.hazard, cfg.recovery)
    _assert_rel(v.ee[:61], ee[:61], FP64_RTOL, "netting EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "netting CVA")


@pytest.mark.parametrize("dt,n_steps", [(0.02, 1000), (0.005, 3000), (0.02, 1250)],
                         ids=["stride25-40-dates", "stride100-30-dates-L1-coefficients", "stride25-50-dates"])
def test_cubic_windows_strides_vs_oracle(engine, dt, n_steps):
    mk, _ = _own_market()
    engine.set_market(mk)
    stride = int(round(0.5 / dt))
    nd = n_steps // stride
    sw = Swap(n_periods=nd)
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=200, n_steps=n_steps, dt=dt, seed=9)
    v, x, xo, ee, cva, pfe = _run_and_oracle(engine, mk, sw, cfg, nd)
    assert engine.remainder_form() == "response"
    _assert_rel(x, xo[:, :nd + 1].T, FP64_RTOL, "exposures", floor=_floor(nd))
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")


def test_windows_on_external_double_normals(engine):
    """FP64 normals that FP32 cannot hold, through the three windows of the driver's 25y swap."""
    mk, sw = _own_market()
    engine.set_market(mk)
    engine.set_swap(sw)
    n_paths, n_steps = 130, 2500
    normals = np.random.default_rng(5).standard_normal((n_paths, n_steps, 3))
    v = engine.run_with_normals(normals, n_steps, 0.01, "fp64")
    assert engine.remainder_form() == "response"
    xo = O.exposure_paths(mk, sw, n_steps, 0.01, normals)
    ee = O.expected_exposure(xo)
    _assert_rel(v.ee, ee, FP64_RTOL, "EE")


@pytest.mark.parametrize("shape", ["10y-synthetic-swap", "25y-driver-swap"])
def test_cubic_market_mixed_precision_vs_fp64_and_oracle(engine, shape, tmp_path):
    """Mixed precision on the driver's table runs the cubic polynomial form (its
    residual, 1.1e-7 of the factors' scale, left out; the 10y swap with the
    remainder's FP32 responses, the 25y swap convected): EE and CVA within 1e-4 of
    the FP64 run on the same paths, per-path exposures within 1e-4 of the
    exposure scale from the oracle on the full table.  The predictor-corrector
    scheme takes the table step on such a market."""
    import json

    mk, drv = _own_market()
    sw, n_steps = (Swap(), 1000) if shape.startswith("10y") else (drv, 2500)
    engine.set_market(mk)
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=2000, n_steps=n_steps, dt=0.01, seed=4)
    nd = n_steps // 50
    f64 = engine.run(cfg, "fp64")
    engine.keep_exposures(True)
    try:
        mx = engine.run(cfg, "mixed")
        x = engine.exposures()
    finally:
        engine.keep_exposures(False)
    # the FP32 response form where the counting dates fit its slots (10y: 8)
    assert engine.remainder_form() == ("response" if shape.startswith("10y") else "convect")
    engine.write_report(tmp_path / "r.json")
    assert json.loads((tmp_path / "r.json").read_text())["run"]["vol_form"] == "cubic_resid"
    np.testing.assert_allclose(mx.ee[:nd], f64.ee[:nd], rtol=1e-4)
    assert abs(mx.cva - f64.cva) <= 1e-4 * f64.cva
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    xo = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)[:, :nd + 1].T
    assert np.max(np.abs(x - xo)) <= 1e-4 * np.max(np.abs(xo))
    engine.set_scheme("predictor_corrector")
    try:
        engine.run(cfg, "mixed")
        engine.write_report(tmp_path / "p.json")
        assert json.loads((tmp_path / "p.json").read_text())["run"]["vol_form"] == "table"
    finally:
        engine.set_scheme("euler")
