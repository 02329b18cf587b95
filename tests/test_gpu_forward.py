"""GPU parity of the forward valuation (EE / PFE / CVA) against the oracle and
the reference's golden vectors, through the C ABI.

Tolerances: FP64 EE, PFE and CVA within 1e-10 relative of the oracle on
identical normals; mixed precision (FP32 curve and pricing, FP64 discount
accumulation and reductions) within 1e-4 relative per EE point and for CVA,
and inside the Monte Carlo standard error.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from conftest import market_from_golden
from cva_hjm_cuda_gb300 import _lib
from cva_hjm_cuda_gb300.market import Market, RunConfig, Swap, quantile_rank

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 1e-4


def _curand_normals(g):
    return O.curand_normals_double(g["normals"]["count"], seed=g["normals"]["seed"]).reshape(g["n_paths"], g["n_steps"], 3)


def _assert_rel(actual, desired, rtol, what, floor=None):
    actual, desired = np.asarray(actual), np.asarray(desired)
    scale = np.max(np.abs(desired)) if desired.size else 0.0
    err = np.abs(actual - desired)
    bad = err > rtol * np.maximum(np.abs(desired), 1e-300)
    # exact zeros must stay exact; tiny values are compared against the profile's scale
    bad &= err > (rtol * 1e-3 if floor is None else floor) * scale
    assert not np.any(bad), f"{what}: max rel err {np.max(err / np.maximum(np.abs(desired), 1e-300)):.3e}"


def _setup(engine, mk, sw):
    engine.set_market(mk)
    engine.set_swap(sw)


def _oracle_all(mk, sw, n_steps, dt, normals, n_dates, hazard=0.02, recovery=0.4, q=0.975):
    x = O.exposure_paths(mk, sw, n_steps, dt, normals)
    ee = O.expected_exposure(x)
    cva, dcva = O.cva(ee, n_dates, mk.dtau, hazard, recovery)
    c = O.cva_paths(x, n_dates, mk.dtau, hazard, recovery)
    pfe = O.pfe(x, n_dates, q)
    return x, ee, cva, dcva, c, pfe


# ---------------------------------------------------------------- normals / RNG
def test_philox_words_match_curand_host(engine):
    seed = 1234
    n = 1024
    words = engine.philox_words(n, step=0, seed=seed)
    ref = O.curand_philox_u32(4 * n, seed).reshape(n, 4)
    assert np.array_equal(words, ref)


def test_philox_words_match_oracle_any_counter(engine):
    seed = 0xDEADBEEF12345678
    words = engine.philox_words(64, step=777, seed=seed, path_offset=(1 << 32) - 5)
    for p in range(64):
        gp = (1 << 32) - 5 + p
        exp = O.philox((777, 0, gp & 0xFFFFFFFF, gp >> 32), (seed & 0xFFFFFFFF, seed >> 32))
        assert np.array_equal(words[p], exp)


def test_device_normals_close_to_host_transform(engine):
    dev = engine.dump_normals(64, 200, seed=1234)
    host = O.host_normals(1234, 0, 64, 200)
    # same Philox words; the SFU log/sincos differ from libm in the last bits only
    assert np.max(np.abs(dev - host)) < 2e-5
    assert np.array_equal(dev, engine.dump_normals(64, 200, seed=1234))


# --------------------------------------------------------- reference's own draws
def test_fp64_on_reference_draws_10y(engine, golden_10y):
    g = golden_10y
    mk, sw = market_from_golden(g)
    _setup(engine, mk, sw)
    normals = _curand_normals(g)
    engine.keep_exposures(True)
    v = engine.run_with_normals(normals, g["n_steps"], g["dt"], "fp64")
    _assert_rel(v.ee, g["ee"], FP64_RTOL, "EE vs reference")
    x = engine.exposures()  # [dates][paths]
    _assert_rel(x.T[:16], np.array(g["exposures_first_paths"])[:, :21], FP64_RTOL, "exposures vs reference")
    xo, ee, cva, dcva, c, pfe = _oracle_all(mk, sw, g["n_steps"], g["dt"], normals, 21)
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")
    _assert_rel(v.dcva_dhazard, dcva, FP64_RTOL, "dCVA/dhazard")
    _assert_rel(v.pfe[:21], pfe, FP64_RTOL, "PFE")
    assert np.all(v.pfe[21:] == 0) and np.all(v.ee[21:] == 0)
    engine.keep_exposures(False)


def test_fp64_on_reference_driver_draws_25y(engine, golden_25y):
    g = golden_25y
    mk, sw = market_from_golden(g)
    _setup(engine, mk, sw)
    v = engine.run_with_normals(_curand_normals(g), g["n_steps"], g["dt"], "fp64")
    _assert_rel(v.ee, g["ee"], FP64_RTOL, "EE vs reference driver")


def test_mixed_on_reference_draws_10y(engine, golden_10y):
    g = golden_10y
    mk, sw = market_from_golden(g)
    _setup(engine, mk, sw)
    v = engine.run_with_normals(_curand_normals(g), g["n_steps"], g["dt"], "mixed")
    _assert_rel(v.ee[:20], np.array(g["ee"])[:20], MIXED_RTOL, "mixed EE vs reference")


# --------------------------------------------------------- product path (Philox)
@pytest.fixture(scope="module")
def config1(engine):
    """Config 1 shape: 5,000 paths, 10y, dt 0.01, payer swap N=1e6 K=2.5%, hazard 2%, R 40%."""
    mk, sw = Market(), Swap()
    cfg = RunConfig(n_paths=5000, n_steps=1000, dt=0.01, seed=1234)
    _setup(engine, mk, sw)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    return mk, sw, cfg, normals, _oracle_all(mk, sw, cfg.n_steps, cfg.dt, normals, 21)


def test_fp64_philox_config1_vs_oracle(engine, config1):
    mk, sw, cfg, normals, (xo, ee, cva, dcva, c, pfe) = config1
    _setup(engine, mk, sw)
    engine.keep_exposures(True)
    v = engine.run(cfg, "fp64")
    x = engine.exposures()
    engine.keep_exposures(False)
    _assert_rel(v.ee, ee, FP64_RTOL, "EE")
    _assert_rel(x, xo[:, :21].T, FP64_RTOL, "exposures")
    # the all-FP64 step (convected remainder, FP64 parts) to FP64 rounding
    engine.keep_exposures(True)
    engine.set_remainder_form("convect")
    try:
        engine.run(cfg, "fp64")
        _assert_rel(engine.exposures(), xo[:, :21].T, FP64_RTOL, "all-FP64 exposures")
    finally:
        engine.set_remainder_form("auto")
        engine.keep_exposures(False)
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")
    _assert_rel(v.pfe[:21], pfe, FP64_RTOL, "PFE")
    se = c.std(ddof=1) / np.sqrt(len(c))
    _assert_rel(v.cva_stderr, se, 1e-8, "CVA stderr")
    # the per-path CVA contributions average to the EE-based CVA
    assert abs(c.mean() - cva) < 1e-12 * cva


def test_mixed_philox_config1_vs_fp64_oracle(engine, config1):
    mk, sw, cfg, normals, (xo, ee, cva, dcva, c, pfe) = config1
    _setup(engine, mk, sw)
    v = engine.run(cfg, "mixed")
    rel = np.abs(v.ee[:20] - ee[:20]) / ee[:20]
    assert np.max(rel) < MIXED_RTOL, f"per-point EE rel err {rel}"
    assert abs(v.cva - cva) < MIXED_RTOL * cva
    assert abs(v.cva - cva) < v.cva_stderr
    _assert_rel(v.pfe[:20], pfe[:20], MIXED_RTOL, "mixed PFE")


def test_external_normals_reproduce_philox_path(engine, config1):
    """The same kernel fed the dumped normals gives the Philox run's numbers."""
    mk, sw, cfg, normals, _ = config1
    _setup(engine, mk, sw)
    a = engine.run(cfg, "fp64")
    b = engine.run_with_normals(normals, cfg.n_steps, cfg.dt, "fp64")
    np.testing.assert_array_equal(a.ee, b.ee)
    assert a.cva == b.cva


# ------------------------------------------------------------------ properties
def test_runs_are_bitwise_deterministic(engine):
    _setup(engine, Market(), Swap())
    cfg = RunConfig(n_paths=20000)
    for prec in ("fp64", "mixed"):
        a, b = engine.run(cfg, prec), engine.run(cfg, prec)
        assert np.array_equal(a.ee, b.ee) and np.array_equal(a.pfe, b.pfe) and a.cva == b.cva


def test_path_sharding_reproduces_full_run(engine):
    """Counter-based normals: paths [0,N) equal paths [0,N/2) + [N/2,N)."""
    _setup(engine, Market(), Swap())
    n = 2 * 3000
    full = engine.run(RunConfig(n_paths=n), "fp64", pfe=False)
    h1 = engine.run(RunConfig(n_paths=n // 2), "fp64", pfe=False)
    h2 = engine.run(RunConfig(n_paths=n // 2, path_offset=n // 2), "fp64", pfe=False)
    _assert_rel((h1.ee + h2.ee) / 2, full.ee, 1e-13, "sharded EE")


def test_pfe_is_exact_order_statistic(engine):
    _setup(engine, Market(), Swap())
    engine.keep_exposures(True)
    for prec, n in (("fp64", 10007), ("mixed", 4099)):
        cfg = RunConfig(n_paths=n, pfe_quantile=0.9)
        v = engine.run(cfg, prec)
        x = engine.exposures()
        k = quantile_rank(0.9, n)
        np.testing.assert_array_equal(v.pfe[:21], np.sort(x, axis=1)[:, k - 1])
    engine.keep_exposures(False)


def test_tiny_and_ragged_path_counts(engine):
    _setup(engine, Market(), Swap())
    for n in (1, 2, 127, 129):
        cfg = RunConfig(n_paths=n)
        v = engine.run(cfg, "fp64")
        normals = engine.dump_normals(n, cfg.n_steps, cfg.seed)
        _, ee, cva, _, _, pfe = _oracle_all(Market(), Swap(), cfg.n_steps, cfg.dt, normals, 21)
        _assert_rel(v.ee, ee, FP64_RTOL, f"EE n={n}")
        _assert_rel(v.pfe[:21], pfe, FP64_RTOL, f"PFE n={n}")


def test_dropin_entry_point_matches_c_abi(engine):
    """calculateExposureMultiGPU (simulation_gpu.h:12) through the C++ drop-in."""
    from cva_hjm_cuda_gb300.engine import calculate_exposure_gpu

    mk, sw = Market(), Swap()
    _setup(engine, mk, sw)
    ref = engine.run(RunConfig(n_paths=3000, seed=1234), "fp64", pfe=False)
    ee = np.zeros(51)
    calculate_exposure_gpu(ee, sw.notional, sw.strike, 10.0, 0.5, sw.accrual, mk.spot, mk.drift, mk.vol.ravel(),
                           0.0, 1, 3000, 0.01)
    np.testing.assert_array_equal(ee, ref.ee)


def test_invalid_arguments_raise(engine):
    _setup(engine, Market(), Swap())
    for kw, status in (({"n_steps": 1010}, 1), ({"n_steps": 2550}, 1), ({"n_paths": 0}, 1), ({"dt": 0.0}, 1)):
        cfg = RunConfig(**kw)
        with pytest.raises(_lib.HJMError) as ei:
            engine.run(cfg, "fp64")
        assert ei.value.status == status
    with pytest.raises(KeyError):
        engine.run(RunConfig(), "fp16")


def test_enqueue_fetch_and_timings(engine):
    _setup(engine, Market(), Swap())
    cfg = RunConfig(n_paths=8192)
    engine.enqueue(cfg, "mixed")
    v = engine.fetch()
    t = engine.timings()
    assert v.cva > 0 and t["path_ms"] > 0 and t["total_ms"] >= t["path_ms"]


def test_fma_peaks_are_measured(engine):
    fp64 = engine.fma_peak_tflops("fp64")
    fp32 = engine.fma_peak_tflops("mixed")
    assert fp64 > 0.1 and fp32 > 10.0 and fp32 > fp64


def test_coarsest_time_step(engine):
    """dt = dtau/2 (c = 0.5, the largest the growth-scaled step takes): FP64
    and mixed match the oracle; on 61 tenors with 60 dates the FP32 scaled
    curve would grow by e^83, so mixed precision is refused while FP64 runs."""
    mk, sw = Market(), Swap()
    _setup(engine, mk, sw)
    cfg = RunConfig(n_paths=2000, n_steps=40, dt=0.25, seed=5)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x, ee, cva, *_ = _oracle_all(mk, sw, cfg.n_steps, cfg.dt, normals, 21)
    v = engine.run(cfg, "fp64")
    _assert_rel(v.ee, ee, FP64_RTOL, "EE c=0.5")
    m = engine.run(cfg, "mixed")
    _assert_rel(m.ee[:20], ee[:20], MIXED_RTOL, "mixed EE c=0.5")

    mk61, sw61 = Market(n_tenor=61), Swap(n_tenor=61, n_periods=60)
    _setup(engine, mk61, sw61)
    long = RunConfig(n_paths=500, n_steps=120, dt=0.25, seed=6)
    with pytest.raises(_lib.HJMError) as ei:
        engine.run(long, "mixed")
    assert ei.value.status == 2
    normals = engine.dump_normals(long.n_paths, long.n_steps, long.seed)
    x, ee, *_ = _oracle_all(mk61, sw61, long.n_steps, long.dt, normals, 61)
    _assert_rel(engine.run(long, "fp64").ee[:61], ee[:61], FP64_RTOL, "EE 61 tenors c=0.5")


@pytest.mark.parametrize("n_steps", [50, 100])
def test_one_and_two_dates_every_mode(engine, n_steps):
    """The shortest runs: one block (date 1 only, no evolution) and two
    blocks, through FP64, mixed, predictor-corrector, the adjoint and the
    multi-level estimator."""
    from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS

    mk, sw = Market(), Swap(n_periods=2)
    _setup(engine, mk, sw)
    cfg = RunConfig(n_paths=777, n_steps=n_steps, dt=0.01, seed=2)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    n_dates = n_steps // 50 + 1
    x, ee, cva, *_ = _oracle_all(mk, sw, cfg.n_steps, cfg.dt, normals, n_dates)
    _assert_rel(engine.run(cfg, "fp64").ee[:n_dates], ee[:n_dates], FP64_RTOL, "fp64")
    _assert_rel(engine.run(cfg, "mixed").ee[:n_dates], ee[:n_dates], MIXED_RTOL, "mixed")
    engine.set_scheme("predictor_corrector")
    try:
        xp = O.exposure_paths_pc(mk, sw, cfg.n_steps, cfg.dt, normals)
        _assert_rel(engine.run(cfg, "fp64").ee[:n_dates], O.expected_exposure(xp)[:n_dates], FP64_RTOL, "pc")
    finally:
        engine.set_scheme("euler")
    engine.set_market_poly(51, 0.5, mk.spot, DEFAULT_VOL_COEFFS)
    engine.set_swap(sw)
    v = engine.run(cfg, "mixed", pfe=False)
    for k in (0, 32):  # (the response form's adjoint, the convected one's)
        s = engine.run_adjoint(cfg, checkpoint_every=k)
        assert abs(s.cva - v.cva) <= 1e-6 * abs(v.cva) and np.all(np.isfinite(s.dcva_dspot))
    m = engine.run_mlmc([777, 512], n_steps=n_steps // 2, dt=0.02, seed=2)
    assert np.isfinite(m["cva"]) and m["levels"][1]["n_paths"] == 512


@pytest.mark.slow
def test_large_run_equals_its_halves(engine):
    """33,554,432 paths (2^25) in mixed precision with PFE: a 2.8 GB exposure
    store and 524,288 CTAs.  The full run's EE and CVA equal the path-weighted
    mean of its two halves run separately through path_offset (the same
    normals), up to the reduction's rounding."""
    _setup(engine, Market(), Swap())
    n = 1 << 25
    full = engine.run(RunConfig(n_paths=n, seed=9), "mixed")
    a = engine.run(RunConfig(n_paths=n // 2, seed=9), "mixed", pfe=False)
    b = engine.run(RunConfig(n_paths=n // 2, seed=9, path_offset=n // 2), "mixed", pfe=False)
    np.testing.assert_allclose(full.ee, 0.5 * (a.ee + b.ee), rtol=1e-12, atol=1e-12 * np.max(full.ee))
    assert full.cva == pytest.approx(0.5 * (a.cva + b.cva), rel=1e-12)
    assert np.all(np.diff(full.pfe[:20]) < 0.5 * full.pfe[0])  # finite and ordered like a quantile profile
    assert np.all(full.pfe[:20] >= full.ee[:20])
