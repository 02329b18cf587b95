"""Parity at the configured full sizes, against the oracle.

A full-size launch has 16,384 to 65,536 CTAs in many waves, the cached
response table and 64-bit exposure-store offsets; the oracle cannot run a
million paths in a test, but the normals are counter-addressed by global path
index, so any path of the full launch can be re-priced alone.  Each test runs
the configured workload once with the per-path exposures kept, then re-prices
4,096 of its paths with the oracle on their own normals (hjm_dump_normals at
the path's offset): 64 runs of 64 consecutive paths spread over the whole
launch -- the first and the last CTA, CTAs of the last (tail) wave, and runs
that straddle two CTAs.

* config 2: 1,048,576 paths x 1,000 steps, FP64: per-path exposures within
  1e-10 relative (1e-13 of the exposure scale for values near zero);
* config 3: 4,194,304 paths, mixed precision: within 1e-4 of the exposure scale;
* the reference driver's PCA table at 1,048,576 paths, FP64 (the cubic form
  with its residual): as config 2;
* config 4: 1,048,576 paths, the adjoint: checkpoints every 32 steps against
  the store-the-seeds mode (1e-4), and the gradient of the whole run equal to
  the mean of the gradients of its 16 path ranges (the estimator is a path
  mean; 1e-12 relative), and one range deep inside the launch against central
  finite differences of the FP64 valuation of its paths (2e-3).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from conftest import load_golden
from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS, Market, RunConfig, Swap, nelson_siegel_curve, tenor_grid

pytestmark = pytest.mark.gpu

RUN = 64  # consecutive paths per sampled run


def _sample_starts(n_paths: int, cta: int) -> list[int]:
    n_ctas = n_paths // cta
    starts = {0, n_paths - RUN, n_paths - cta * 3, n_paths // 2 + cta // 2, n_paths // 3 + 5}
    for k in range(1, 60):
        starts.add((k * n_ctas // 60) * cta)
    starts = sorted(s for s in starts if 0 <= s <= n_paths - RUN)
    return starts[:64]


def _resample(engine, mk, sw, cfg, x_dev, starts, n_dates):
    """Oracle exposures of the sampled runs and the device's for the same paths."""
    got, want = [], []
    for s0 in starts:
        normals = engine.dump_normals(RUN, cfg.n_steps, cfg.seed, path_offset=cfg.path_offset + s0)
        want.append(O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)[:, :n_dates])
        got.append(x_dev[:n_dates, s0:s0 + RUN].T)
    return np.concatenate(got), np.concatenate(want)


def _full_run(engine, cfg, precision):
    mk, sw = Market(), Swap()
    engine.set_market(mk)
    engine.set_swap(sw)
    engine.keep_exposures(True)
    try:
        v = engine.run(cfg, precision, pfe=False)
        x = engine.exposures()  # [dates][paths]
    finally:
        engine.keep_exposures(False)
    return mk, sw, v, x


def test_config2_fp64_sampled_paths_vs_oracle(engine):
    cfg = RunConfig(n_paths=1_048_576, n_steps=1000, dt=0.01, seed=1234)
    mk, sw, v, x = _full_run(engine, cfg, "fp64")
    assert engine.remainder_form() == "response"
    starts = _sample_starts(cfg.n_paths, 64)
    assert len(starts) == 64 and starts[0] == 0 and starts[-1] == cfg.n_paths - RUN
    got, want = _resample(engine, mk, sw, cfg, x, starts, 21)
    scale = np.max(np.abs(want))
    err = np.abs(got - want)
    bad = (err > 1e-10 * np.abs(want)) & (err > 1e-13 * scale)
    assert not np.any(bad), f"max rel err {np.max(err / np.maximum(np.abs(want), 1e-300)):.3e}"
    # the EE of the full run is the mean of its exposures (reduction of 16,384 CTA rows)
    np.testing.assert_allclose(v.ee[:21], x[:21].mean(axis=1), rtol=1e-12, atol=1e-12 * np.max(v.ee))


def test_reference_table_1m_sampled_paths_vs_oracle(engine):
    """The reference driver's PCA table (cubic factors with a residual) at 1,048,576 paths,
    FP64, the 10y swap: the cubic response form's launch re-priced on 4,096 paths."""
    g = load_golden("ref_driver_own_market.json")
    mk, sw = Market(vol=np.array(g["vol"]).reshape(3, 51)), Swap()
    cfg = RunConfig(n_paths=1_048_576, n_steps=1000, dt=0.01, seed=1234)
    engine.set_market(mk)
    engine.set_swap(sw)
    assert engine.vol_form() == "cubic_resid"
    engine.keep_exposures(True)
    try:
        v = engine.run(cfg, "fp64", pfe=False)
        x = engine.exposures()
    finally:
        engine.keep_exposures(False)
    assert engine.remainder_form() == "response"
    got, want = _resample(engine, mk, sw, cfg, x, _sample_starts(cfg.n_paths, 64), 21)
    scale = np.max(np.abs(want))
    err = np.abs(got - want)
    bad = (err > 1e-10 * np.abs(want)) & (err > 1e-13 * scale)
    assert not np.any(bad), f"max rel err {np.max(err / np.maximum(np.abs(want), 1e-300)):.3e}"
    np.testing.assert_allclose(v.ee[:21], x[:21].mean(axis=1), rtol=1e-12, atol=1e-12 * np.max(v.ee))


def test_config3_mixed_sampled_paths_vs_oracle(engine):
    cfg = RunConfig(n_paths=4_194_304, n_steps=1000, dt=0.01, seed=1234)
    mk, sw, v, x = _full_run(engine, cfg, "mixed")
    starts = _sample_starts(cfg.n_paths, 128)
    got, want = _resample(engine, mk, sw, cfg, x, starts, 21)
    scale = np.max(np.abs(want))
    assert np.max(np.abs(got - want)) <= 1e-4 * scale
    np.testing.assert_allclose(v.ee[:21], x[:21].mean(axis=1), rtol=1e-9, atol=1e-9 * np.max(v.ee))


def test_config4_adjoint_full_size(engine):
    tau = tenor_grid(51, 0.5)
    engine.set_market_poly(51, 0.5, nelson_siegel_curve(tau), DEFAULT_VOL_COEFFS)
    engine.set_swap(Swap())
    n = 1_048_576
    cfg = RunConfig(n_paths=n, seed=1234)
    a32 = engine.run_adjoint(cfg, checkpoint_every=32)
    a0 = engine.run_adjoint(cfg, checkpoint_every=0)  # the response form's adjoint
    assert abs(a32.cva - a0.cva) <= 1e-6 * a0.cva
    for name in ("dcva_dspot", "dcva_ddrift"):
        g32, g0 = getattr(a32, name), getattr(a0, name)
        np.testing.assert_allclose(g32, g0, rtol=1e-4, atol=1e-4 * np.max(np.abs(g0)), err_msg=name)
    np.testing.assert_allclose(a32.dcva_dvolcoef, a0.dcva_dvolcoef, rtol=1e-4,
                               atol=1e-4 * np.max(np.abs(a0.dcva_dvolcoef)))
    # the estimator is a mean over paths: the whole run's gradient is the mean of
    # the gradients of its 16 path ranges
    parts = [engine.run_adjoint(RunConfig(n_paths=n // 16, seed=1234, path_offset=k * (n // 16)),
                                checkpoint_every=32) for k in range(16)]
    for name in ("dcva_dspot", "dcva_ddrift", "dcva_dvolcoef"):
        whole = getattr(a32, name)
        mean = np.mean([getattr(p, name) for p in parts], axis=0)
        np.testing.assert_allclose(whole, mean, rtol=1e-12, atol=1e-12 * np.max(np.abs(whole)), err_msg=name)
    assert abs(a32.cva - np.mean([p.cva for p in parts])) <= 1e-12 * a32.cva
    # one of those ranges, deep inside the launch, against central finite
    # differences of the FP64 valuation of the same paths (bump 1e-5, within
    # 2e-3 of the difference or 1 % of the largest forward sensitivity)
    k = 11
    part = parts[k]
    spot = nelson_siegel_curve(tau)

    def val(sp, hz=0.02):
        engine.set_market_poly(51, 0.5, sp, DEFAULT_VOL_COEFFS)
        c = RunConfig(n_paths=n // 16, seed=1234, path_offset=k * (n // 16), hazard=hz)
        return engine.run(c, "fp64", pfe=False).cva

    gmax = np.max(np.abs(part.dcva_dspot))
    for t in (5, 15, 19):
        up, dn = spot.copy(), spot.copy()
        up[t] += 1e-5
        dn[t] -= 1e-5
        fd = (val(up) - val(dn)) / 2e-5
        assert abs(part.dcva_dspot[t] - fd) <= 2e-3 * max(abs(fd), 0.01 * gmax), (t, part.dcva_dspot[t], fd)
    fd = (val(spot, 0.02 + 1e-5) - val(spot, 0.02 - 1e-5)) / 2e-5
    assert abs(part.dcva_dhazard - fd) <= 1e-6 * abs(fd)
