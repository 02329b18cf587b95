"""GPU parity of the polynomial-volatility path (hjm_set_market_poly).

With every factor a polynomial of degree <= 2 in the tenor T, the kernels
carry the stochastic curve as S + U T + W T^2 plus a convected remainder that
is driven only at the last tenor, instead of injecting the three factor
columns into every tenor each step.  The decomposition is exact algebra, so
the oracle's table-driven restatement of simulation_cpu.h (volatility table
sampled from the same polynomials, trapezoid drift) is the reference:

* FP64 EE, exposures, PFE and CVA within 1e-10 relative of the oracle;
* mixed precision within 1e-4 relative and inside the Monte Carlo error;
* external normals on the polynomial path reproduce the Philox run;
* the 30-year (61-tenor) grid, ragged path counts, and the netting set.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from cva_hjm_cuda_gb300.market import (DEFAULT_VOL_COEFFS, Market, RunConfig, Swap, nelson_siegel_curve,
                                       random_netting_set, tenor_grid)

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 1e-4
# Per-path exposures of the FP64 response form (the default FP64 step for
# quadratic factors) against the all-FP64 convected form: the response form's
# stochastic parts S, U, W and remainder are double-FP32 sums (2^-48 of the
# accumulator per addition within a block, FP64 across blocks), so a path's
# exposures differ by ~5e-14 of the exposure scale; against the oracle both
# forms meet FP64_RTOL with its default floor (1e-13 of the scale).
EXPOSURE_FLOOR = 1e-13


def _assert_rel(actual, desired, rtol, what, floor=None):
    actual, desired = np.asarray(actual), np.asarray(desired)
    scale = np.max(np.abs(desired)) if desired.size else 0.0
    err = np.abs(actual - desired)
    bad = err > rtol * np.maximum(np.abs(desired), 1e-300)
    bad &= err > (rtol * 1e-3 if floor is None else floor) * scale
    assert not np.any(bad), f"{what}: max rel err {np.max(err / np.maximum(np.abs(desired), 1e-300)):.3e}"


def _poly_market(engine, nt=51, coef=DEFAULT_VOL_COEFFS):
    mk = Market(n_tenor=nt, vol_coeffs=np.array(coef))
    engine.set_market_poly(nt, mk.dtau, mk.spot, coef)
    return mk


@pytest.fixture(scope="module")
def poly_config1(engine):
    mk = _poly_market(engine)
    sw = Swap()
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=5000, n_steps=1000, dt=0.01, seed=4321)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, _ = O.cva(ee, 21, mk.dtau, cfg.hazard, cfg.recovery)
    pfe = O.pfe(x, 21, cfg.pfe_quantile)
    return mk, sw, cfg, normals, x, ee, cva, pfe


def test_poly_fp64_vs_oracle(engine, poly_config1):
    mk, sw, cfg, normals, xo, ee, cva, pfe = poly_config1
    _poly_market(engine)
    engine.set_swap(sw)
    engine.keep_exposures(True)
    v = engine.run(cfg, "fp64")
    x = engine.exposures()
    engine.keep_exposures(False)
    _assert_rel(x, xo[:, :21].T, FP64_RTOL, "exposures")
    _assert_rel(v.ee, ee, FP64_RTOL, "EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")
    _assert_rel(v.pfe[:21], pfe, FP64_RTOL, "PFE")


def test_poly_mixed_vs_oracle(engine, poly_config1):
    mk, sw, cfg, normals, xo, ee, cva, pfe = poly_config1
    _poly_market(engine)
    engine.set_swap(sw)
    v = engine.run(cfg, "mixed")
    rel = np.abs(v.ee[:20] - ee[:20]) / ee[:20]
    assert np.max(rel) < MIXED_RTOL, f"per-point EE rel err {rel}"
    assert abs(v.cva - cva) < MIXED_RTOL * cva
    assert abs(v.cva - cva) < v.cva_stderr
    _assert_rel(v.pfe[:20], pfe[:20], MIXED_RTOL, "mixed PFE")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_poly_external_normals_reproduce_philox(engine, poly_config1, precision):
    mk, sw, cfg, normals, *_ = poly_config1
    _poly_market(engine)
    engine.set_swap(sw)
    a = engine.run(cfg, precision)
    b = engine.run_with_normals(normals, cfg.n_steps, cfg.dt, precision)
    np.testing.assert_array_equal(a.ee, b.ee)
    assert a.cva == b.cva


@pytest.fixture
def generic_path(engine):
    """Force the generic table-driven Euler step for the test's duration."""
    engine.vol_decomposition(False)
    try:
        yield
    finally:
        engine.vol_decomposition(True)


def test_quadratic_table_is_detected_as_polynomial(engine, golden_10y):
    from conftest import market_from_golden

    mk, sw = market_from_golden(golden_10y)  # the configured workloads' synthetic factors
    engine.set_market(mk)
    assert engine.vol_decomposition()
    assert engine.vol_form() == "poly_tri"  # factor k of degree k, as fitted from the table
    # a bump of 1.6e-4 of the scale is neither a quadratic nor a cubic up to 2^-20
    bumped = Market(vol=mk.vol + 1e-6 * np.sin(np.arange(51))[None, :])
    engine.set_market(bumped)
    assert not engine.vol_decomposition()
    engine.vol_decomposition(False)
    engine.set_market(mk)
    assert not engine.vol_decomposition()
    engine.vol_decomposition(True)
    assert engine.vol_decomposition()


def test_generic_path_vs_oracle(engine, poly_config1, generic_path):
    mk, sw, cfg, normals, xo, ee, cva, pfe = poly_config1
    engine.set_market(mk)
    engine.set_swap(sw)
    assert not engine.vol_decomposition()
    v = engine.run(cfg, "fp64")
    _assert_rel(v.ee, ee, FP64_RTOL, "EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")
    _assert_rel(v.pfe[:21], pfe, FP64_RTOL, "PFE")
    m = engine.run(cfg, "mixed")
    assert np.max(np.abs(m.ee[:20] - ee[:20]) / ee[:20]) < MIXED_RTOL
    assert abs(m.cva - cva) < MIXED_RTOL * cva


def test_non_polynomial_table_vs_oracle(engine):
    """A table that is no quadratic runs the generic step, at the same parity."""
    mk = Market(vol=Market().vol * (1.0 + 0.1 * np.cos(np.arange(51) / 7.0))[None, :])
    sw = Swap()
    engine.set_market(mk)
    engine.set_swap(sw)
    assert not engine.vol_decomposition()
    cfg = RunConfig(n_paths=3000, seed=8)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, _ = O.cva(ee, 21, mk.dtau, cfg.hazard, cfg.recovery)
    v = engine.run(cfg, "fp64")
    _assert_rel(v.ee, ee, FP64_RTOL, "EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")


def test_poly_matches_table_market(engine):
    """The same market on the generic step and on the decomposition."""
    cfg = RunConfig(n_paths=30000, seed=99)
    mk = Market()
    engine.vol_decomposition(False)
    try:
        engine.set_market(mk)
        engine.set_swap(Swap())
        t64, tmx = engine.run(cfg, "fp64"), engine.run(cfg, "mixed")
    finally:
        engine.vol_decomposition(True)
    _poly_market(engine)
    engine.set_swap(Swap())
    p64, pmx = engine.run(cfg, "fp64"), engine.run(cfg, "mixed")
    _assert_rel(p64.ee, t64.ee, FP64_RTOL, "fp64 EE poly vs table")
    _assert_rel(p64.cva, t64.cva, FP64_RTOL, "fp64 CVA poly vs table")
    _assert_rel(pmx.ee[:20], tmx.ee[:20], MIXED_RTOL, "mixed EE poly vs table")
    assert abs(pmx.cva - tmx.cva) < MIXED_RTOL * tmx.cva


@pytest.mark.parametrize("n_paths", [1, 63, 257])
def test_poly_30y_ragged_vs_oracle(engine, n_paths):
    mk = _poly_market(engine, nt=61)
    sw = Swap(n_tenor=61, n_periods=60)
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=n_paths, n_steps=3000, dt=0.01, seed=11)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, _ = O.cva(ee, 61, mk.dtau, cfg.hazard, cfg.recovery)
    v = engine.run(cfg, "fp64")
    _assert_rel(v.ee[:61], ee[:61], FP64_RTOL, "30y EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "30y CVA")
    m = engine.run(cfg, "mixed")
    if n_paths >= 63:
        assert abs(m.cva - cva) < 1e-3 * cva


def test_poly_netting_set_vs_oracle(engine):
    mk = _poly_market(engine, nt=61)
    ns = random_netting_set(64)
    engine.set_netting_set(ns)
    payA, payB = ns.payoff_vectors(61)
    cfg = RunConfig(n_paths=2000, n_steps=3000, dt=0.01, seed=3)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x = O.exposure_paths_netting(mk, payA, payB, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, _ = O.cva(ee, 61, mk.dtau, cfg.hazard, cfg.recovery)
    v = engine.run(cfg, "fp64")
    _assert_rel(v.ee[:61], ee[:61], FP64_RTOL, "netting EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "netting CVA")


FULL_COEFFS = np.array([[0.0060, 0.00010, -0.000004],
                        [-0.0036, 0.00040, 0.000003],
                        [0.0020, -0.00060, 0.00002]])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_general_quadratic_factors_vs_oracle(engine, precision):
    """Quadratic factors without the triangular zeros take the full projection."""
    mk = _poly_market(engine, coef=FULL_COEFFS)
    assert engine.vol_form() == "poly"
    sw = Swap()
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=4000, seed=21)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, _ = O.cva(ee, 21, mk.dtau, cfg.hazard, cfg.recovery)
    v = engine.run(cfg, precision)
    tol = FP64_RTOL if precision == "fp64" else MIXED_RTOL
    _assert_rel(v.ee[:20], ee[:20], tol, "EE")
    _assert_rel(v.cva, cva, tol, "CVA")
    # the same market as a table is detected as the same (general) form
    engine.set_market(mk)
    assert engine.vol_form() == "poly"


# ---------------------------------------------------------------------------
# FP64 remainder forms: convected over the live tenors, or impulse responses
# at the sampled tenors (at most 24 dates)
# ---------------------------------------------------------------------------
@pytest.fixture
def remainder_form(engine):
    yield engine.set_remainder_form
    engine.set_remainder_form("auto")


def _oracle_run(engine, mk, sw, cfg):
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    nd = cfg.n_steps // int(round(mk.dtau / cfg.dt))
    cva, _ = O.cva(ee, nd + 1, mk.dtau, cfg.hazard, cfg.recovery)
    return x, ee, cva, O.pfe(x, nd + 1, cfg.pfe_quantile)


@pytest.mark.parametrize("nt,coef,n_steps", [(51, DEFAULT_VOL_COEFFS, 1000), (51, FULL_COEFFS, 1000),
                                             (61, DEFAULT_VOL_COEFFS, 1000), (51, DEFAULT_VOL_COEFFS, 1200)],
                         ids=["51-tri", "51-general", "61-tri", "51-tri-24-dates"])
def test_remainder_forms_agree_and_match_oracle(engine, remainder_form, nt, coef, n_steps):
    """The response form (double-FP32 parts and sums) against the all-FP64
    convected form on the same paths, 24 dates being the most the form takes
    (the remainder at the last date nearest the transport front, largest),
    and both against the oracle."""
    mk = _poly_market(engine, nt=nt, coef=coef)
    nd = n_steps // 50
    sw = Swap(n_tenor=nt, n_periods=nd)
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=3000, n_steps=n_steps, seed=77)
    out = {}
    engine.keep_exposures(True)
    try:
        for form in ("convect", "response"):
            remainder_form(form)
            v = engine.run(cfg, "fp64")
            assert engine.remainder_form() == form
            out[form] = (v, engine.exposures())
    finally:
        engine.keep_exposures(False)
    (vc, xc), (vr, xr) = out["convect"], out["response"]
    _assert_rel(xr, xc, 1e-12, "exposures response vs convect", floor=EXPOSURE_FLOOR)
    _assert_rel(vr.ee, vc.ee, 1e-12, "EE response vs convect")
    _assert_rel(vr.cva, vc.cva, 1e-12, "CVA response vs convect")
    x, ee, cva, pfe = _oracle_run(engine, mk, sw, cfg)
    _assert_rel(xr, x[:, :nd + 1].T, FP64_RTOL, "exposures vs oracle")
    _assert_rel(xc, x[:, :nd + 1].T, FP64_RTOL, "all-FP64 exposures vs oracle")
    _assert_rel(vr.ee, ee, FP64_RTOL, "EE vs oracle")
    _assert_rel(vr.cva, cva, FP64_RTOL, "CVA vs oracle")
    _assert_rel(vr.pfe[:nd + 1], pfe, FP64_RTOL, "PFE vs oracle")


@pytest.mark.parametrize("n_paths,n_steps,dt", [(1, 1000, 0.01), (63, 500, 0.02), (257, 1200, 0.01),
                                                (100, 250, 0.01), (64, 1000, 0.005), (100, 50, 0.05),
                                                (65, 1000, 0.004), (129, 1050, 0.01), (130, 1250, 0.01),
                                                (131, 1300, 0.01), (67, 1800, 0.01)],
                         ids=["1-path", "stride25", "24-dates", "5-dates", "stride100", "stride10-all-zero",
                              "stride125-coefficients-via-L1", "21-dates", "25-dates", "26-dates-one-window",
                              "36-dates-two-windows"])
def test_response_form_shapes_vs_oracle(engine, remainder_form, n_paths, n_steps, dt):
    """Ragged path counts, strides 10 to 125, 5 to 36 dates.  The remainder
    reaches dates 10 and later only (stride 50), so the windows hold slots
    from date 10 on: 20 and 21 dates in the 12-slot kernel, 24 and 25 in the
    16-slot one, 26 in one window of the 20-slot one, 36 in two windows
    (dates 13 to 36 in the 24-slot kernel, then 1 to 12 in the 12-slot one);
    with stride 10 the
    remainder never reaches a sampled tenor (all responses zero); beyond 112
    steps per block the frame's coefficients are read through L1 instead of
    shared memory."""
    mk = _poly_market(engine)
    stride = int(round(mk.dtau / dt))
    sw = Swap(n_periods=max(n_steps // stride, 1))
    engine.set_swap(sw)
    remainder_form("response")
    cfg = RunConfig(n_paths=n_paths, n_steps=n_steps, dt=dt, seed=5)
    v = engine.run(cfg, "fp64")
    assert engine.remainder_form() == "response"
    x, ee, cva, pfe = _oracle_run(engine, mk, sw, cfg)
    nd = n_steps // stride
    _assert_rel(v.ee[:nd + 1], ee[:nd + 1], FP64_RTOL, "EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")


def test_remainder_form_choice_and_limits(engine, remainder_form, tmp_path):
    import json

    from cva_hjm_cuda_gb300 import _lib

    _poly_market(engine)
    engine.set_swap(Swap())
    engine.run(RunConfig(n_paths=256), "fp64")
    assert engine.remainder_form() == "response"  # 20 dates on 51 tenors: the cheaper form
    engine.write_report(tmp_path / "r.json")
    assert json.loads((tmp_path / "r.json").read_text())["run"]["remainder"] == "response"
    engine.run(RunConfig(n_paths=256), "mixed")
    assert engine.remainder_form() == "response"  # mixed precision: the 10y swap's counting dates fit 8 slots
    _poly_market(engine, nt=61)
    engine.set_swap(Swap(n_tenor=61, n_periods=60))
    cfg30 = RunConfig(n_paths=256, n_steps=3000)
    engine.run(cfg30, "fp64")
    assert engine.remainder_form() == "response"  # 60 dates: three windows
    engine.run(cfg30, "mixed")
    assert engine.remainder_form() == "convect"  # mixed precision: 44 counting dates do not fit 16 slots
    remainder_form("convect")
    engine.run(cfg30, "fp64")
    assert engine.remainder_form() == "convect"
    # the volatility-table response form: 60 dates in windows as well
    engine.set_market(_bumpy_market(61))
    remainder_form("response")
    engine.run(cfg30, "fp64")
    assert engine.remainder_form() == "response"
    remainder_form("auto")
    engine.run(cfg30, "fp64")
    assert engine.remainder_form() == "response"
    engine.set_market(Market(vol=Market().vol * (1.0 + 0.1 * np.cos(np.arange(51) / 7.0))[None, :]))
    engine.set_swap(Swap())
    remainder_form("auto")
    engine.run(RunConfig(n_paths=256), "fp64")
    assert engine.remainder_form() == "response"  # table step: the factors' responses
    remainder_form("convect")
    engine.run(RunConfig(n_paths=256), "fp64")
    assert engine.remainder_form() == "convect"
    with pytest.raises(_lib.HJMError):
        _lib.check(engine.lib.hjm_ctx_set_remainder_form(engine.ctx, 7), engine.ctx)


# ---------------------------------------------------------------------------
# the volatility-table step (a table of any shape) in the response form: the
# whole stochastic curve as double-FP32 sums of the three factors' impulse
# responses
# ---------------------------------------------------------------------------
def _bumpy_market(nt=51):
    mk = Market(n_tenor=nt)
    return Market(n_tenor=nt, vol=mk.vol * (1.0 + 0.1 * np.cos(np.arange(nt) / 7.0))[None, :])


@pytest.mark.parametrize("scheme", ["euler", "predictor_corrector"])
@pytest.mark.parametrize("nt", [51, 61])
def test_table_step_response_vs_convected_and_oracle(engine, remainder_form, scheme, nt):
    mk = _bumpy_market(nt)
    sw = Swap(n_tenor=nt)
    engine.set_scheme(scheme)
    try:
        engine.set_market(mk)
        engine.set_swap(sw)
        assert engine.vol_form() == "table"
        cfg = RunConfig(n_paths=2500, seed=31)
        out = {}
        engine.keep_exposures(True)
        for form in ("convect", "response"):
            remainder_form(form)
            out[form] = (engine.run(cfg, "fp64"), engine.exposures())
            assert engine.remainder_form() == form
        remainder_form("auto")
        normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
        ext = engine.run_with_normals(normals, cfg.n_steps, cfg.dt, "fp64")
        assert engine.remainder_form() == "response"
    finally:
        engine.keep_exposures(False)
        engine.set_scheme("euler")
    (vc, xc), (vr, xr) = out["convect"], out["response"]
    # the response sums run in double-FP32 (2^-48 per addition, random-walk
    # over the run): exposures near zero compared absolutely below 1e-13 of
    # the scale, as for the decomposition's response form
    _assert_rel(xr, xc, 1e-11, "exposures response vs convect", floor=EXPOSURE_FLOOR)
    paths = O.exposure_paths_pc if scheme == "predictor_corrector" else O.exposure_paths
    x = paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, _ = O.cva(ee, 21, mk.dtau, cfg.hazard, cfg.recovery)
    _assert_rel(xr, x[:, :21].T, FP64_RTOL, "exposures vs oracle")
    _assert_rel(vr.ee[:21], ee[:21], FP64_RTOL, "EE vs oracle")
    _assert_rel(vr.cva, cva, FP64_RTOL, "CVA vs oracle")
    _assert_rel(vr.pfe[:21], O.pfe(x, 21, cfg.pfe_quantile), FP64_RTOL, "PFE vs oracle")
    np.testing.assert_array_equal(ext.ee, vr.ee)


@pytest.mark.parametrize("n_paths,n_steps,dt", [(1, 1000, 0.01), (257, 1200, 0.01), (63, 500, 0.02)],
                         ids=["1-path", "24-dates", "stride25"])
def test_table_step_response_shapes_vs_oracle(engine, remainder_form, n_paths, n_steps, dt):
    mk = _bumpy_market()
    engine.set_market(mk)
    stride = int(round(mk.dtau / dt))
    sw = Swap(n_periods=n_steps // stride)
    engine.set_swap(sw)
    remainder_form("response")
    cfg = RunConfig(n_paths=n_paths, n_steps=n_steps, dt=dt, seed=8)
    v = engine.run(cfg, "fp64")
    assert engine.remainder_form() == "response"
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    nd = n_steps // stride
    cva, _ = O.cva(ee, nd + 1, mk.dtau, cfg.hazard, cfg.recovery)
    _assert_rel(v.ee[:nd + 1], ee[:nd + 1], FP64_RTOL, "EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")


@pytest.mark.parametrize("scheme", ["euler", "predictor_corrector"])
@pytest.mark.parametrize("nt,n_steps", [(51, 2500), (61, 3000)], ids=["25y-51-tenors", "30y-61-tenors"])
def test_table_step_response_windows_vs_convected_and_oracle(engine, remainder_form, scheme, nt, n_steps):
    """More than 24 dates on a table of any shape: the response form prices
    them in windows of 24 (the latest first, the earlier ones taking the later
    cash flows per path); per-path exposures against the all-FP64 convected
    table step (1e-11) and the oracle (1e-10), both absolutely below 5e-13 of
    the scale (over 50 or 60 dates the FP64 forms themselves differ by ~1e-13
    of it)."""
    mk = _bumpy_market(nt)
    sw = Swap(n_tenor=nt, n_periods=n_steps // 50)
    engine.set_scheme(scheme)
    try:
        engine.set_market(mk)
        engine.set_swap(sw)
        assert engine.vol_form() == "table"
        cfg = RunConfig(n_paths=129, n_steps=n_steps, seed=41)
        out = {}
        engine.keep_exposures(True)
        for form in ("convect", "response"):
            remainder_form(form)
            out[form] = (engine.run(cfg, "fp64"), engine.exposures())
            assert engine.remainder_form() == form
        remainder_form("auto")
        normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
        ext = engine.run_with_normals(normals, cfg.n_steps, cfg.dt, "fp64")
    finally:
        engine.keep_exposures(False)
        engine.set_scheme("euler")
    (vc, xc), (vr, xr) = out["convect"], out["response"]
    nd = n_steps // 50 + 1
    _assert_rel(xr[:nd], xc[:nd], 1e-11, "exposures response vs convect", floor=5e-13)
    paths = O.exposure_paths_pc if scheme == "predictor_corrector" else O.exposure_paths
    x = paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, _ = O.cva(ee, nd, mk.dtau, cfg.hazard, cfg.recovery)
    _assert_rel(xr[:nd], x[:, :nd].T, FP64_RTOL, "exposures vs oracle", floor=5e-13)
    _assert_rel(vr.ee[:nd], ee[:nd], FP64_RTOL, "EE vs oracle")
    _assert_rel(vr.cva, cva, FP64_RTOL, "CVA vs oracle")
    np.testing.assert_array_equal(ext.ee, vr.ee)


def test_response_tables_follow_shape_market_and_scheme(engine):
    """The context caches the response tables per run shape, scheme, factor
    loadings (the parts' frame coefficients) and (table step) volatility
    table: alternating them on one context gives bit for bit what a fresh
    context gives for each case."""
    from cva_hjm_cuda_gb300 import HJMEngine

    cases = [
        ("poly", "euler", RunConfig(n_paths=700, seed=2)),
        ("poly-scaled", "euler", RunConfig(n_paths=700, seed=2)),
        ("poly", "euler", RunConfig(n_paths=700, seed=2)),
        ("table", "euler", RunConfig(n_paths=700, seed=2)),
        ("poly", "euler", RunConfig(n_paths=700, n_steps=500, dt=0.02, seed=2)),
        ("table2", "predictor_corrector", RunConfig(n_paths=700, seed=2)),
        ("table", "predictor_corrector", RunConfig(n_paths=700, seed=2)),
        ("poly", "predictor_corrector", RunConfig(n_paths=700, n_steps=1200, seed=2)),
        ("poly", "euler", RunConfig(n_paths=700, seed=2)),
    ]

    def setup(eng, market, scheme, cfg):
        eng.set_scheme(scheme)
        if market == "poly":
            eng.set_market(Market())
        elif market == "poly-scaled":
            mk = Market()
            eng.set_market_poly(51, mk.dtau, mk.spot, DEFAULT_VOL_COEFFS * 1.3)
        else:
            bump = 0.1 if market == "table" else -0.07
            eng.set_market(Market(vol=Market().vol * (1.0 + bump * np.cos(np.arange(51) / 7.0))[None, :]))
        stride = int(round(0.5 / cfg.dt))
        eng.set_swap(Swap(n_periods=cfg.n_steps // stride))

    got = []
    try:
        for market, scheme, cfg in cases:
            setup(engine, market, scheme, cfg)
            got.append(engine.run(cfg, "fp64"))
            assert engine.remainder_form() == "response"
    finally:
        engine.set_scheme("euler")
    for (market, scheme, cfg), g in zip(cases, got):
        with HJMEngine(0) as fresh:
            setup(fresh, market, scheme, cfg)
            f = fresh.run(cfg, "fp64")
        np.testing.assert_array_equal(g.ee, f.ee)
        assert g.cva == f.cva


@pytest.mark.parametrize("coef", [DEFAULT_VOL_COEFFS, FULL_COEFFS], ids=["degree<=k", "general"])
def test_response_form_on_double_normals_vs_oracle(engine, remainder_form, coef):
    """External FP64 normals that FP32 cannot hold (the response form splits
    each into hi + lo and carries both through the parts' double-FP32 terms),
    triangular and general quadratic factors: per-path exposures, EE and CVA
    against the oracle on the same draws."""
    mk = _poly_market(engine, coef=coef)
    sw = Swap()
    engine.set_swap(sw)
    remainder_form("response")
    n_paths, n_steps, dt = 300, 1000, 0.01
    normals = np.random.default_rng(31).standard_normal((n_paths, n_steps, 3))
    engine.keep_exposures(True)
    try:
        v = engine.run_with_normals(normals, n_steps, dt, "fp64")
        assert engine.remainder_form() == "response"
        x = engine.exposures()
    finally:
        engine.keep_exposures(False)
    xo = O.exposure_paths(mk, sw, n_steps, dt, normals)
    ee = O.expected_exposure(xo)
    cva, _ = O.cva(ee, 21, mk.dtau, 0.02, 0.4)
    _assert_rel(x, xo[:, :21].T, FP64_RTOL, "exposures")
    _assert_rel(v.ee[:21], ee[:21], FP64_RTOL, "EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")
