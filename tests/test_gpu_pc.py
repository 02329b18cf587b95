"""GPU parity of the predictor-corrector time scheme (hjm_ctx_set_scheme)
against the oracle's restatement of the same scheme on the device's normals,
on the decomposed step (quadratic factors) and on the generic table step.

FP64 EE, PFE, CVA and per-path exposures within 1e-10 relative; mixed
precision within 1e-4 and inside the Monte Carlo error; the scheme differs
from Euler by its O(dt^2) convection term (~1e-4 of EE at dt = 0.01).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from cva_hjm_cuda_gb300 import _lib
from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS, Market, RunConfig, Swap

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 1e-4


def _assert_rel(actual, desired, rtol, what, floor=None):
    actual, desired = np.asarray(actual), np.asarray(desired)
    scale = np.max(np.abs(desired)) if desired.size else 0.0
    err = np.abs(actual - desired)
    bad = (err > rtol * np.maximum(np.abs(desired), 1e-300)) & (err > (rtol * 1e-3 if floor is None else floor) * scale)
    assert not np.any(bad), f"{what}: max rel err {np.max(err / np.maximum(np.abs(desired), 1e-300)):.3e}"


@pytest.fixture
def pc(engine):
    engine.set_scheme("predictor_corrector")
    try:
        yield engine
    finally:
        engine.set_scheme("euler")


@pytest.fixture(scope="module")
def case(engine):
    mk, sw = Market(), Swap()
    engine.set_market(mk)
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=4000, n_steps=1000, dt=0.01, seed=99)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x = O.exposure_paths_pc(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, _ = O.cva(ee, 21, mk.dtau, cfg.hazard, cfg.recovery)
    return mk, sw, cfg, normals, x, ee, cva


def test_pc_fp64_vs_oracle(pc, case):
    mk, sw, cfg, normals, x, ee, cva = case
    pc.set_market(mk)
    pc.set_swap(sw)
    pc.keep_exposures(True)
    v = pc.run(cfg, "fp64")
    xs = pc.exposures()
    pc.keep_exposures(False)
    _assert_rel(xs, x[:, :21].T, FP64_RTOL, "exposures")
    _assert_rel(v.ee, ee, FP64_RTOL, "EE")
    _assert_rel(v.cva, cva, FP64_RTOL, "CVA")
    _assert_rel(v.pfe[:21], O.pfe(x, 21, cfg.pfe_quantile), FP64_RTOL, "PFE")


def test_pc_mixed_vs_oracle(pc, case):
    mk, sw, cfg, normals, x, ee, cva = case
    pc.set_market(mk)
    pc.set_swap(sw)
    v = pc.run(cfg, "mixed")
    assert np.max(np.abs(v.ee[:20] - ee[:20]) / ee[:20]) < MIXED_RTOL
    assert abs(v.cva - cva) < MIXED_RTOL * cva
    assert abs(v.cva - cva) < v.cva_stderr


def test_pc_differs_from_euler_by_the_convection_order(engine, case):
    mk, sw, cfg, normals, x, ee_pc, cva = case
    engine.set_market(mk)
    engine.set_swap(sw)
    eu = engine.run(cfg, "fp64")
    rel = np.abs(eu.ee[:20] - ee_pc[:20]) / ee_pc[:20]
    assert 1e-7 < rel.max() < 1e-2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pc_external_normals_and_61_tenors(pc, precision):
    mk, sw = Market(n_tenor=61), Swap(n_tenor=61, n_periods=60)
    pc.set_market(mk)
    pc.set_swap(sw)
    cfg = RunConfig(n_paths=257, n_steps=3000, dt=0.01, seed=4)
    normals = pc.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    a = pc.run(cfg, precision)
    b = pc.run_with_normals(normals, cfg.n_steps, cfg.dt, precision)
    np.testing.assert_array_equal(a.ee, b.ee)
    ee = O.expected_exposure(O.exposure_paths_pc(mk, sw, cfg.n_steps, cfg.dt, normals))
    tol = FP64_RTOL if precision == "fp64" else 1e-3
    _assert_rel(a.ee[:61], ee[:61], tol, "61-tenor EE")


def test_pc_adjoint_cva_equals_pc_mixed_valuation(pc):
    """The predictor-corrector adjoint runs the convected mixed-precision
    valuation's forward pass (the shared path state), so CVA, its standard
    error and dCVA/dhazard are that valuation's bit for bit (the default
    valuation, the remainder's FP32 responses, within FP32 rounding); it keeps
    the sampled states (checkpoint_every = 0 only)."""
    mk = Market()
    pc.set_market_poly(51, 0.5, mk.spot, DEFAULT_VOL_COEFFS)
    pc.set_swap(Swap())
    cfg = RunConfig(n_paths=40000, seed=77)
    r = pc.run(cfg, "mixed", pfe=False)
    assert pc.remainder_form() == "response"
    pc.set_remainder_form("convect")
    try:
        v = pc.run(cfg, "mixed", pfe=False)
    finally:
        pc.set_remainder_form("auto")
    assert abs(r.cva - v.cva) <= 1e-6 * v.cva
    a = pc.run_adjoint(cfg, checkpoint_every=0)
    assert a.cva == v.cva
    assert a.cva_stderr == v.cva_stderr
    assert a.dcva_dhazard == v.dcva_dhazard
    with pytest.raises(_lib.HJMError) as ei:
        pc.run_adjoint(cfg, checkpoint_every=32)
    assert ei.value.status == 2
    assert pc.lib.hjm_ctx_set_scheme(pc.ctx, 7) == 1  # unknown scheme: HJM_ERR_INVALID_ARGUMENT


def test_pc_adjoint_matches_fp64_finite_differences(pc):
    """dCVA/d(initial forwards), d(volatility coefficients) and d(hazard) of the
    predictor-corrector adjoint against central differences of the FP64
    predictor-corrector valuation on the same paths, within 2e-3 (the bumps of
    the Euler adjoint's test: 1e-5 on forwards and hazard, 1e-8 25^-d on the
    coefficient of T^d)."""
    from cva_hjm_cuda_gb300.market import nelson_siegel_curve, tenor_grid

    cfg = RunConfig(n_paths=100000, seed=2024)
    spot = nelson_siegel_curve(tenor_grid(51, 0.5))
    coef = np.array(DEFAULT_VOL_COEFFS, dtype=float)

    def val(sp, cf, hz=0.02):
        pc.set_market_poly(51, 0.5, sp, cf)
        pc.set_swap(Swap())
        c = RunConfig(n_paths=cfg.n_paths, n_steps=cfg.n_steps, dt=cfg.dt, seed=cfg.seed, hazard=hz)
        return pc.run(c, "fp64", pfe=False).cva

    pc.set_market_poly(51, 0.5, spot, coef)
    pc.set_swap(Swap())
    sens = pc.run_adjoint(cfg, checkpoint_every=0)

    def close(g, fd, group_max):
        return abs(g - fd) <= 2e-3 * max(abs(fd), 0.01 * group_max)

    scale_s = np.max(np.abs(sens.dcva_dspot))
    for t in (0, 1, 5, 10, 19, 20, 30, 50):
        h = 1e-5
        up, dn = spot.copy(), spot.copy()
        up[t] += h
        dn[t] -= h
        fd = (val(up, coef) - val(dn, coef)) / (2 * h)
        assert close(sens.dcva_dspot[t], fd, scale_s), (t, sens.dcva_dspot[t], fd)
    w = np.array([25.0 ** (q % 3) for q in range(9)])
    gc = sens.dcva_dvolcoef.ravel()
    scale_c = np.max(np.abs(gc / w))
    for q in range(9):
        h = 1e-8 / w[q]
        up, dn = coef.copy(), coef.copy()
        up.flat[q] += h
        dn.flat[q] -= h
        fd = (val(spot, up) - val(spot, dn)) / (2 * h)
        assert close(gc[q] / w[q], fd / w[q], scale_c), (q, gc[q], fd)
    fd = (val(spot, coef, 0.02 + 1e-5) - val(spot, coef, 0.02 - 1e-5)) / 2e-5
    assert abs(sens.dcva_dhazard - fd) <= 1e-6 * abs(fd)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pc_generic_table_step_vs_oracle(pc, case, precision):
    """The same scheme on the generic table step (the decomposition off)."""
    mk, sw, cfg, normals, x, ee, cva = case
    pc.vol_decomposition(False)
    try:
        pc.set_market(mk)
        pc.set_swap(sw)
        v = pc.run(cfg, precision)
    finally:
        pc.vol_decomposition(True)
    tol = FP64_RTOL if precision == "fp64" else MIXED_RTOL
    _assert_rel(v.ee[:20], ee[:20], tol, "EE (table step)")
    _assert_rel(v.cva, cva, tol, "CVA (table step)")


def test_pc_general_quadratic_factors(pc):
    coef = np.array([[0.0060, 0.00010, -0.000004], [-0.0036, 0.00040, 0.000003], [0.0020, -0.00060, 0.00002]])
    mk = Market(vol_coeffs=coef)
    pc.set_market_poly(51, 0.5, mk.spot, coef)
    sw = Swap()
    pc.set_swap(sw)
    assert pc.vol_form() == "poly"
    cfg = RunConfig(n_paths=3000, seed=12)
    normals = pc.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    ee = O.expected_exposure(O.exposure_paths_pc(mk, sw, cfg.n_steps, cfg.dt, normals))
    _assert_rel(pc.run(cfg, "fp64").ee[:20], ee[:20], FP64_RTOL, "EE (general quadratic)")


@pytest.mark.parametrize("general", [False, True], ids=["tri", "general-quadratic"])
def test_pc_response_form_vs_convected_and_oracle(pc, case, general):
    """The predictor-corrector's response form (parts and remainder as
    double-FP32 sums; the default for the 10y swap) against its all-FP64
    convected form on the same paths (1e-11 relative, 1e-13 of the scale) and
    against the oracle (1e-10); the external-normals path takes the same
    form."""
    mk, sw, cfg, normals, x, ee, cva = case
    if general:
        coef = np.array([[0.0060, 0.00010, -0.000004], [-0.0036, 0.00040, 0.000003], [0.0020, -0.00060, 0.00002]])
        mk = Market(vol_coeffs=coef)
        pc.set_market_poly(51, 0.5, mk.spot, coef)
        x = O.exposure_paths_pc(mk, sw, cfg.n_steps, cfg.dt, normals)
        ee = O.expected_exposure(x)
        cva, _ = O.cva(ee, 21, mk.dtau, cfg.hazard, cfg.recovery)
    else:
        pc.set_market(mk)
    pc.set_swap(sw)
    out = {}
    pc.keep_exposures(True)
    try:
        for form in ("convect", "response"):
            pc.set_remainder_form(form)
            out[form] = (pc.run(cfg, "fp64"), pc.exposures())
            assert pc.remainder_form() == form
        pc.set_remainder_form("auto")
        ext = pc.run_with_normals(normals, cfg.n_steps, cfg.dt, "fp64")
        assert pc.remainder_form() == "response"
    finally:
        pc.keep_exposures(False)
        pc.set_remainder_form("auto")
    (vc, xc), (vr, xr) = out["convect"], out["response"]
    # per path the response form's double-FP32 parts (2^-48 of the
    # accumulator per addition within a block) leave ~5e-14 of the largest
    # exposure; both forms meet the oracle's FP64 tolerance
    _assert_rel(xr, xc, 1e-11, "exposures response vs convect", floor=1e-13)
    _assert_rel(vr.ee, vc.ee, 1e-11, "EE response vs convect")
    _assert_rel(xr, x[:, :21].T, FP64_RTOL, "exposures vs oracle")
    _assert_rel(vr.ee, ee, FP64_RTOL, "EE vs oracle")
    _assert_rel(vr.cva, cva, FP64_RTOL, "CVA vs oracle")
    np.testing.assert_array_equal(ext.ee, vr.ee)


@pytest.mark.parametrize("nt,n_paths,n_steps,dt", [(51, 1, 1000, 0.01), (51, 257, 1200, 0.01), (51, 63, 500, 0.02),
                                                   (51, 65, 1000, 0.004), (61, 257, 1000, 0.01),
                                                   (51, 129, 2500, 0.01), (61, 65, 3000, 0.01)],
                         ids=["1-path", "24-dates", "stride25", "stride125-coefficients-via-L1", "61-tenors",
                              "50-dates-in-windows", "61-tenors-60-dates-in-windows"])
def test_pc_response_form_shapes_vs_oracle(pc, nt, n_paths, n_steps, dt):
    mk = Market(n_tenor=nt)
    pc.set_market(mk)
    stride = int(round(mk.dtau / dt))
    sw = Swap(n_tenor=nt, n_periods=n_steps // stride)
    pc.set_swap(sw)
    pc.set_remainder_form("response")
    try:
        cfg = RunConfig(n_paths=n_paths, n_steps=n_steps, dt=dt, seed=6)
        v = pc.run(cfg, "fp64")
        assert pc.remainder_form() == "response"
    finally:
        pc.set_remainder_form("auto")
    normals = pc.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    ee = O.expected_exposure(O.exposure_paths_pc(mk, sw, cfg.n_steps, cfg.dt, normals))
    nd = n_steps // stride
    _assert_rel(v.ee[:nd + 1], ee[:nd + 1], FP64_RTOL, "EE")


@pytest.mark.parametrize("nt,n_steps", [(51, 2500), (61, 3000)], ids=["25y-51-tenors", "30y-61-tenors"])
def test_pc_response_windows_vs_convected_and_oracle(pc, nt, n_steps):
    """More than 24 dates: the predictor-corrector's response form prices
    them in windows (hjm_eresp.cu); per-path exposures against its all-FP64
    convected form on the same paths (1e-11 relative) and against the oracle
    (1e-10).  Exposures near zero are compared absolutely, below 5e-13 of the
    scale: over 50 or 60 dates the two FP64 forms and the oracle order their
    operations differently by ~1e-13 of the scale (the Euler tests' floor for
    runs of more than 24 dates).  The last date samples the last tenor, where
    the step's curvature noise enters after the step (a lag -1 term)."""
    mk = Market(n_tenor=nt)
    pc.set_market(mk)
    sw = Swap(n_tenor=nt, n_periods=n_steps // 50)
    pc.set_swap(sw)
    cfg = RunConfig(n_paths=193, n_steps=n_steps, dt=0.01, seed=17)
    out = {}
    pc.keep_exposures(True)
    try:
        for form in ("convect", "response"):
            pc.set_remainder_form(form)
            out[form] = (pc.run(cfg, "fp64"), pc.exposures())
            assert pc.remainder_form() == form
        pc.set_remainder_form("auto")
        pc.run(cfg, "fp64")
        assert pc.remainder_form() == "response"
    finally:
        pc.keep_exposures(False)
        pc.set_remainder_form("auto")
    (vc, xc), (vr, xr) = out["convect"], out["response"]
    nd = n_steps // 50 + 1
    _assert_rel(xr[:nd], xc[:nd], 1e-11, "exposures response vs convect", floor=5e-13)
    normals = pc.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    x = O.exposure_paths_pc(mk, sw, cfg.n_steps, cfg.dt, normals)
    _assert_rel(xr[:nd], x[:, :nd].T, FP64_RTOL, "exposures vs oracle", floor=5e-13)
    _assert_rel(vr.ee[:nd], O.expected_exposure(x)[:nd], FP64_RTOL, "EE vs oracle")
