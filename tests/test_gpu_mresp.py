"""GPU parity of the mixed-precision response form (hjm_mresp.cu).

With polynomial volatility factors under the Euler step, a mixed-precision
valuation carries the remainder of the decomposition as FP32 impulse-response
sums at the dates it reaches (8 slots for the 10y swap, 16 for the 12y one)
instead of convecting it over every tenor; runs whose counting dates do not
fit 16 slots (25y, 30y) convect.

* Per-path exposures within 1e-4 of the exposure scale from the oracle on the
  device's normals, and within FP32 rounding (2e-6 of the scale) of the
  convected pairs on the same paths; EE and CVA likewise.
* The quadratic market (8 and 16 slots), the reference driver's own table
  (the cubic form), ragged path counts, PFE, external normals (equal bit for
  bit to the generator's run on the same draws) and the allocation-free entry.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from conftest import load_golden, market_from_golden
from cva_hjm_cuda_gb300.market import Market, RunConfig, Swap

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-4
# the two mixed forms round the remainder differently in FP32: per-path
# exposures agree to ~1e-7 of the exposure scale, EE and CVA to ~1e-8
FORM_TOL = 2e-6


def _both_forms(engine, cfg, pfe=True):
    """(valuation, exposures [dates][paths], form) for AUTO, then for CONVECT."""
    out = []
    engine.keep_exposures(True)
    try:
        for form in ("auto", "convect"):
            engine.set_remainder_form(form)
            v = engine.run(cfg, "mixed", pfe=pfe)
            out.append((v, engine.exposures(), engine.remainder_form()))
    finally:
        engine.set_remainder_form("auto")
        engine.keep_exposures(False)
    return out


def _own_market():
    g = load_golden("ref_driver_own_market.json")
    mk, _ = market_from_golden(g)
    return mk


@pytest.mark.parametrize("case", ["quadratic-10y", "quadratic-12y", "reference-table-10y"])
def test_mixed_response_vs_convected_and_oracle(engine, case):
    mk = _own_market() if case.startswith("reference") else Market()
    n_periods = 24 if "12y" in case else 20
    sw = Swap(n_periods=n_periods)
    engine.set_market(mk)
    engine.set_swap(sw)
    n_steps = 50 * n_periods
    cfg = RunConfig(n_paths=3001, n_steps=n_steps, dt=0.01, seed=11)
    (r, xr, fr), (c, xc, fc) = _both_forms(engine, cfg)
    assert (fr, fc) == ("response", "convect")
    nd = n_periods + 1
    scale = np.max(np.abs(xc))
    assert np.max(np.abs(xr - xc)) <= FORM_TOL * scale
    np.testing.assert_allclose(r.ee[:nd], c.ee[:nd], rtol=FORM_TOL, atol=FORM_TOL * np.max(c.ee))
    assert abs(r.cva - c.cva) <= FORM_TOL * c.cva
    # PFE: the order statistic of the same exposures, each within FORM_TOL
    np.testing.assert_allclose(r.pfe[:nd], c.pfe[:nd], rtol=0, atol=FORM_TOL * scale)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    xo = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)[:, :nd].T
    assert np.max(np.abs(xr - xo)) <= MIXED_RTOL * np.max(np.abs(xo))
    ee_o = O.expected_exposure(xo.T)[:nd]
    np.testing.assert_allclose(r.ee[:nd], ee_o, rtol=MIXED_RTOL, atol=MIXED_RTOL * np.max(ee_o))


def test_mixed_response_external_normals_equal_generator(engine):
    """hjm_run_with_normals on the generator's own draws (FP32 values widened)
    gives the Philox run's results bit for bit through the response form."""
    engine.set_market(Market())
    engine.set_swap(Swap())
    cfg = RunConfig(n_paths=1000, n_steps=1000, dt=0.01, seed=3)
    v = engine.run(cfg, "mixed")
    assert engine.remainder_form() == "response"
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    w = engine.run_with_normals(normals, cfg.n_steps, cfg.dt, "mixed")
    assert engine.remainder_form() == "response"
    assert np.array_equal(v.ee, w.ee)
    assert np.array_equal(v.pfe, w.pfe)
    assert v.cva == w.cva


@pytest.mark.parametrize("n_steps", [50, 100, 150])
def test_mixed_response_shortest_runs(engine, n_steps):
    """One to three dates (one date: no evolution; the look-ahead draw stays
    within the run's steps), external normals included."""
    mk, sw = Market(), Swap(n_periods=n_steps // 50)
    engine.set_market(mk)
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=777, n_steps=n_steps, dt=0.01, seed=2)
    nd = n_steps // 50 + 1
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    xo = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)[:, :nd].T
    ee_o = O.expected_exposure(xo.T)[:nd]
    for v in (engine.run(cfg, "mixed"), engine.run_with_normals(normals, cfg.n_steps, cfg.dt, "mixed")):
        assert engine.remainder_form() == "response"
        np.testing.assert_allclose(v.ee[:nd], ee_o, rtol=MIXED_RTOL, atol=MIXED_RTOL * np.max(np.abs(ee_o)))


def test_mixed_response_long_runs_convect(engine):
    """The 25y swap's counting dates (38) do not fit 16 slots: the run convects,
    and its results match the oracle."""
    mk, sw = Market(), Swap(n_periods=50)
    engine.set_market(mk)
    engine.set_swap(sw)
    cfg = RunConfig(n_paths=500, n_steps=2500, dt=0.01, seed=8)
    v = engine.run(cfg, "mixed")
    assert engine.remainder_form() == "convect"
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    xo = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)[:, :51].T
    ee_o = O.expected_exposure(xo.T)[:51]
    np.testing.assert_allclose(v.ee[:50], ee_o[:50], rtol=MIXED_RTOL, atol=MIXED_RTOL * np.max(ee_o))


def test_mixed_response_path_ranges_compose(engine):
    """Paths are independent: a run over [0, n) equals, in EE sums, the runs
    over its two halves (path_offset), and a ragged count runs its tail CTA."""
    engine.set_market(Market())
    engine.set_swap(Swap())
    n = 2 * 12_345
    full = engine.run(RunConfig(n_paths=n, seed=9), "mixed", pfe=False)
    a = engine.run(RunConfig(n_paths=n // 2, seed=9), "mixed", pfe=False)
    b = engine.run(RunConfig(n_paths=n // 2, seed=9, path_offset=n // 2), "mixed", pfe=False)
    np.testing.assert_allclose(full.ee, 0.5 * (a.ee + b.ee), rtol=1e-12, atol=1e-12 * np.max(full.ee))


@pytest.mark.parametrize("n_periods", [20, 24])
def test_response_adjoint_vs_convected_adjoint(engine, n_periods, tmp_path):
    """The adjoint in the response form (the sampled states kept, the sweep's
    last-tenor adjoint from the table: 8 slots for 10y, 16 for 12y) against
    the convected adjoint on the same paths: every sensitivity within 1e-4 of
    its group's largest (FP32 rounding of two orderings), CVA within 1e-6."""
    import json

    from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS, nelson_siegel_curve, tenor_grid

    engine.set_market_poly(51, 0.5, nelson_siegel_curve(tenor_grid(51, 0.5)), DEFAULT_VOL_COEFFS)
    engine.set_swap(Swap(n_periods=n_periods))
    cfg = RunConfig(n_paths=30_011, n_steps=50 * n_periods, seed=21)
    a = engine.run_adjoint(cfg, checkpoint_every=0)
    engine.write_report(tmp_path / "a.json")
    assert json.loads((tmp_path / "a.json").read_text())["run"]["remainder"] == "response"
    engine.set_remainder_form("convect")
    try:
        c = engine.run_adjoint(cfg, checkpoint_every=0)
        engine.write_report(tmp_path / "c.json")
        assert json.loads((tmp_path / "c.json").read_text())["run"]["remainder"] == "convect"
    finally:
        engine.set_remainder_form("auto")
    assert abs(a.cva - c.cva) <= 1e-6 * c.cva
    assert abs(a.dcva_dhazard - c.dcva_dhazard) <= 1e-6 * abs(c.dcva_dhazard)
    for name in ("dcva_dspot", "dcva_ddrift", "dcva_dvolcoef"):
        ga, gc = np.ravel(getattr(a, name)), np.ravel(getattr(c, name))
        if name == "dcva_dvolcoef":  # in units of a volatility change at T = 25y
            w = np.array([25.0 ** (q % 3) for q in range(9)])
            ga, gc = ga / w, gc / w
        np.testing.assert_allclose(ga, gc, rtol=0, atol=1e-4 * np.max(np.abs(gc)), err_msg=name)


def test_pc_mixed_response_vs_convected_and_oracle(engine):
    """The predictor-corrector step in mixed precision: its remainder (sources
    at L - 1 and L from the old and new W) in FP32 responses of the
    three-point step, the parts by the same kernel with the N-projected
    loadings; against its convected kernel and the PC oracle."""
    mk, sw = Market(), Swap()
    engine.set_market(mk)
    engine.set_swap(sw)
    engine.set_scheme("predictor_corrector")
    try:
        cfg = RunConfig(n_paths=3001, seed=13)
        (r, xr, fr), (c, xc, fc) = _both_forms(engine, cfg)
        assert (fr, fc) == ("response", "convect")
        scale = np.max(np.abs(xc))
        assert np.max(np.abs(xr - xc)) <= FORM_TOL * scale
        np.testing.assert_allclose(r.ee[:21], c.ee[:21], rtol=FORM_TOL, atol=FORM_TOL * np.max(c.ee))
        assert abs(r.cva - c.cva) <= FORM_TOL * c.cva
        normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
        xo = O.exposure_paths_pc(mk, sw, cfg.n_steps, cfg.dt, normals)[:, :21].T
        assert np.max(np.abs(xr - xo)) <= MIXED_RTOL * np.max(np.abs(xo))
        # the 25y swap (its last date samples the last tenor) convects
        engine.set_swap(Swap(n_periods=50))
        engine.run(RunConfig(n_paths=300, n_steps=2500, seed=13), "mixed")
        assert engine.remainder_form() == "convect"
    finally:
        engine.set_scheme("euler")
