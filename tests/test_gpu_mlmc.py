"""Multi-level Monte Carlo (hjm_run_mlmc).

* the coupled level kernel against the oracle: the level-1 correction's EE and
  CVA differences equal the oracle's fine-minus-coarse exposures on the same
  normals (fine grid: the device's normals of level 1; coarse grid: their
  pairwise sums / sqrt 2, formed in FP32 as the kernel does);
* the estimator: three levels (dt 0.02, 0.01, 0.005) agree with a plain
  valuation on the finest grid within the combined standard errors, and the
  coupling makes each correction's per-path variance a small fraction of the
  level-0 variance;
* the path allocation helper and argument checks.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from cva_hjm_cuda_gb300 import _lib
from cva_hjm_cuda_gb300.engine import mlmc_allocation
from cva_hjm_cuda_gb300.market import Market, RunConfig, Swap

pytestmark = pytest.mark.gpu


def _coarse_normals(fine: np.ndarray) -> np.ndarray:
    f = fine.astype(np.float32)
    s = (f[:, 0::2, :] + f[:, 1::2, :]).astype(np.float32)
    return (s * np.float32(0.70710678118654752)).astype(np.float32).astype(np.float64)


def test_level_correction_vs_oracle(engine):
    mk, sw = Market(), Swap()
    engine.set_market(mk)
    engine.set_swap(sw)
    n0, n1, steps0, dt0 = 4096, 3000, 500, 0.02
    base = engine.run_mlmc([n0], n_steps=steps0, dt=dt0, seed=21)
    two = engine.run_mlmc([n0, n1], n_steps=steps0, dt=dt0, seed=21)
    diff = two["ee"] - base["ee"]
    fine = engine.dump_normals(n1, 2 * steps0, seed=21, path_offset=1 << 40)
    coarse = _coarse_normals(fine)
    xf = O.exposure_paths(mk, sw, 2 * steps0, dt0 / 2, fine)
    xc = O.exposure_paths(mk, sw, steps0, dt0, coarse)
    ee_d = O.expected_exposure(xf - xc)
    scale = np.max(np.abs(base["ee"]))
    assert np.max(np.abs(diff[:21] - ee_d[:21])) < 1e-6 * scale
    cva_f = O.cva_paths(xf, 21, mk.dtau, 0.02, 0.4)
    cva_c = O.cva_paths(xc, 21, mk.dtau, 0.02, 0.4)
    d = cva_f - cva_c
    lev1 = two["levels"][1]
    assert lev1["n_paths"] == n1
    assert abs(lev1["cva_diff"] - d.mean()) < 1e-6 * base["cva"]
    assert lev1["stderr"] == pytest.approx(d.std(ddof=1) / np.sqrt(n1), rel=1e-3)
    assert two["levels"][0]["cva_diff"] == base["cva"]


def test_estimator_matches_finest_grid_and_reduces_variance(engine):
    mk, sw = Market(), Swap()
    engine.set_market(mk)
    engine.set_swap(sw)
    m = engine.run_mlmc([400_000, 100_000, 50_000], n_steps=500, dt=0.02, seed=5)
    plain = engine.run(RunConfig(n_paths=400_000, n_steps=2000, dt=0.005, seed=77), "mixed", pfe=False)
    tol = 4.0 * np.hypot(m["cva_stderr"], plain.cva_stderr)
    assert abs(m["cva"] - plain.cva) < tol, (m["cva"], plain.cva, tol)
    v = [lv["stderr"] ** 2 * lv["n_paths"] for lv in m["levels"]]
    assert v[1] < 0.05 * v[0] and v[2] < 0.05 * v[0], v
    assert all(lv["ms"] > 0 for lv in m["levels"])


def test_allocation_and_errors(engine):
    n = mlmc_allocation([1.0, 0.01, 0.0025], [1.0, 3.0, 6.0], 0.01, min_paths=1)
    assert n[0] > n[1] > n[2] >= 1
    assert np.all(mlmc_allocation([1.0, 1e-9], [1.0, 3.0], 0.01) >= 1024)
    # cost-weighted optimum: the estimator variance meets the target
    assert np.sum(np.array([1.0, 0.01, 0.0025]) / n) <= 0.01**2 * 1.0001
    engine.set_market(Market())
    engine.set_swap(Swap())
    with pytest.raises(_lib.HJMError):
        engine.run_mlmc([], n_steps=500, dt=0.02)
    with pytest.raises(_lib.HJMError):
        engine.run_mlmc([100, 0], n_steps=500, dt=0.02)
    with pytest.raises(_lib.HJMError):  # dt / 2^l must keep an integer number of steps per block
        engine.run_mlmc([100, 100], n_steps=40, dt=0.25 * 1.5)


def test_mlmc_report(engine, tmp_path):
    import json

    engine.set_market(Market())
    engine.set_swap(Swap())
    m = engine.run_mlmc([8192, 2048], n_steps=500, dt=0.02, seed=3)
    engine.write_report(tmp_path / "m.json")
    r = json.loads((tmp_path / "m.json").read_text())
    assert r["kind"] == "mlmc" and len(r["levels"]) == 2
    assert r["cva"] == m["cva"] and r["run"]["n_steps"] == 1000 and r["run"]["n_paths"] == 8192 + 2048
    np.testing.assert_array_equal(r["ee"], m["ee"])


@pytest.fixture
def pc_engine(engine):
    engine.set_scheme("predictor_corrector")
    try:
        yield engine
    finally:
        engine.set_scheme("euler")


def test_pc_level_correction_vs_oracle(pc_engine):
    """The predictor-corrector's coupled level kernel against the oracle's
    predictor-corrector on the same fine normals and their coarse sums."""
    eng = pc_engine
    mk, sw = Market(), Swap()
    eng.set_market(mk)
    eng.set_swap(sw)
    n0, n1, steps0, dt0 = 4096, 3000, 500, 0.02
    base = eng.run_mlmc([n0], n_steps=steps0, dt=dt0, seed=21)
    two = eng.run_mlmc([n0, n1], n_steps=steps0, dt=dt0, seed=21)
    diff = two["ee"] - base["ee"]
    fine = eng.dump_normals(n1, 2 * steps0, seed=21, path_offset=1 << 40)
    coarse = _coarse_normals(fine)
    xf = O.exposure_paths_pc(mk, sw, 2 * steps0, dt0 / 2, fine)
    xc = O.exposure_paths_pc(mk, sw, steps0, dt0, coarse)
    ee_d = O.expected_exposure(xf - xc)
    scale = np.max(np.abs(base["ee"]))
    assert np.max(np.abs(diff[:21] - ee_d[:21])) < 1e-6 * scale
    d = O.cva_paths(xf, 21, mk.dtau, 0.02, 0.4) - O.cva_paths(xc, 21, mk.dtau, 0.02, 0.4)
    lev1 = two["levels"][1]
    assert abs(lev1["cva_diff"] - d.mean()) < 1e-6 * base["cva"]
    assert lev1["stderr"] == pytest.approx(d.std(ddof=1) / np.sqrt(n1), rel=1e-3)
    # level 0 is the predictor-corrector valuation itself
    plain = eng.run(RunConfig(n_paths=n0, n_steps=steps0, dt=dt0, seed=21), "mixed", pfe=False)
    assert two["levels"][0]["cva_diff"] == plain.cva


def test_pc_estimator_matches_finest_grid(pc_engine):
    eng = pc_engine
    eng.set_market(Market())
    eng.set_swap(Swap())
    m = eng.run_mlmc([400_000, 100_000, 50_000], n_steps=500, dt=0.02, seed=5)
    plain = eng.run(RunConfig(n_paths=400_000, n_steps=2000, dt=0.005, seed=77), "mixed", pfe=False)
    tol = 4.0 * np.hypot(m["cva_stderr"], plain.cva_stderr)
    assert abs(m["cva"] - plain.cva) < tol, (m["cva"], plain.cva, tol)
    v = [lv["stderr"] ** 2 * lv["n_paths"] for lv in m["levels"]]
    assert v[1] < 0.05 * v[0] and v[2] < 0.05 * v[0], v
