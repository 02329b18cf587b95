"""The report file (hjm_write_report): JSON and CSV of the last valuation or
adjoint run, numbers round-tripping exactly."""
from __future__ import annotations

import csv
import json

import numpy as np
import pytest

from cva_hjm_cuda_gb300 import _lib
from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS, Market, RunConfig, Swap

pytestmark = pytest.mark.gpu


def test_valuation_report_json_and_csv(engine, tmp_path):
    engine.set_market(Market())
    engine.set_swap(Swap())
    cfg = RunConfig(n_paths=20000, seed=3)
    v = engine.run(cfg, "fp64")
    engine.write_report(tmp_path / "r.json")
    r = json.loads((tmp_path / "r.json").read_text())
    assert r["kind"] == "valuation"
    assert r["run"]["n_paths"] == 20000 and r["run"]["precision"] == "fp64"
    assert r["run"]["vol_form"] == "poly_tri" and r["run"]["sampled_dates"] == 20
    assert r["cva"] == v.cva and r["cva_stderr"] == v.cva_stderr and r["dcva_dhazard"] == v.dcva_dhazard
    np.testing.assert_array_equal(r["ee"], v.ee)
    np.testing.assert_array_equal(r["pfe"], v.pfe)
    np.testing.assert_array_equal(r["dates"], 0.5 * np.arange(51))

    engine.write_report(tmp_path / "r.csv", fmt="csv")
    rows = list(csv.reader((tmp_path / "r.csv").read_text().splitlines()[1:]))
    kv = {k: val for k, val in rows[1: rows.index(["date", "t", "ee", "pfe"])]}
    assert float(kv["cva"]) == v.cva
    table = rows[rows.index(["date", "t", "ee", "pfe"]) + 1:]
    assert len(table) == 51
    np.testing.assert_array_equal([float(x[2]) for x in table], v.ee)


def test_adjoint_report(engine, tmp_path):
    mk = Market()
    engine.set_market_poly(51, 0.5, mk.spot, DEFAULT_VOL_COEFFS)
    engine.set_swap(Swap())
    s = engine.run_adjoint(RunConfig(n_paths=10000, seed=9), checkpoint_every=32)
    engine.write_report(tmp_path / "a.json")
    r = json.loads((tmp_path / "a.json").read_text())
    assert r["kind"] == "adjoint" and r["run"]["checkpoint_every"] == 32
    assert r["cva"] == s.cva
    np.testing.assert_array_equal(r["dcva_dspot"], s.dcva_dspot)
    np.testing.assert_array_equal(r["dcva_ddrift"], s.dcva_ddrift)
    np.testing.assert_array_equal(np.reshape(r["dcva_dvolcoef"], -1), np.reshape(s.dcva_dvolcoef, -1))


def test_report_errors(engine, tmp_path):
    from cva_hjm_cuda_gb300.engine import HJMEngine

    with HJMEngine(0) as fresh:
        with pytest.raises(_lib.HJMError):
            fresh.write_report(tmp_path / "none.json")  # nothing run yet
    with pytest.raises(KeyError):
        engine.write_report(tmp_path / "x", fmt="xml")
    with pytest.raises(_lib.HJMError):
        engine.write_report(tmp_path / "no_such_dir" / "r.json")
