"""GPU parity of the netting-set valuation (config 5 shape: 64 payer/receiver
swaps, maturities 1-30y, 61-tenor curve, 3,000 steps), netted before max(., 0),
against the oracle's netting form (cash flow D_i (payA_i L_i - payB_i), which
reduces to the reference's single-swap cash flow for one swap)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from cva_hjm_cuda_gb300.market import Market, NettingSet, RunConfig, Swap, random_netting_set

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 1e-4


def _rel_ok(a, b, rtol):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.max(np.abs(b))
    return np.all(np.abs(a - b) <= rtol * np.maximum(np.abs(b), 1e-3 * scale))


def test_single_swap_netting_set_equals_swap(engine):
    mk = Market()
    engine.set_market(mk)
    engine.set_swap(Swap())
    a = engine.run(RunConfig(n_paths=10000), "fp64")
    engine.set_netting_set(NettingSet(np.array([1e6]), np.array([0.025]), np.array([20], np.int32),
                                      np.array([1], np.int32)))
    b = engine.run(RunConfig(n_paths=10000), "fp64")
    np.testing.assert_allclose(b.ee, a.ee, rtol=1e-14, atol=0)
    assert b.cva == pytest.approx(a.cva, rel=1e-14)


@pytest.fixture(scope="module")
def netting_case(engine):
    mk = Market(n_tenor=61)
    ns = random_netting_set(64, seed=20261203)
    cfg = RunConfig(n_paths=3000, n_steps=3000, dt=0.01, seed=31)
    engine.set_market(mk)
    engine.set_netting_set(ns)
    normals = engine.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed)
    pa, pb = ns.payoff_vectors(61, 0.5)
    x = O.exposure_paths_netting(mk, pa, pb, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, _ = O.cva(ee, 61, 0.5, cfg.hazard, cfg.recovery)
    return mk, ns, cfg, x, ee, cva


def test_netting_fp64_vs_oracle(engine, netting_case):
    mk, ns, cfg, x, ee, cva = netting_case
    engine.set_market(mk)
    engine.set_netting_set(ns)
    v = engine.run(cfg, "fp64")
    assert _rel_ok(v.ee, ee, FP64_RTOL)
    assert v.cva == pytest.approx(cva, rel=FP64_RTOL)
    np.testing.assert_allclose(v.pfe[:61], O.pfe(x, 61, 0.975), rtol=FP64_RTOL,
                               atol=FP64_RTOL * np.max(np.abs(x)))


def test_netting_mixed_vs_oracle(engine, netting_case):
    mk, ns, cfg, x, ee, cva = netting_case
    engine.set_market(mk)
    engine.set_netting_set(ns)
    v = engine.run(cfg, "mixed")
    assert _rel_ok(v.ee, ee, MIXED_RTOL), np.max(np.abs(v.ee - ee) / np.maximum(ee, 1e-3 * ee.max()))
    assert abs(v.cva - cva) <= MIXED_RTOL * cva
    assert abs(v.cva - cva) < v.cva_stderr


def test_netting_adjoint_vs_fp64_finite_differences(engine):
    mk = Market(n_tenor=61)
    ns = random_netting_set(64, seed=20261203)
    cfg = RunConfig(n_paths=20000, n_steps=3000, dt=0.01, seed=8)
    coef = mk.vol_coeffs
    engine.set_market_poly(61, 0.5, mk.spot, coef)
    engine.set_netting_set(ns)
    sens = engine.run_adjoint(cfg, checkpoint_every=32)
    v = engine.run(cfg, "mixed", pfe=False)
    # with 60 dates the valuation keeps the remainder's discount sums in FP32
    # beside FP64 sums of the scalar parts (its compact shared memory), the
    # adjoint's forward pass FP64 sums per tenor: the CVAs agree to rounding
    assert abs(sens.cva - v.cva) <= 1e-9 * abs(v.cva)
    gmax = np.max(np.abs(sens.dcva_dspot))
    for t in (2, 10, 30, 45, 60):
        h = 1e-5
        up, dn = mk.spot.copy(), mk.spot.copy()
        up[t] += h
        dn[t] -= h
        vals = []
        for sp in (up, dn):
            engine.set_market_poly(61, 0.5, sp, coef)
            engine.set_netting_set(ns)
            vals.append(engine.run(cfg, "fp64", pfe=False).cva)
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(sens.dcva_dspot[t] - fd) <= 2e-3 * max(abs(fd), 0.01 * gmax), (t, sens.dcva_dspot[t], fd)
