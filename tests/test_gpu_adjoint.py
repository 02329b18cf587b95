"""GPU checks of the pathwise CVA adjoint (hjm_run_adjoint), through the C ABI
and the thin torch.autograd.Function wrapper.

* the adjoint launch values CVA exactly as the mixed-precision forward does;
* the checkpoint/recompute mode agrees with the store-the-seeds mode;
* gradients agree with central finite differences of the FP64 valuation on the
  same paths (common random numbers), within 2e-3 relative: bump 1e-5 on the
  initial forwards and the hazard rate; on the volatility coefficient of T^d
  the bump is 1e-8 * 25^-d, because a 1e-5 bump of a diffusion coefficient
  moves so many paths across the max(V, 0) kink that the finite difference
  itself changes by ~2 % between h and 10 h (the FP64 valuation leaves
  ~1e-11 relative rounding noise at the small bump);
* gradients agree with the reference's own bump-and-revalue: the oracle
  restatement of simulation_cpu.h revalued on bumped inputs with the device's
  normals, within 2e-3 relative.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS, Market, RunConfig, Swap, nelson_siegel_curve, poly_vols, tenor_grid

pytestmark = pytest.mark.gpu

FD_RTOL = 2e-3


def _poly(engine, spot=None, coef=DEFAULT_VOL_COEFFS, nt=51):
    tau = tenor_grid(nt, 0.5)
    spot = nelson_siegel_curve(tau) if spot is None else spot
    engine.set_market_poly(nt, 0.5, spot, coef)
    engine.set_swap(Swap(n_tenor=nt))
    return spot


def test_adjoint_cva_equals_mixed_forward(engine):
    """Each adjoint launch runs its valuation's forward pass unchanged: the
    convected adjoint (checkpoints, or the convected form requested) the
    convected mixed valuation's, bit for bit in CVA, standard error and
    dCVA/dhazard (checkpoint writes only read the state); the response form's
    adjoint (no checkpoints, the default) the response valuation's, whose
    per-path cash flows it reproduces (its CTAs sum them in other groups)."""
    _poly(engine)
    cfg = RunConfig(n_paths=40000, seed=77)
    engine.set_remainder_form("convect")
    try:
        v = engine.run(cfg, "mixed", pfe=False)
        a0c = engine.run_adjoint(cfg, checkpoint_every=0)
    finally:
        engine.set_remainder_form("auto")
    r = engine.run(cfg, "mixed", pfe=False)
    assert engine.remainder_form() == "response"
    assert abs(r.cva - v.cva) <= 1e-6 * v.cva
    for a in (a0c, engine.run_adjoint(cfg, checkpoint_every=32)):
        assert a.cva == v.cva
        assert a.cva_stderr == v.cva_stderr
        assert a.dcva_dhazard == v.dcva_dhazard
    a0 = engine.run_adjoint(cfg, checkpoint_every=0)
    assert abs(a0.cva - r.cva) <= 1e-12 * r.cva
    assert abs(a0.cva_stderr - r.cva_stderr) <= 1e-9 * r.cva_stderr
    assert abs(a0.dcva_dhazard - r.dcva_dhazard) <= 1e-12 * abs(r.dcva_dhazard)


def test_checkpoint_mode_matches_seed_mode(engine):
    """The convected adjoint with checkpoints against the convected adjoint
    that keeps the sampled states (the same forward pass: CVA bit for bit)."""
    _poly(engine)
    cfg = RunConfig(n_paths=20000, seed=5)
    engine.set_remainder_form("convect")
    try:
        a = engine.run_adjoint(cfg, checkpoint_every=0)
    finally:
        engine.set_remainder_form("auto")
    for k in (32, 50, 7):
        b = engine.run_adjoint(cfg, checkpoint_every=k)
        assert b.cva == a.cva
        np.testing.assert_allclose(b.dcva_dspot, a.dcva_dspot, rtol=1e-4, atol=1e-4 * np.max(np.abs(a.dcva_dspot)))
        np.testing.assert_allclose(b.dcva_ddrift, a.dcva_ddrift, rtol=1e-4, atol=1e-4 * np.max(np.abs(a.dcva_ddrift)))
        np.testing.assert_allclose(b.dcva_dvolcoef, a.dcva_dvolcoef, rtol=1e-4,
                                   atol=1e-4 * np.max(np.abs(a.dcva_dvolcoef)))


def _fd_fp64(engine, cfg, spot, coef, hazard, which, idx, h):
    def val(sp, cf, hz):
        _poly(engine, sp, cf)
        c = RunConfig(n_paths=cfg.n_paths, n_steps=cfg.n_steps, dt=cfg.dt, seed=cfg.seed, hazard=hz)
        return engine.run(c, "fp64", pfe=False).cva

    if which == "spot":
        up, dn = spot.copy(), spot.copy()
        up[idx] += h
        dn[idx] -= h
        return (val(up, coef, hazard) - val(dn, coef, hazard)) / (2 * h)
    if which == "coef":
        up, dn = coef.copy(), coef.copy()
        up.flat[idx] += h
        dn.flat[idx] -= h
        return (val(spot, up, hazard) - val(spot, dn, hazard)) / (2 * h)
    return (val(spot, coef, hazard + h) - val(spot, coef, hazard - h)) / (2 * h)


def _coef_bump(q):
    return 1e-8 / 25.0 ** (q % 3)


def _close(g, fd, group_max, rtol=FD_RTOL):
    """rtol relative to the finite difference, or to 1 % of the group's largest
    sensitivity for entries that are nearly zero."""
    return abs(g - fd) <= rtol * max(abs(fd), 0.01 * group_max)


def test_autograd_wrapper_matches_fp64_finite_differences(engine):
    torch = pytest.importorskip("torch")
    from cva_hjm_cuda_gb300.autograd import cva_with_adjoint

    cfg = RunConfig(n_paths=100000, seed=2024)
    spot = nelson_siegel_curve(tenor_grid(51, 0.5))
    coef = DEFAULT_VOL_COEFFS.copy()
    sp = torch.tensor(spot, dtype=torch.float64, requires_grad=True)
    cf = torch.tensor(coef, dtype=torch.float64, requires_grad=True)
    hz = torch.tensor(0.02, dtype=torch.float64, requires_grad=True)
    cva = cva_with_adjoint(sp, cf, hz, engine, Swap(), cfg, 0.5, 32)
    cva.backward()
    gs, gc, gh = sp.grad.numpy(), cf.grad.numpy().ravel(), float(hz.grad)
    scale_s = np.max(np.abs(gs))
    for t in (0, 1, 2, 5, 10, 15, 19, 20, 30, 49, 50):
        fd = _fd_fp64(engine, cfg, spot, coef, 0.02, "spot", t, 1e-5)
        assert _close(gs[t], fd, scale_s), (t, gs[t], fd)
    for q in range(9):
        fd = _fd_fp64(engine, cfg, spot, coef, 0.02, "coef", q, _coef_bump(q))
        # compare in units of a volatility change at T = 25y (coefficient of T^d scaled by 25^d)
        w = 25.0 ** (q % 3)
        scale_c = np.max(np.abs(gc / np.array([25.0 ** (r % 3) for r in range(9)])))
        assert _close(gc[q] / w, fd / w, scale_c), (q, gc[q], fd)
    fd = _fd_fp64(engine, cfg, spot, coef, 0.02, "hazard", 0, 1e-5)
    assert abs(gh - fd) <= 1e-6 * abs(fd)


def test_adjoint_matches_reference_bump_and_revalue(engine):
    """Bump-and-revalue with the oracle (the reference's CPU path restated) on the
    device's own normals, against the adjoint of the same paths."""
    n_paths, n_steps, dt, seed = 3000, 1000, 0.01, 99
    spot = _poly(engine)
    coef = DEFAULT_VOL_COEFFS.copy()
    sens = engine.run_adjoint(RunConfig(n_paths=n_paths, seed=seed), checkpoint_every=32)
    normals = engine.dump_normals(n_paths, n_steps, seed)
    sw = Swap()
    tau = tenor_grid(51, 0.5)

    def oracle_cva(sp, cf, hz=0.02):
        vol = poly_vols(tau, cf)
        mk = Market(n_tenor=51, dtau=0.5, spot=sp, vol=vol, drift=O.trapezoid_drift(vol, 0.5))
        x = O.exposure_paths(mk, sw, n_steps, dt, normals)
        return O.cva(O.expected_exposure(x), 21, 0.5, hz, 0.4)[0]

    base = oracle_cva(spot, coef)
    assert sens.cva == pytest.approx(base, rel=1e-4)
    scale_s = np.max(np.abs(sens.dcva_dspot))
    for t in (1, 7, 20, 40):
        h = 1e-5
        up, dn = spot.copy(), spot.copy()
        up[t] += h
        dn[t] -= h
        fd = (oracle_cva(up, coef) - oracle_cva(dn, coef)) / (2 * h)
        assert _close(sens.dcva_dspot[t], fd, scale_s), (t, sens.dcva_dspot[t], fd)
    for q in (0, 4, 8):
        h = _coef_bump(q)
        up, dn = coef.copy(), coef.copy()
        up.flat[q] += h
        dn.flat[q] -= h
        fd = (oracle_cva(spot, up) - oracle_cva(spot, dn)) / (2 * h)
        g = sens.dcva_dvolcoef.flat[q]
        assert _close(g, fd, abs(fd)), (q, g, fd)


def test_adjoint_rejects_bad_checkpoint_interval(engine):
    from cva_hjm_cuda_gb300 import _lib

    _poly(engine)
    with pytest.raises(_lib.HJMError) as ei:
        engine.run_adjoint(RunConfig(n_paths=1000), checkpoint_every=51)
    assert ei.value.status == 2
