"""A thin torch.autograd.Function over the pathwise adjoint kernel.

Used to check the adjoint (hjm_run_adjoint) against bumped finite
differences: its forward is one mixed-precision CVA valuation on the device,
its backward hands torch the per-input sensitivities the adjoint kernel
produced in the same launch.  It is not a differentiable engine: torch never
traces through the kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import HJMEngine
from .market import RunConfig, Swap


class CVAAdjoint(torch.autograd.Function):
    """CVA(spot [n_tenor], vol_coeffs [3, 3], hazard []) -> scalar (float64)."""

    @staticmethod
    def forward(ctx, spot, vol_coeffs, hazard, engine: HJMEngine, swap: Swap, cfg: RunConfig, dtau: float,
                checkpoint_every: int):
        spot_np = spot.detach().cpu().double().numpy()
        coef_np = vol_coeffs.detach().cpu().double().numpy().reshape(3, 3)
        engine.set_market_poly(spot_np.size, dtau, spot_np, coef_np)
        engine.set_swap(swap)
        run = RunConfig(n_paths=cfg.n_paths, n_steps=cfg.n_steps, dt=cfg.dt, seed=cfg.seed,
                        hazard=float(hazard.detach().cpu()), recovery=cfg.recovery, path_offset=cfg.path_offset)
        sens = engine.run_adjoint(run, checkpoint_every=checkpoint_every)
        ctx.save_for_backward(torch.from_numpy(np.asarray(sens.dcva_dspot)).to(spot),
                              torch.from_numpy(np.asarray(sens.dcva_dvolcoef)).to(vol_coeffs),
                              torch.tensor(sens.dcva_dhazard, dtype=hazard.dtype, device=hazard.device))
        ctx.drift_grad = np.asarray(sens.dcva_ddrift)
        return torch.tensor(sens.cva, dtype=torch.float64, device=spot.device)

    @staticmethod
    def backward(ctx, grad):
        dspot, dcoef, dhaz = ctx.saved_tensors
        return grad * dspot, grad * dcoef.reshape(3, 3), grad * dhaz, None, None, None, None, None


def cva_with_adjoint(spot, vol_coeffs, hazard, engine: HJMEngine, swap: Swap, cfg: RunConfig, dtau: float = 0.5,
                     checkpoint_every: int = 32):
    return CVAAdjoint.apply(spot, vol_coeffs, hazard, engine, swap, cfg, dtau, checkpoint_every)
