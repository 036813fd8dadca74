"""Differentiable shaded visibility DFT.

``VisDFT.apply(bright, ...)`` evaluates V = A(bright) with ``viss_vis_dft``; its
backward is the adjoint pass ``viss_recon`` (norm 1, unit weights, the same
occlusion mask):  d L / d bright = Re(A^H g),  g = dL/dRe V + i dL/dIm V
(torch's convention for complex outputs).  The map is linear in the brightness
only when the occluded value is 0 (a multiplicative mask); otherwise the
occluded terms are a constant offset and still drop out of the gradient.

``fit_sky_and_gains`` fits a non-negative sky and one complex gain per
baseline, V_k = g_{b(k)} A(x)_k, to observed visibilities by projected
gradient descent (Adam) through this function.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import torch

from .api import DftConfig, recon, vis_dft


class VisDFT(torch.autograd.Function):
    @staticmethod
    def forward(ctx, bright, cfg: DftConfig, u, v, w, l, m, n, snap, pair, sat_pos, shade):
        V = vis_dft(cfg, u, v, w, l, m, n, bright.contiguous(), shade=shade, snap=snap, pair=pair, sat_pos=sat_pos)
        ctx.cfg = cfg
        ctx.save_for_backward(u, v, w, l, m, n)
        ctx.geo = (snap, pair, sat_pos, shade)
        return V

    @staticmethod
    def backward(ctx, gV):
        u, v, w, l, m, n = ctx.saved_tensors
        snap, pair, sat_pos, shade = ctx.geo
        cfg = ctx.cfg
        # adjoint: same phase convention and mask, no weights, no 1/K
        rm = {0: 0, 1: 0, 2: 0, 3: 2}[cfg.mask]  # geometric mask -> geometric recon mask
        acfg = cfg.with_(recon_mask=rm, norm=1.0)
        if cfg.mask in (1, 2):
            raise NotImplementedError("the adjoint of the REF window masks is not provided")
        g = gV.contiguous().to(torch.complex64)
        AHg = recon(acfg, u, v, w, g, l, m, n, snap=snap, pair=pair, sat_pos=sat_pos)
        return (AHg.real, None, None, None, None, None, None, None, None, None, None, None)


def vis_dft_autograd(bright, cfg: DftConfig, u, v, w, l, m, n, snap=None, pair=None, sat_pos=None, shade=None):
    return VisDFT.apply(bright, cfg, u, v, w, l, m, n, snap, pair, sat_pos, shade)


@dataclass
class FitResult:
    sky: torch.Tensor
    gains: torch.Tensor
    losses: list


def fit_sky_and_gains(V_obs: torch.Tensor, cfg: DftConfig, u, v, w, l, m, n, snap, pair, sat_pos, baseline: torch.Tensor,
                      nbaselines: int, steps: int = 100, lr_sky: float = 0.05, lr_gain: float = 0.01,
                      sky0: Optional[torch.Tensor] = None, fit_gains: bool = True) -> FitResult:
    """min_{x >= 0, g} sum_k |g_{b(k)} A(x)_k - V_obs_k|^2 / sum_k |V_obs_k|^2."""
    J = l.numel()
    x = (sky0.clone() if sky0 is not None else torch.zeros(J, device=l.device)).float().requires_grad_(True)
    gr = torch.ones(nbaselines, device=l.device, requires_grad=fit_gains)
    gi = torch.zeros(nbaselines, device=l.device, requires_grad=fit_gains)
    params = [{"params": [x], "lr": lr_sky}]
    if fit_gains:
        params.append({"params": [gr, gi], "lr": lr_gain})
    opt = torch.optim.Adam(params)
    norm = (V_obs.abs() ** 2).sum()
    losses = []
    b = baseline.long()
    for _ in range(steps):
        opt.zero_grad()
        A = vis_dft_autograd(x, cfg, u, v, w, l, m, n, snap, pair, sat_pos)
        g = torch.complex(gr, gi)[b]
        loss = ((g * A - V_obs).abs() ** 2).sum() / norm
        loss.backward()
        opt.step()
        with torch.no_grad():
            x.clamp_(min=0.0)
        losses.append(float(loss.item()))
    return FitResult(sky=x.detach(), gains=torch.complex(gr, gi).detach(), losses=losses)
