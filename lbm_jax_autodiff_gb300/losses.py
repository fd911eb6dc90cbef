"""Optimisation losses of jax_lbm (optim/losses.py), on this package's ops.

Same names, arguments and formulas as the reference; the drag and velocity
terms go through the CUDA kernels (drag_coefficient, compute_density,
compute_velocity) and their VJPs, the porosity regularisers are torch
reductions.  The batched solver evaluates the two drag losses on the device
inside its Adam step (Batch.optimize, loss="cd" / "target").
"""

import torch

from .core.equilibrium import compute_density, compute_velocity
from .core.forces import drag_coefficient


def target_cd_loss(force, inlet_velocity, area, target_cd):
    """(Cd - target_cd)^2 (optim/losses.py:34-70)."""
    cd = drag_coefficient(force, inlet_velocity, area)
    return (cd - target_cd) ** 2


def minimize_cd_loss(force, inlet_velocity, area):
    """Cd itself (optim/losses.py:71-99)."""
    return drag_coefficient(force, inlet_velocity, area)


def target_velocity_loss(f, target_u, mask=None):
    """Mean over cells (or over mask) of |u - target_u|^2 (optim/losses.py:102-148)."""
    rho = compute_density(f)
    u = compute_velocity(f, rho)
    diff_sq = ((u - target_u) ** 2).sum(dim=0)
    if mask is not None:
        diff_sq = torch.where(mask, diff_sq, torch.zeros_like(diff_sq))
        n_cells = mask.to(diff_sq.dtype).sum() + 1e-10
    else:
        n_cells = float(diff_sq.numel())
    return diff_sq.sum() / n_cells


def total_variation_penalty(porosity):
    """Sum of |differences| of neighbouring cells along each axis (optim/losses.py:151-181)."""
    dx = (porosity[1:, :, :] - porosity[:-1, :, :]).abs()
    dy = (porosity[:, 1:, :] - porosity[:, :-1, :]).abs()
    dz = (porosity[:, :, 1:] - porosity[:, :, :-1]).abs()
    return dx.sum() + dy.sum() + dz.sum()


def volume_penalty(porosity, target_fraction=0.1):
    """(mean porosity - target_fraction)^2 (optim/losses.py:184-210)."""
    return (porosity.mean() - target_fraction) ** 2
