"""Losses of optim/losses.py on this package's ops: values from the
reference's docstring examples and the defining formulas; gradients through
the CUDA VJPs."""
import pytest
import torch

from lbm_jax_autodiff_gb300 import losses
from oracle import ops as oops
from oracle.lattice import Consts


def test_porosity_penalties_cpu():
    """total_variation_penalty / volume_penalty (plain reductions, no GPU)."""
    p = torch.zeros((8, 8, 8), dtype=torch.float32)
    assert float(losses.total_variation_penalty(p)) == 0.0
    # reference example: zeros, target 0.1 -> 0.010000000707805157 in float32
    assert float(losses.volume_penalty(p)) == pytest.approx(0.010000000707805157, abs=0)
    g = torch.Generator().manual_seed(0)
    q = torch.rand((6, 5, 4), generator=g, dtype=torch.float64)
    tv = (q[1:] - q[:-1]).abs().sum() + (q[:, 1:] - q[:, :-1]).abs().sum() + \
        (q[:, :, 1:] - q[:, :, :-1]).abs().sum()
    assert float(losses.total_variation_penalty(q)) == pytest.approx(float(tv), rel=1e-15)


@pytest.mark.gpu
def test_drag_losses(cuda):
    force = torch.tensor([0.01, 0.0, 0.0], dtype=torch.float64, device="cuda")
    # reference example: Cd = 0.01 / (0.5 * 0.05^2 * 100) = 0.08
    assert float(losses.minimize_cd_loss(force, 0.05, 100.0)) == pytest.approx(0.08, rel=1e-9)
    assert float(losses.target_cd_loss(force, 0.05, 100.0, 1.0)) == pytest.approx(
        (0.08 - 1.0) ** 2, rel=1e-9)
    f = force.clone().requires_grad_(True)
    losses.target_cd_loss(f, 0.05, 100.0, 1.0).backward()
    # d/dFx (Cd - 1)^2 = 2 (Cd - 1) / (0.5 U^2 A + 1e-10)
    expect = 2 * (0.08 - 1.0) / (0.5 * 0.05 ** 2 * 100.0 + 1e-10)
    assert float(f.grad[0]) == pytest.approx(expect, rel=1e-9)


@pytest.mark.gpu
def test_target_velocity_loss(cuda):
    """Against the oracle's density/velocity on a seeded perturbed state."""
    nx, ny, nz = 8, 6, 4
    g = torch.Generator().manual_seed(1)
    K = Consts(torch.float64)
    w = torch.as_tensor(K.w, dtype=torch.float64).view(19, 1, 1, 1)
    f = w * (1.0 + 0.01 * torch.randn((19, nx, ny, nz), generator=g, dtype=torch.float64))
    target = 0.01 * torch.randn((3, nx, ny, nz), generator=g, dtype=torch.float64)
    mask = torch.rand((nx, ny, nz), generator=g) > 0.5
    rho = oops.compute_density(f)
    u = oops.compute_velocity(f, rho)
    d = ((u - target) ** 2).sum(0)
    expect_all = d.sum() / d.numel()
    expect_mask = torch.where(mask, d, torch.zeros_like(d)).sum() / (mask.double().sum() + 1e-10)
    fc, tc, mc = f.cuda(), target.cuda(), mask.cuda()
    assert float(losses.target_velocity_loss(fc, tc)) == pytest.approx(float(expect_all), rel=1e-12)
    assert float(losses.target_velocity_loss(fc, tc, mc)) == pytest.approx(float(expect_mask),
                                                                           rel=1e-12)
    fg = fc.clone().requires_grad_(True)
    losses.target_velocity_loss(fg, tc, mc).backward()
    fo = f.clone().requires_grad_(True)
    ro = oops.compute_density(fo)
    uo = oops.compute_velocity(fo, ro)
    do = ((uo - target) ** 2).sum(0)
    (torch.where(mask, do, torch.zeros_like(do)).sum() / (mask.double().sum() + 1e-10)).backward()
    assert torch.allclose(fg.grad.cpu(), fo.grad, rtol=1e-10, atol=1e-14)
