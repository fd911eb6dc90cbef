"""The CPU oracle pinned to the reference's own published numbers.

Golden values (reference project):
  d(sum f_eq)/d rho = 64.000001 (FP64, 4x4x4)      paper/paper.tex:501, tests/test_gradients_f64.py:48-64
  d rho_bar / d U = 0.611238 (FP64, 5 BGK steps)   paper/paper.tex:502, tests/test_gradients_f64.py:95-127
  Bouzidi dCd/dr = 93.33275 (FP64, 10 BGK steps)   paper/paper.tex:503, tests/test_gradients_f64.py:129-217
  Poiseuille 60x20x4, tau 0.8, 3000 BGK steps      README.md:57-69, paper/paper.tex:371-387
"""

import json
import os

import pytest
import torch

from oracle import drivers, geometry, ops
from oracle.ops import consts_for

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_equilibrium_grad_64():
    c = consts_for(torch.float64, ref_consts=True)
    rho = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    fe = ops.equilibrium(rho * torch.ones(4, 4, 4, dtype=torch.float64),
                         torch.zeros(3, 4, 4, 4, dtype=torch.float64), c)
    fe.sum().backward()
    # published AD value 64.000001: the float32-rounded weights sum to 1 + 1.5e-8
    assert abs(rho.grad.item() - 64.000001) < 5e-7


def test_inlet_gradient_0611238():
    dt = torch.float64
    c = consts_for(dt, True)

    def sim(ux):
        f = drivers.initial_state(8, 4, 4, 0.0, dt, c)
        q = -torch.ones((19, 8, 4, 4), dtype=dt)
        for _ in range(5):
            f = ops.zou_he_outlet(ops.zou_he_inlet(ops.stream(ops.bgk(f, 0.8, c), q, True),
                                                   (ux, 0.0, 0.0)), 1.0)
        return ops.compute_density(f[:, 2:-2]).mean()

    u = torch.tensor(0.05, dtype=dt, requires_grad=True)
    sim(u).backward()
    assert abs(u.grad.item() - 0.611238) < 5e-7
    eps = 1e-7
    with torch.no_grad():
        fd = (sim(torch.tensor(0.05 + eps, dtype=dt)) - sim(torch.tensor(0.05 - eps, dtype=dt))) / (2 * eps)
    assert abs(fd.item() - 0.611238) < 5e-6


def test_bouzidi_dcd_dr_9333275():
    r = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    cd = drivers.cd_of_radius_bgk_f64(r)
    cd.backward()
    assert abs(r.grad.item() - 93.33275) < 1e-5 * 93.33275


def test_poiseuille_published_profile():
    """60x20x4 channel, uniform inlet 0.05, tau 0.8, 3000 BGK steps (examples/01)."""
    nx, ny, nz = 60, 20, 4
    solid = drivers.channel_walls(nx, ny, nz)
    q = geometry.compute_q_from_solid(solid, 0.5)
    f = drivers.initial_state(nx, ny, nz, 0.0)
    cfg = drivers.StepConfig(tau=0.8, inlet=(0.05, 0.0, 0.0), collision="bgk")
    with torch.no_grad():
        f, _, _ = drivers.run(f, q, cfg, 3000, solid=solid)
    u = ops.compute_velocity(f, ops.compute_density(f))
    prof = u[0, nx // 2].mean(dim=-1)
    published = {1: 0.008247, 5: 0.057873, 9: 0.076879, 15: 0.048352, 19: 0.000200, 0: 0.000200}
    for y, v in published.items():
        assert abs(prof[y].item() - v) <= 6e-7, (y, prof[y].item(), v)


def test_drag_coefficient_known_value():
    """Cd(F=0.01, U=0.05, A=100) = 0.08 (tests/test_forces.py:86-91)."""
    cd = ops.drag_coefficient(torch.tensor([0.01, 0.0, 0.0]), 0.05, 100.0)
    assert abs(cd.item() - 0.08) < 5e-4


def test_projected_area_box_and_ground():
    """3x4x4 box -> 16; ground value 2 excluded (tests/test_forces.py:62-83)."""
    s = torch.zeros((16, 8, 8), dtype=torch.int32)
    s[5:8, 2:6, 2:6] = 1
    assert ops.projected_area(s) == 16.0
    g = torch.zeros((16, 8, 8), dtype=torch.int32)
    g[:, 0, :] = 2
    assert ops.projected_area(g) == 0.0


def test_golden_fixtures_consistent():
    """Committed fixtures were produced by tests/golden/make_golden.py from this oracle."""
    path = os.path.join(GOLDEN, "pins.json")
    if not os.path.exists(path):
        pytest.skip("fixtures not generated")
    with open(path) as fh:
        d = json.load(fh)
    assert abs(d["bouzidi_dcd_dr_f64"] - 93.33275) < 1e-3
    assert abs(d["inlet_grad_f64"] - 0.611238) < 1e-6
