"""In-place ("AA") streaming of lbm_run against the two-buffer scheme: the
same states, samples and guard counts, to the bit, across chunked runs with
both layouts, for the boundary rules that read beyond the plain pull
(Bouzidi links, x-face fallbacks, Zou-He, momentum-exchange samples)."""

import pytest
import torch

import lbm_jax_autodiff_gb300 as L
from oracle import drivers

pytestmark = pytest.mark.gpu


def _pair(nx, ny, nz, tau, storage="fp32", geometry=None, **kw):
    sims = []
    for mode in ("ab", "aa"):
        s = L.Simulation(nx, ny, nz, tau, storage=storage, **kw)
        s.set_streaming(mode)
        geometry(s)
        sims.append(s)
    return sims


CASES = [
    # storage, collision, smagorinsky, guard, sphere
    ("fp32", "mrt", True, "pre", dict(kind="dist", q_mode="bouzidi", porosity="hard")),
    ("fp32", "bgk", False, "post", dict(kind="sigmoid", q_mode="bouzidi", porosity="soft",
                                        sharpness=10.0)),
    ("fp64", "mrt", False, "off", dict(kind="sigmoid", q_mode="halfway", porosity="hard")),
]


@pytest.mark.parametrize("storage,collision,smag,guard,sph", CASES)
def test_aa_matches_ab(cuda, storage, collision, smag, guard, sph):
    ab, aa = _pair(48, 24, 24, 0.56, storage=storage, collision=collision,
                   use_smagorinsky=smag, guard=guard,
                   geometry=lambda s: s.set_sphere(0.6, center=(-1.0, 0.1, 0.0), **sph))
    f0 = ab.equilibrium_state()
    for s in (ab, aa):
        s.set_state(f0)
    for chunk in (7, 1, 12, 5):          # odd and even chunks: both layouts at the ends
        s_ab = ab.run(chunk, sample_every=chunk)
        s_aa = aa.run(chunk, sample_every=chunk)
        assert torch.equal(s_ab, s_aa)
        assert torch.equal(ab.get_state(), aa.get_state())
    assert ab.guard_resets == aa.guard_resets
    for s in (ab, aa):
        s.run(3)
    out = torch.empty_like(f0).cpu().pin_memory()
    aa.get_state_host(out)
    torch.cuda.synchronize()
    assert torch.equal(out, ab.get_state().cpu())
    ab.close()
    aa.close()


def test_aa_channel_with_inlet_profile(cuda):
    """The 64x21x8 channel (solid walls, parabolic inlet, BGK)."""
    nx, ny, nz = 64, 21, 8
    prof = drivers.parabolic_inlet(ny, nz, 0.05)
    face = torch.stack([prof, torch.zeros_like(prof), torch.zeros_like(prof)]).contiguous().cuda()

    def geom(s):
        s.set_mask(drivers.channel_walls(nx, ny, nz).cuda())
        s.set_inlet_profile(face)

    ab, aa = _pair(nx, ny, nz, 0.8, collision="bgk", geometry=geom)
    f0 = drivers.initial_state(nx, ny, nz, 0.0).cuda()
    for s in (ab, aa):
        s.set_state(f0)
        s.run(301)
    assert torch.equal(ab.get_state(), aa.get_state())
    ab.close()
    aa.close()


def test_aa_gradient_and_mode_rules(cuda):
    """A gradient evaluation on an AA handle (it takes the second buffer back
    for its own passes) equals the two-buffer handle's; switching schemes or
    the geometry under a running state asks for the state again; the
    unsupported combinations are refused."""
    from lbm_jax_autodiff_gb300._native import LBMError
    sph = dict(kind="sigmoid", q_mode="bouzidi", porosity="soft")
    ab, aa = _pair(32, 16, 16, 0.56, collision="mrt",
                   geometry=lambda s: s.set_sphere(0.5, **sph))
    f0 = ab.equilibrium_state()
    for s in (ab, aa):
        s.set_state(f0)
    assert ab.cd_and_grad(30, checkpoint_every=7) == aa.cd_and_grad(30, checkpoint_every=7)
    aa.run(4)
    assert torch.equal(aa.get_state(), (ab.run(4), ab.get_state())[1])
    aa.set_sphere(0.55, **sph)
    with pytest.raises(LBMError, match="STATE"):
        aa.run(1)
    aa.set_state(f0)
    aa.run(2)
    aa.set_streaming("ab")
    with pytest.raises(LBMError, match="STATE"):
        aa.run(1)
    aa.set_state(f0)
    aa.run(1)
    nonper = L.Simulation(16, 8, 8, 0.6, periodic_yz=False)
    with pytest.raises(LBMError, match="UNSUPPORTED"):
        nonper.set_streaming("aa")
    half = L.Simulation(16, 8, 8, 0.6, storage="fp16")
    with pytest.raises(LBMError, match="UNSUPPORTED"):
        half.set_streaming("aa")
    for s in (ab, aa, nonper, half):
        s.close()


@pytest.mark.parametrize("grid", [(3, 1, 2), (5, 3, 1), (4, 2, 6), (3, 4, 1)])
def test_aa_tiny_grids_match_ab_and_the_oracle(cuda, grid):
    """Grids where the y / z wraps land on the cell itself or its only
    neighbour, and (nx = 3) one interior plane between the x faces: AA equals
    A/B to the bit, and both follow the FP32 oracle."""
    nx, ny, nz = grid
    solid = torch.zeros((nx, ny, nz), dtype=torch.int32)
    q = -torch.ones((19, nx, ny, nz))

    def geom(s):
        s.set_mask(solid.cuda(), q=q.cuda())

    ab, aa = _pair(nx, ny, nz, 0.7, collision="mrt", geometry=geom,
                   inlet_velocity=(0.05, 0.0, 0.0))
    g = torch.Generator().manual_seed(5)
    f0 = drivers.initial_state(nx, ny, nz, 0.05)
    f0 = (f0 + 1e-3 * torch.randn(f0.shape, generator=g)).contiguous()
    for s in (ab, aa):
        s.set_state(f0.cuda())
        s.run(9)
    assert torch.equal(ab.get_state(), aa.get_state())
    cfg = drivers.StepConfig(tau=0.7, inlet=(0.05, 0.0, 0.0), collision="mrt")
    with torch.no_grad():
        f_or, _, _ = drivers.run(f0, q, cfg, 9, solid=solid)
    assert (aa.get_state().cpu() - f_or).abs().max().item() <= 1e-5
    ab.close()
    aa.close()


@pytest.mark.parametrize("grid", [(3, 1, 2), (4, 2, 6), (6, 3, 4)])
@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_pair_kernels_on_tiny_grids(cuda, grid, storage):
    """The 16-bit pair step where a pair's y / z neighbours wrap onto itself
    or its partner: within the 16-bit storage error of the FP32 oracle."""
    nx, ny, nz = grid
    solid = torch.zeros((nx, ny, nz), dtype=torch.int32)
    q = -torch.ones((19, nx, ny, nz))
    s = L.Simulation(nx, ny, nz, 0.7, collision="mrt", storage=storage,
                     inlet_velocity=(0.05, 0.0, 0.0))
    s.set_mask(solid.cuda(), q=q.cuda())
    g = torch.Generator().manual_seed(6)
    f0 = drivers.initial_state(nx, ny, nz, 0.05)
    f0 = (f0 + 1e-3 * torch.randn(f0.shape, generator=g)).contiguous()
    s.set_state(f0.cuda())
    s.run(9)
    cfg = drivers.StepConfig(tau=0.7, inlet=(0.05, 0.0, 0.0), collision="mrt")
    with torch.no_grad():
        f_or, _, _ = drivers.run(f0, q, cfg, 9, solid=solid)
    tol = 1e-4 if storage == "fp16" else 1e-3
    assert (s.get_state().cpu() - f_or).abs().max().item() <= tol
    s.close()
