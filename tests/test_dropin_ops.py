"""Per-op drop-ins (jax_lbm.core / jax_lbm.geometry signatures) on the GPU vs
the CPU oracle: forward values and torch-autograd gradients (the jax.grad
stand-in), FP64 tight and FP32 at the reference's tolerances."""

import pytest
import torch

import lbm_jax_autodiff_gb300 as L
from lbm_jax_autodiff_gb300.core import forces as gforces
from lbm_jax_autodiff_gb300.geometry import bouzidi as gbz
from lbm_jax_autodiff_gb300.geometry import primitives as gprim
from lbm_jax_autodiff_gb300.geometry import smooth as gsmooth
from oracle import drivers, geometry, ops
from oracle.ops import consts_for

pytestmark = pytest.mark.gpu
DT = torch.float64
SHAPE = (10, 6, 5)


def _f(seed=0, dtype=DT, ux=0.05):
    g = torch.Generator().manual_seed(seed)
    nx, ny, nz = SHAPE
    f0 = drivers.initial_state(nx, ny, nz, ux, dtype, consts_for(dtype))
    return (f0 + 1e-3 * torch.randn(f0.shape, generator=g, dtype=dtype)).contiguous()


def _links(seed=1, dtype=DT, frac=0.15):
    g = torch.Generator().manual_seed(seed)
    q = torch.rand((19,) + SHAPE, generator=g, dtype=dtype) * 0.98 + 0.01
    keep = torch.rand((19,) + SHAPE, generator=g) < frac
    q = torch.where(keep, q, torch.full_like(q, -1.0))
    q[0] = -1.0
    q[1:, 2, 1, 1] = 0.5     # exact ties at 0.5 exercise the clip rule
    return q.contiguous()


def _both(fn_gpu, fn_or, inputs, tol=1e-10, seed=5):
    """Run fn on GPU and on the oracle with grads; compare outputs and input grads."""
    gi = [x.detach().cuda().requires_grad_(x.requires_grad) for x in inputs]
    ci = [x.detach().clone().requires_grad_(x.requires_grad) for x in inputs]
    og, oc = fn_gpu(*gi), fn_or(*ci)
    outs_g = og if isinstance(og, tuple) else (og,)
    outs_c = oc if isinstance(oc, tuple) else (oc,)
    gen = torch.Generator().manual_seed(seed)
    loss_g, loss_c = 0.0, 0.0
    for a, b in zip(outs_g, outs_c):
        b = b.to(a.dtype)
        scale = max(1.0, b.abs().max().item())
        assert (a.detach().cpu() - b.detach()).abs().max().item() <= tol * scale, "forward mismatch"
        if a.dtype.is_floating_point and a.requires_grad:
            w = torch.randn(b.shape, generator=gen, dtype=b.dtype)
            loss_g = loss_g + (a * w.cuda()).sum()
            loss_c = loss_c + (b * w).sum()
    if isinstance(loss_g, torch.Tensor):
        loss_g.backward()
        loss_c.backward()
        for a, b in zip(gi, ci):
            if b.requires_grad:
                assert a.grad is not None
                scale = max(1.0, b.grad.abs().max().item())
                err = (a.grad.cpu() - b.grad).abs().max().item()
                assert err <= tol * scale, "grad mismatch %.3e" % err


def test_density_velocity_equilibrium(cuda):
    f = _f().requires_grad_(True)
    _both(L.compute_density, ops.compute_density, [f])
    rho = ops.compute_density(_f()).detach().requires_grad_(True)
    _both(L.compute_velocity, ops.compute_velocity, [f, rho])
    u = ops.compute_velocity(_f(), ops.compute_density(_f())).detach().requires_grad_(True)
    _both(lambda r, uu: L.equilibrium(r, uu), lambda r, uu: ops.equilibrium(r, uu), [rho, u])


@pytest.mark.parametrize("kind", ["bgk", "mrt"])
@pytest.mark.parametrize("field", [False, True])
def test_collisions(cuda, kind, field):
    f = _f().requires_grad_(True)
    if field:
        tau = (0.6 + 0.05 * torch.rand(SHAPE, dtype=DT)).requires_grad_(True)
    else:
        tau = torch.tensor(0.58, dtype=DT, requires_grad=True)
    gk = getattr(L, kind)
    ok = getattr(ops, kind)
    _both(lambda a, t: gk(a, t), lambda a, t: ok(a, t), [f, tau], tol=1e-11)


def test_smagorinsky_tau(cuda):
    f = _f(seed=3).requires_grad_(True)
    tau = torch.tensor(0.56, dtype=DT, requires_grad=True)
    _both(lambda a, t: L.smagorinsky_tau(a, t, 0.1), lambda a, t: ops.smagorinsky_tau(a, t, 0.1),
          [f, tau], tol=1e-10)


@pytest.mark.parametrize("periodic", [True, False])
def test_stream_bouzidi(cuda, periodic):
    f = _f().requires_grad_(True)
    q = _links().requires_grad_(True)
    _both(lambda a, b: L.stream(a, b, periodic), lambda a, b: ops.stream(a, b, periodic), [f, q])


def test_zou_he(cuda):
    f = _f().requires_grad_(True)
    ux = torch.tensor(0.05, dtype=DT, requires_grad=True)
    _both(lambda a, u: L.zou_he_inlet(a, (u, 0.0, 0.01)),
          lambda a, u: ops.zou_he_inlet(a, (u, 0.0, 0.01)), [f, ux])
    prof = drivers.parabolic_inlet(SHAPE[1], SHAPE[2], 0.05, DT).requires_grad_(True)
    _both(lambda a, p: L.zou_he_inlet(a, (p, 0.0, 0.0)),
          lambda a, p: ops.zou_he_inlet(a, (p, 0.0, 0.0)), [f, prof])
    _both(lambda a: L.zou_he_inlet(a, (0.05, 0.0, 0.0), rho_target=1.02),
          lambda a: ops.zou_he_inlet(a, (0.05, 0.0, 0.0), rho_target=1.02), [f])
    ro = torch.tensor(1.01, dtype=DT, requires_grad=True)
    _both(lambda a, r: L.zou_he_outlet(a, r), lambda a, r: ops.zou_he_outlet(a, r), [f, ro])


def test_soft_bounce_back(cuda):
    f = _f().requires_grad_(True)
    p = torch.rand(SHAPE, dtype=DT).requires_grad_(True)
    _both(gsmooth.soft_bounce_back, ops.soft_bounce_back, [f, p])


def test_momentum_exchange_and_drag(cuda):
    fp = _f(1).requires_grad_(True)
    fs = _f(2).requires_grad_(True)
    q = _links()
    _both(lambda a, b: L.momentum_exchange(a, b, q.cuda()),
          lambda a, b: ops.momentum_exchange(a, b, q).to(DT), [fp, fs])
    F = torch.tensor([0.01, 0.002, 0.0], dtype=DT, requires_grad=True)
    _both(lambda x: L.drag_coefficient(x, 0.05, 100.0), lambda x: ops.drag_coefficient(x, 0.05, 100.0),
          [F])
    tot, pres = gforces.momentum_exchange_decomposed(fp.cuda().detach(), fs.cuda().detach(), q.cuda())
    ot, op_ = ops.momentum_exchange_decomposed(fp.detach(), fs.detach(), q)
    assert torch.allclose(tot.cpu(), ot.to(DT), atol=1e-12)
    assert torch.allclose(pres.cpu(), op_.to(DT), atol=1e-12)


def test_projected_area_and_q_builders(cuda):
    s = torch.zeros((16, 8, 8), dtype=torch.int32)
    s[5:8, 2:6, 2:6] = 1
    assert float(L.projected_area(s.cuda())) == 16.0
    g = torch.zeros((16, 8, 8), dtype=torch.int32)
    g[:, 0, :] = 2
    assert float(L.projected_area(g.cuda())) == 0.0
    q = gbz.compute_q_from_solid(s.cuda())
    assert torch.equal(q.cpu(), geometry.compute_q_from_solid(s))


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_create_sphere_and_box(cuda, dtype):
    solid, q = gprim.create_sphere(64, 32, 32, (0.0, 0.0, 0.0), 0.5, dtype=dtype)
    s_o, q_o = geometry.create_sphere(64, 32, 32, (0.0, 0.0, 0.0), 0.5, dtype)
    assert torch.equal(solid.cpu(), s_o)
    assert ((q.cpu() >= 0) == (q_o >= 0)).all()
    tol = 2e-6 if dtype == torch.float32 else 1e-12
    assert (q.cpu() - q_o).abs().max().item() <= tol
    sb, qb = gprim.create_box(16, 8, 8, (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), dtype=dtype)
    sbo = torch.zeros((16, 8, 8), dtype=torch.int32)
    wx, wy, wz = geometry.world_coords(16, 8, 8, dtype)
    sbo[(wx >= -0.5) & (wx <= 0.5) & (wy >= -0.5) & (wy <= 0.5) & (wz >= -0.5) & (wz <= 0.5)] = 1
    assert torch.equal(sb.cpu(), sbo)
    assert torch.equal(qb.cpu(), geometry.compute_q_from_solid(sbo, 0.5, dtype))


@pytest.mark.parametrize("q_mode,por", [("bouzidi", "soft"), ("halfway", "soft"),
                                        ("bouzidi", "hard")])
def test_sphere_geometry_radius_gradient(cuda, q_mode, por):
    nx, ny, nz = 32, 16, 16
    r = torch.tensor(0.55, dtype=DT, requires_grad=True)
    p_o, s_o, q_o = geometry.sphere_geometry(nx, ny, nz, r, q_mode, por, 20.0, dtype=DT)
    rg = torch.tensor(0.55, dtype=DT, requires_grad=True)
    p_g, s_g, q_g = gsmooth.sphere_geometry(nx, ny, nz, rg, q_mode, por, 20.0, dtype=DT)
    assert torch.equal(s_g.cpu(), s_o)
    assert (q_g.cpu() - q_o).abs().max().item() <= 1e-12
    assert (p_g.cpu() - p_o).abs().max().item() <= 1e-12
    w1 = torch.randn(q_o.shape, dtype=DT, generator=torch.Generator().manual_seed(0))
    w2 = torch.randn(p_o.shape, dtype=DT, generator=torch.Generator().manual_seed(1))
    ((q_o * w1).sum() + (p_o * w2).sum()).backward()
    ((q_g * w1.cuda()).sum() + (p_g * w2.cuda()).sum()).backward()
    assert abs(rg.grad.item() - r.grad.item()) <= 1e-9 * max(1.0, abs(r.grad.item()))


def test_state_step_and_simulate(cuda):
    """state.step with the post-BC guard (state.py:129-171) vs the oracle."""
    nx, ny, nz = 24, 12, 12
    solid, q = geometry.create_sphere(nx, ny, nz, (0.0, 0.0, 0.0), 0.6, torch.float32)
    f0 = drivers.initial_state(nx, ny, nz, 0.0)
    cfg = drivers.StepConfig(tau=0.7, inlet=(0.05, 0.0, 0.0), collision="mrt", guard="post",
                             smagorinsky_cs=0.1)
    with torch.no_grad():
        f_or, _, _ = drivers.run(f0, q, cfg, 20, solid=solid)
    st = L.LBMState(f=f0.cuda(), solid=solid.cuda(), q=q.cuda())
    pr = L.LBMParams(tau=0.7, inlet_velocity=torch.tensor([0.05, 0.0, 0.0]), collision_mode=1,
                     use_smagorinsky=1, smagorinsky_cs=0.1)
    out = L.simulate(st, pr, 20)
    assert (out.f.cpu() - f_or).abs().max().item() <= 2e-6
    one = L.step(st, pr)
    with torch.no_grad():
        f1, _, _ = drivers.step(f0, q, cfg, solid=solid)
    assert (one.f.cpu() - f1).abs().max().item() <= 1e-6


def test_cd_of_radius_autograd(cuda):
    from lbm_jax_autodiff_gb300.autograd import cd_of_radius
    nx, ny, nz = 32, 16, 16
    sim = L.Simulation(nx, ny, nz, 0.56, collision="mrt", storage="fp64")
    sim.set_state(sim.equilibrium_state())
    r = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    cd = cd_of_radius(r, sim, 12, kind="sigmoid", q_mode="bouzidi", porosity="soft")
    cd.backward()
    ro = torch.tensor(0.5, dtype=DT, requires_grad=True)
    cdo = drivers.simulate_cd(ro, nx, ny, nz, 12, 0.56, dtype=DT, consts=consts_for(DT))
    cdo.backward()
    assert abs(cd.item() - cdo.item()) <= 1e-10 * abs(cdo.item())
    assert abs(r.grad.item() - ro.grad.item()) <= 1e-8 * abs(ro.grad.item())
