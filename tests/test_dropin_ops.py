"""Per-op drop-ins (jax_lbm.core / jax_lbm.geometry signatures) on the GPU vs
the CPU oracle: forward values and torch-autograd gradients (the jax.grad
stand-in).

Each op runs on three cases:
  - FP64 on a 10x6x5 grid (less than one block), to 1e-10 relative;
  - FP32 on a 48x24x24 grid (108 blocks of 256 cells) and on an odd 37x19x13
    grid (a ragged last block), at the FP32 bar: outputs and VJPs within
    1e-5 of the FP32 oracle, relative to max(1, |oracle|).
"""

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

# (grid, dtype, relative tolerance)
CASES = [
    pytest.param(((10, 6, 5), torch.float64, 1e-10), id="fp64-10x6x5"),
    pytest.param(((48, 24, 24), torch.float32, 1e-5), id="fp32-48x24x24"),
    pytest.param(((37, 19, 13), torch.float32, 1e-5), id="fp32-37x19x13"),
]


@pytest.fixture(params=CASES)
def case(request):
    return request.param


def _f(seed=0, dtype=DT, ux=0.05, shape=SHAPE):
    g = torch.Generator().manual_seed(seed)
    nx, ny, nz = shape
    f0 = drivers.initial_state(nx, ny, nz, ux, dtype, consts_for(dtype))
    return (f0 + 1e-3 * torch.randn(f0.shape, generator=g, dtype=torch.float64).to(dtype)).contiguous()


def _links(seed=1, dtype=DT, frac=0.15, shape=SHAPE):
    g = torch.Generator().manual_seed(seed)
    q = torch.rand((19,) + tuple(shape), generator=g, dtype=torch.float64).to(dtype) * 0.98 + 0.01
    keep = torch.rand((19,) + tuple(shape), generator=g) < frac
    q = torch.where(keep, q, torch.full_like(q, -1.0))
    q[0] = -1.0
    q[1:, 2, 1, 1] = 0.5     # exact ties at 0.5 exercise the clip rule
    return q.contiguous()


def _both(fn_gpu, fn_or, inputs, tol=1e-10, seed=5):
    """Run fn on GPU and on the oracle with grads; compare outputs and input
    grads elementwise, relative to max(1, max |oracle|)."""
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
        err = (a.detach().cpu().double() - b.detach().double()).abs().max().item()
        assert err <= tol * scale, "forward mismatch %.3e" % err
        if a.dtype.is_floating_point and a.requires_grad:
            w = torch.randn(b.shape, generator=gen, dtype=torch.float64).to(b.dtype)
            loss_g = loss_g + (a * w.cuda()).sum()
            loss_c = loss_c + (b * w).sum()
    if isinstance(loss_g, torch.Tensor):
        loss_g.backward()
        loss_c.backward()
        for a, b in zip(gi, ci):
            if b.requires_grad:
                assert a.grad is not None
                scale = max(1.0, b.grad.abs().max().item())
                err = (a.grad.cpu().double() - b.grad.double()).abs().max().item()
                assert err <= tol * scale, "grad mismatch %.3e" % err


def test_density_velocity_equilibrium(cuda, case):
    shape, dt, tol = case
    f = _f(dtype=dt, shape=shape).requires_grad_(True)
    _both(L.compute_density, ops.compute_density, [f], tol)
    rho = ops.compute_density(_f(dtype=dt, shape=shape)).detach().requires_grad_(True)
    _both(L.compute_velocity, ops.compute_velocity, [f, rho], tol)
    f1 = _f(dtype=dt, shape=shape)
    u = ops.compute_velocity(f1, ops.compute_density(f1)).detach().requires_grad_(True)
    _both(lambda r, uu: L.equilibrium(r, uu), lambda r, uu: ops.equilibrium(r, uu), [rho, u], tol)


@pytest.mark.parametrize("kind", ["bgk", "mrt"])
@pytest.mark.parametrize("field", [False, True])
def test_collisions(cuda, case, kind, field):
    shape, dt, tol = case
    f = _f(dtype=dt, shape=shape).requires_grad_(True)
    if field:
        g = torch.Generator().manual_seed(7)
        tau = (0.6 + 0.05 * torch.rand(shape, generator=g, dtype=torch.float64)).to(dt)
        tau = tau.requires_grad_(True)
    else:
        tau = torch.tensor(0.58, dtype=dt, requires_grad=True)
    gk = getattr(L, kind)
    ok = getattr(ops, kind)
    _both(lambda a, t: gk(a, t), lambda a, t: ok(a, t), [f, tau],
          tol=1e-11 if dt == torch.float64 else tol)


def test_smagorinsky_tau(cuda, case):
    shape, dt, tol = case
    f = _f(seed=3, dtype=dt, shape=shape).requires_grad_(True)
    tau = torch.tensor(0.56, dtype=dt, requires_grad=True)
    _both(lambda a, t: L.smagorinsky_tau(a, t, 0.1), lambda a, t: ops.smagorinsky_tau(a, t, 0.1),
          [f, tau], tol=tol)


@pytest.mark.parametrize("periodic", [True, False])
def test_stream_bouzidi(cuda, case, periodic):
    shape, dt, tol = case
    f = _f(dtype=dt, shape=shape).requires_grad_(True)
    q = _links(dtype=dt, shape=shape).requires_grad_(True)
    _both(lambda a, b: L.stream(a, b, periodic), lambda a, b: ops.stream(a, b, periodic), [f, q],
          tol)


def test_zou_he(cuda, case):
    shape, dt, tol = case
    f = _f(dtype=dt, shape=shape).requires_grad_(True)
    ux = torch.tensor(0.05, dtype=dt, requires_grad=True)
    _both(lambda a, u: L.zou_he_inlet(a, (u, 0.0, 0.01)),
          lambda a, u: ops.zou_he_inlet(a, (u, 0.0, 0.01)), [f, ux], tol)
    prof = drivers.parabolic_inlet(shape[1], shape[2], 0.05, dt).requires_grad_(True)
    _both(lambda a, p: L.zou_he_inlet(a, (p, 0.0, 0.0)),
          lambda a, p: ops.zou_he_inlet(a, (p, 0.0, 0.0)), [f, prof], tol)
    _both(lambda a: L.zou_he_inlet(a, (0.05, 0.0, 0.0), rho_target=1.02),
          lambda a: ops.zou_he_inlet(a, (0.05, 0.0, 0.0), rho_target=1.02), [f], tol)
    ro = torch.tensor(1.01, dtype=dt, requires_grad=True)
    _both(lambda a, r: L.zou_he_outlet(a, r), lambda a, r: ops.zou_he_outlet(a, r), [f, ro], tol)


def test_soft_bounce_back(cuda, case):
    shape, dt, tol = case
    f = _f(dtype=dt, shape=shape).requires_grad_(True)
    g = torch.Generator().manual_seed(11)
    p = torch.rand(shape, generator=g, dtype=torch.float64).to(dt).requires_grad_(True)
    _both(gsmooth.soft_bounce_back, ops.soft_bounce_back, [f, p], tol)


def test_momentum_exchange_and_drag(cuda, case):
    shape, dt, tol = case
    fp = _f(1, dtype=dt, shape=shape).requires_grad_(True)
    fs = _f(2, dtype=dt, shape=shape).requires_grad_(True)
    q = _links(dtype=dt, shape=shape)
    # the force is an FP64 sum on both sides; its value is O(links), so the
    # relative bar applies to max(1, |F|)
    _both(lambda a, b: L.momentum_exchange(a, b, q.cuda()),
          lambda a, b: ops.momentum_exchange(a, b, q).to(torch.float64), [fp, fs], tol)
    F = torch.tensor([0.01, 0.002, 0.0], dtype=torch.float64, requires_grad=True)
    _both(lambda x: L.drag_coefficient(x, 0.05, 100.0), lambda x: ops.drag_coefficient(x, 0.05, 100.0),
          [F], tol)
    tot, pres = gforces.momentum_exchange_decomposed(fp.cuda().detach(), fs.cuda().detach(), q.cuda())
    ot, op_ = ops.momentum_exchange_decomposed(fp.detach(), fs.detach(), q)
    atol = 1e-12 if dt == torch.float64 else tol * max(1.0, ot.abs().max().item())
    assert torch.allclose(tot.cpu().double(), ot.double(), rtol=0, atol=atol)
    assert torch.allclose(pres.cpu().double(), op_.double(), rtol=0, atol=atol)


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


def test_simulate_gradient_vs_oracle_autograd(cuda):
    """jax.grad through simulate (state.py:174-230) with respect to state.f and
    state.q: the adjoint kernels (lbm_vjp_run) against FP64 autograd through
    the oracle's step order, with the post-boundary guard (which resets no
    cell here, so its gradient is the unguarded one)."""
    dt = torch.float64
    nx, ny, nz, n = 16, 8, 8, 6
    solid, q = geometry.create_sphere(nx, ny, nz, (0.0, 0.0, 0.0), 0.7, dt)
    g = torch.Generator().manual_seed(3)
    f0 = drivers.initial_state(nx, ny, nz, 0.05, dt, consts_for(dt))
    f0 = f0 + 1e-3 * torch.randn(f0.shape, generator=g, dtype=dt)
    w = torch.randn(f0.shape, generator=g, dtype=dt)
    cfg = drivers.StepConfig(tau=0.6, inlet=(0.05, 0.0, 0.0), collision="mrt", guard="post",
                             smagorinsky_cs=0.1)
    fo = f0.clone().requires_grad_(True)
    qo = q.clone().requires_grad_(True)
    f_or, _, resets = drivers.run(fo, qo, cfg, n, solid=solid, consts=consts_for(dt))
    assert resets == 0
    (f_or * w).sum().backward()
    st = L.LBMState(f=f0.cuda().requires_grad_(True), solid=solid.cuda(),
                    q=q.cuda().requires_grad_(True))
    pr = L.LBMParams(tau=0.6, inlet_velocity=torch.tensor([0.05, 0.0, 0.0]), collision_mode=1,
                     use_smagorinsky=1, smagorinsky_cs=0.1)
    out = L.simulate(st, pr, n)
    # FP64 fused step against the FP64 oracle: rounding only
    assert (out.f.detach().cpu() - f_or.detach()).abs().max().item() <= 1e-9
    (out.f * w.cuda()).sum().backward()
    gf = st.f.grad.cpu()
    assert (gf - fo.grad).abs().max().item() <= 1e-8 * fo.grad.abs().max().item()
    links = q >= 0
    gq = st.q.grad.cpu()
    err = (gq[links] - qo.grad[links]).abs().max().item()
    assert err <= 1e-8 * qo.grad[links].abs().max().item()
    assert (gq[~links] == 0).all()


def test_simulate_keeps_geometry_and_state_between_calls(cuda):
    """A loop of simulate calls fed its own output continues from the
    handle's state and keeps its geometry: the same f as one long run."""
    nx, ny, nz = 24, 12, 12
    solid, q = geometry.create_sphere(nx, ny, nz, (0.0, 0.0, 0.0), 0.6, torch.float32)
    f0 = drivers.initial_state(nx, ny, nz, 0.05).cuda()
    st = L.LBMState(f=f0, solid=solid.cuda(), q=q.cuda())
    pr = L.LBMParams(tau=0.7, inlet_velocity=torch.tensor([0.05, 0.0, 0.0]), collision_mode=1)
    one = L.simulate(st, pr, 30)
    cur = st
    for _ in range(3):
        cur = L.simulate(cur, pr, 10)
    assert torch.equal(cur.f, one.f)
    for _ in range(5):
        cur = L.step(cur, pr)
    assert torch.equal(cur.f, L.simulate(st, pr, 35).f)


def test_get_state_and_step_equals_the_two_calls(cuda):
    """lbm_get_state_and_step: f of the current step and one more step, to the
    bit what get_state followed by run(1) gives, in FP32 and FP64, right after
    set_state (the unfused fallback) and in a running state (the fused launch),
    with the post-BC guard resetting planted cells in between."""
    nx, ny, nz = 24, 12, 12
    for dtype, storage in ((torch.float32, "fp32"), (torch.float64, "fp64")):
        solid, q = geometry.create_sphere(nx, ny, nz, (0.0, 0.0, 0.0), 0.6, dtype)
        f0 = drivers.initial_state(nx, ny, nz, 0.05, dtype, consts_for(dtype))
        f0[:, 3, 5, 5] = float("nan")            # reset by the post-BC guard
        sims = []
        for _ in range(2):
            s = L.Simulation(nx, ny, nz, 0.7, collision="mrt", storage=storage, guard="post",
                             inlet_velocity=(0.05, 0.0, 0.0))
            s.set_mask(solid.cuda(), q=q.cuda())
            s.set_state(f0.cuda())
            sims.append(s)
        fused, plain = sims
        bits = torch.int32 if dtype == torch.float32 else torch.int64

        def same(x, y):                          # to the bit, NaN included
            return torch.equal(x.view(bits), y.view(bits))

        for k in range(4):
            a = fused.get_state_and_step()
            b = plain.get_state()
            plain.run(1)
            assert same(a, b), (storage, k)
            fused.run(2)
            plain.run(2)
        assert same(fused.get_state(), plain.get_state())
        assert fused.guard_resets == plain.guard_resets > 0
        for s in sims:
            s.close()


def test_state_calls_mixed_with_restarts(cuda):
    """simulate / step calls that continue, restart from a modified f, and run
    zero steps give the f a fresh handle gives."""
    nx, ny, nz = 24, 12, 12
    solid, q = geometry.create_sphere(nx, ny, nz, (0.0, 0.0, 0.0), 0.6, torch.float32)
    f0 = drivers.initial_state(nx, ny, nz, 0.05).cuda()
    st = L.LBMState(f=f0, solid=solid.cuda(), q=q.cuda())
    pr = L.LBMParams(tau=0.7, inlet_velocity=torch.tensor([0.05, 0.0, 0.0]), collision_mode=1)
    a = L.step(L.simulate(st, pr, 3), pr)            # 4 steps, continuing
    z = L.simulate(a, pr, 0)
    assert torch.equal(z.f, a.f)
    b = L.step(z, pr)                                # 5 steps
    g = b.f.clone()
    b.f.mul_(1.0)                                    # same values, a new version: restart
    c = L.simulate(b, pr, 2)                         # 7 steps
    ref = L.simulate(L.LBMState(f=g, solid=st.solid, q=st.q), pr, 2)
    assert torch.equal(c.f, ref.f)
    assert torch.equal(c.f, L.simulate(st, pr, 7).f)
    L.clear_handles()                                # a fresh handle gives the same f
    assert torch.equal(c.f, L.simulate(st, pr, 7).f)
