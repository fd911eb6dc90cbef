"""The jax.ffi wrappers (lbm_jax_autodiff_gb300.jax_ffi) run through a
stand-in for jax (tests/jaxlike.py) that calls the registered XLA targets the
way XLA does.  JAX itself is absent here, so this is what executes the
wrappers' operand / result order, descriptors and custom_vjp rules: each
wrapper's value and VJP must equal the torch drop-in's value and autograd
gradient on the same inputs, and the fused targets the solver handle's."""

import sys

import pytest
import torch

import lbm_jax_autodiff_gb300 as L
from lbm_jax_autodiff_gb300.geometry.smooth import soft_bounce_back
from oracle import drivers

pytestmark = pytest.mark.gpu


@pytest.fixture
def jf(cuda, monkeypatch):
    import jaxlike
    from lbm_jax_autodiff_gb300 import jax_ffi
    jax, jnp = jaxlike.make()
    monkeypatch.setitem(sys.modules, "jax", jax)
    monkeypatch.setitem(sys.modules, "jax.numpy", jnp)
    monkeypatch.setattr(torch.Tensor, "astype", lambda self, dt: self.to(dt), raising=False)
    monkeypatch.setattr(jax_ffi, "_fns", None)
    monkeypatch.setattr(jax_ffi, "_registered", False)
    return jax_ffi, jax


def _f(shape=(20, 10, 8), seed=0, dtype=torch.float64):
    g = torch.Generator().manual_seed(seed)
    f0 = drivers.initial_state(*shape, 0.05, dtype)
    return (f0 + 1e-3 * torch.randn(f0.shape, generator=g, dtype=dtype)).cuda()


def _check(jax, jfn, tfn, args, diff, seed=1, tol=1e-12):
    """jfn (a custom_vjp) against tfn (torch autograd) on args; diff: the
    positions of the differentiable args."""
    out, pull = jax.vjp(jfn, *args)
    targs = [a.clone().requires_grad_(True) if k in diff else a for k, a in enumerate(args)]
    tout = tfn(*targs)
    assert torch.allclose(out.double(), tout.detach().double(), rtol=0, atol=tol)
    g = torch.randn(out.shape, generator=torch.Generator().manual_seed(seed),
                    dtype=torch.float64).to(out.device, out.dtype)
    cts = pull(g)
    tg = torch.autograd.grad(tout, [targs[k] for k in diff], g)
    for a, b in zip(cts, tg):
        assert torch.allclose(a.double(), b.double(), rtol=0, atol=tol * max(1.0, b.abs().max().item()))


def test_per_op_wrappers_match_the_torch_dropins(jf):
    jax_ffi, jax = jf
    f = _f()
    rho = f.sum(0)
    u = torch.einsum("ixyz,ic->cxyz", f, torch.tensor(
        [[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
         [1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 0, 1], [-1, 0, -1], [1, 0, -1],
         [-1, 0, 1], [0, 1, 1], [0, -1, -1], [0, 1, -1], [0, -1, 1]],
        dtype=f.dtype, device=f.device)) / rho
    q = torch.where(torch.rand(f.shape, generator=torch.Generator().manual_seed(2),
                               dtype=f.dtype).cuda() < 0.1,
                    torch.full_like(f, 0.3), torch.full_like(f, -1.0))
    por = torch.rand(f.shape[1:], generator=torch.Generator().manual_seed(3),
                     dtype=f.dtype).cuda()
    _check(jax, jax_ffi.compute_density, L.compute_density, (f,), (0,))
    _check(jax, jax_ffi.compute_velocity, L.compute_velocity, (f, rho), (0, 1))
    _check(jax, jax_ffi.equilibrium, L.equilibrium, (rho, u), (0, 1))
    jax_ffi.mrt                                      # builds the wrappers
    fns = jax_ffi._fns
    _check(jax, fns["_mrt_scalar"], lambda a, t: L.mrt(a, t), (f, 0.6), (0,))
    _check(jax, fns["_bgk_scalar"], lambda a, t: L.bgk(a, t), (f, 0.6), (0,))
    assert torch.equal(jax_ffi.mrt(f, 0.6), L.mrt(f, 0.6))
    _check(jax, jax_ffi.smagorinsky_tau, lambda a, t, c: L.smagorinsky_tau(a, t, c),
           (f, 0.55, 0.1), (0,))
    _check(jax, jax_ffi.soft_bounce_back, soft_bounce_back, (f, por), (0, 1))
    _check(jax, jax_ffi.stream, lambda a, b, p: L.stream(a, b, p), (f, q, True), (0, 1))
    _check(jax, jax_ffi.stream, lambda a, b, p: L.stream(a, b, p), (f, q, False), (0, 1))
    _check(jax, fns["_zi_uniform"], lambda a, v, r: L.zou_he_inlet(a, v, r),
           (f, (0.05, 0.0, 0.01), None), (0,))
    _check(jax, fns["_zi_uniform"], lambda a, v, r: L.zou_he_inlet(a, v, r),
           (f, (0.05, 0.0, 0.0), 1.02), (0,))
    prof = drivers.parabolic_inlet(f.shape[2], f.shape[3], 0.05, f.dtype).cuda()
    face = torch.stack([prof, 0.1 * prof, torch.zeros_like(prof)]).contiguous()
    _check(jax, fns["_zi_face"], lambda a, fc, r: L.zou_he_inlet(a, (fc[0], fc[1], fc[2]), r),
           (f, face, None), (0, 1))
    # the public dispatchers pick those forms
    assert torch.equal(jax_ffi.zou_he_inlet(f, (prof, 0.1 * prof, 0.0)),
                       L.zou_he_inlet(f, (prof, 0.1 * prof, 0.0)))
    assert torch.equal(jax_ffi.zou_he_inlet(f, (0.05, 0.0, 0.0), 1.02),
                       L.zou_he_inlet(f, (0.05, 0.0, 0.0), 1.02))
    tau_field = L.smagorinsky_tau(f, 0.55, 0.1)
    for kind in ("mrt", "bgk"):
        _check(jax, fns["_%s_field" % kind], lambda a, t: getattr(L, kind)(a, t),
               (f, tau_field), (0, 1))
        assert torch.equal(getattr(jax_ffi, kind)(f, tau_field), getattr(L, kind)(f, tau_field))
    _check(jax, jax_ffi.zou_he_outlet, lambda a, r: L.zou_he_outlet(a, r), (f, 1.01), (0,))
    fs = _f(seed=4)
    _check(jax, jax_ffi.momentum_exchange, L.momentum_exchange, (f, fs, q), (0, 1), tol=1e-12)


def test_fused_wrappers_match_the_solver(jf):
    jax_ffi, jax = jf
    from lbm_jax_autodiff_gb300 import solver
    nx, ny, nz, tau, n = 32, 16, 16, 0.56, 30
    sph = dict(kind="sigmoid", q_mode="bouzidi", porosity="soft", sharpness=20.0)
    sim = L.Simulation(nx, ny, nz, tau, collision="mrt", use_smagorinsky=True)
    sim.set_sphere(0.5, **sph)
    f0 = sim.equilibrium_state().contiguous()
    sim.set_state(f0)
    smp_ref = sim.run(n, sample_every=10)
    f_ref = sim.get_state()
    p = solver.params_struct(nx, ny, nz, tau, collision="mrt", use_smagorinsky=True)
    s = solver.sphere_struct(0.5, **sph)
    f, smp, status = jax_ffi.fused_run(f0, 0.5, jax_ffi.fused_descriptor(p, s, n, 10), 3)
    assert int(status[0]) == 0
    assert torch.equal(f, f_ref) and torch.equal(smp, smp_ref)
    sim.set_state(f0)
    cd_ref, g_ref = sim.cd_and_grad(n, checkpoint_every=6)
    cd_of, cd_and_grad = jax_ffi.simulate_cd(jax_ffi.fused_descriptor(p, s, n, 0, 6))
    cd, pull = jax.vjp(cd_of, torch.tensor(0.5, dtype=torch.float64), f0)
    g_r, g_f0 = pull(torch.tensor(1.0, dtype=torch.float64, device="cuda"))
    assert float(cd) == cd_ref and float(g_r) == g_ref
    assert not g_f0.any()
    sim.close()
