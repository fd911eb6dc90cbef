"""The XLA custom-call targets (what jax.ffi binds) called directly through
ctypes with device buffers and the text descriptor, checked against the
per-op entry points (JAX itself is not installed on either machine)."""

import ctypes

import pytest
import torch

import lbm_jax_autodiff_gb300 as L
from lbm_jax_autodiff_gb300 import jax_ffi
from oracle import drivers

pytestmark = pytest.mark.gpu


def _run(name, bufs, desc):
    arr = (ctypes.c_void_p * len(bufs))(*[b.data_ptr() for b in bufs])
    d = desc.encode()
    fn = jax_ffi.xla_target(name)
    fn(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), arr, d, len(d))
    torch.cuda.synchronize()


def test_xla_stream_bgk_inlet_momentum(cuda):
    nx, ny, nz = 12, 6, 6
    f = (drivers.initial_state(nx, ny, nz, 0.05, torch.float64) +
         1e-3 * torch.randn(19, nx, ny, nz, dtype=torch.float64)).cuda()
    q = -torch.ones_like(f)
    q[1, 5] = 0.3
    q[7, 6, 2] = 0.7
    desc = jax_ffi.descriptor(nx, ny, nz, 1, periodic_yz=1, tau=0.6, u=(0.05, 0.0, 0.0), rho=1.0)
    out = torch.empty_like(f)
    _run("stream", [f, q, out], desc)
    assert torch.equal(out, L.stream(f, q, True))
    _run("bgk", [f, out], desc)
    assert torch.equal(out, L.bgk(f, 0.6))
    _run("zou_he_inlet", [f, out], desc)
    assert torch.equal(out, L.zou_he_inlet(f, (0.05, 0.0, 0.0)))
    force = torch.empty(3, dtype=torch.float64, device="cuda")
    _run("momentum_exchange", [f, f, q, force], desc)
    assert torch.allclose(force, L.momentum_exchange(f, f, q), atol=0, rtol=0)
    g = torch.randn_like(f)
    gf, gq = torch.empty_like(f), torch.empty_like(q)
    _run("stream_vjp", [f, q, g, gf, gq], desc)
    fr, qr = f.clone().requires_grad_(True), q.clone().requires_grad_(True)
    (L.stream(fr, qr, True) * g).sum().backward()
    assert torch.allclose(gf, fr.grad) and torch.allclose(gq, qr.grad)


def test_xla_failure_fills_results_with_nan(cuda):
    """A target whose call fails writes NaN into its results instead of
    leaving them unwritten (the legacy custom-call API has no status)."""
    nx, ny, nz = 12, 6, 6
    q = -torch.ones((19, nx, ny, nz), dtype=torch.float64, device="cuda")
    out = torch.zeros((19, nx, ny, nz), dtype=torch.float64, device="cuda")
    desc = jax_ffi.descriptor(nx, ny, nz, 1, periodic_yz=1)
    arr = (ctypes.c_void_p * 3)(None, q.data_ptr(), out.data_ptr())   # f missing: LBM_ERR_ARG
    d = desc.encode()
    jax_ffi.xla_target("stream")(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), arr,
                                 d, len(d))
    torch.cuda.synchronize()
    assert torch.isnan(out).all()
    force = torch.zeros(3, dtype=torch.float64, device="cuda")
    arr = (ctypes.c_void_p * 4)(q.data_ptr(), None, q.data_ptr(), force.data_ptr())
    jax_ffi.xla_target("momentum_exchange")(
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), arr, d, len(d))
    torch.cuda.synchronize()
    assert torch.isnan(force).all()


def _fused(nx, ny, nz, tau, n, sample_every=0, K=0, **sph):
    from lbm_jax_autodiff_gb300 import solver
    p = solver.params_struct(nx, ny, nz, tau, collision="mrt", use_smagorinsky=True)
    s = solver.sphere_struct(0.5, **sph)
    return jax_ffi.fused_descriptor(p, s, n, sample_every, K)


def _run_raw(name, bufs, d):
    arr = (ctypes.c_void_p * len(bufs))(*[b.data_ptr() for b in bufs])
    jax_ffi.xla_target(name)(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), arr, d,
                             len(d))
    torch.cuda.synchronize()


def test_xla_fused_run_and_gradient_match_the_solver(cuda):
    """lbm_xla_run / lbm_xla_cd_and_grad (the fused solver behind a custom
    call) against the solver handle on the same problem, to the bit."""
    nx, ny, nz, tau, n = 32, 16, 16, 0.56, 40
    sph = dict(kind="sigmoid", q_mode="bouzidi", porosity="soft", sharpness=20.0)
    sim = L.Simulation(nx, ny, nz, tau, collision="mrt", use_smagorinsky=True)
    sim.set_sphere(0.5, **sph)
    f0 = sim.equilibrium_state().contiguous()
    sim.set_state(f0)
    smp_ref = sim.run(n, sample_every=20)
    f_ref = sim.get_state()
    r = torch.tensor([0.5], dtype=torch.float64, device="cuda")
    f = torch.empty_like(f0)
    smp = torch.empty((2, 4), dtype=torch.float64, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    for _ in range(2):                      # second call: handle and geometry reused
        _run_raw("run", [f0, r, f, smp, status], _fused(nx, ny, nz, tau, n, 20, **sph))
        assert int(status) == 0
        assert torch.equal(f, f_ref) and torch.equal(smp, smp_ref)
    sim.set_state(f0)
    cd_ref, g_ref, ex = sim.cd_and_grad(n, checkpoint_every=8, dcd_dq=True)
    cd = torch.empty(1, dtype=torch.float64, device="cuda")
    g = torch.empty_like(cd)
    dq = torch.empty_like(f0)
    _run_raw("cd_and_grad", [f0, r, cd, g, dq, status], _fused(nx, ny, nz, tau, n, 0, 8, **sph))
    assert int(status) == 0
    assert float(cd) == cd_ref and float(g) == g_ref
    assert torch.equal(dq, ex["dcd_dq"])
    sim.close()


def test_xla_fused_failure_sets_status_and_nan(cuda):
    """An invalid configuration (tau <= 0.5): non-zero status, NaN results."""
    from lbm_jax_autodiff_gb300 import _native as nat
    nx, ny, nz, n = 16, 8, 8, 4
    f0 = torch.zeros((19, nx, ny, nz), dtype=torch.float32, device="cuda")
    r = torch.tensor([0.5], dtype=torch.float64, device="cuda")
    cd = torch.zeros(1, dtype=torch.float64, device="cuda")
    g = torch.zeros_like(cd)
    dq = torch.zeros_like(f0)
    status = torch.zeros((1,), dtype=torch.int32, device="cuda")
    _run_raw("cd_and_grad", [f0, r, cd, g, dq, status], _fused(nx, ny, nz, 0.4, n))
    assert int(status) == nat.LBM_ERR_ARG
    assert torch.isnan(cd).all() and torch.isnan(g).all() and torch.isnan(dq).all()


def test_xla_fused_handles_beyond_the_cache_bound(cuda):
    """Twelve parameter sets (more than the library keeps handles for) run in
    turn and then again: every call matches its own solver handle, so evicted
    handles are rebuilt, not reused."""
    nx, ny, nz, n = 16, 8, 8, 10
    sph = dict(kind="dist", q_mode="bouzidi", porosity="hard")
    taus = [0.52 + 0.01 * k for k in range(12)]
    ref = {}
    for tau in taus:
        sim = L.Simulation(nx, ny, nz, tau, collision="mrt", use_smagorinsky=True)
        sim.set_sphere(0.5, **sph)
        f0 = sim.equilibrium_state().contiguous()
        sim.set_state(f0)
        sim.run(n)
        ref[tau] = (f0, sim.get_state())
        sim.close()
    r = torch.tensor([0.5], dtype=torch.float64, device="cuda")
    smp = torch.zeros((1, 4), dtype=torch.float64, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    for tau in taus + taus[:3]:
        f0, f_ref = ref[tau]
        f = torch.empty_like(f0)
        _run_raw("run", [f0, r, f, smp, status], _fused(nx, ny, nz, tau, n, **sph))
        assert int(status) == 0, tau
        assert torch.equal(f, f_ref), tau
