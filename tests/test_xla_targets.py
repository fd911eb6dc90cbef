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
