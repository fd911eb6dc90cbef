"""BGK, MRT and Smagorinsky (jax_lbm/core/collision.py:46-270) on the sm_103a
kernels, differentiable through torch.autograd (f and tau)."""

import torch

from .. import _ops as op


def _tau_args(tau, f):
    """(tau_field tensor or None, scalar tau value, scalar-tensor or None)."""
    if torch.is_tensor(tau) and tau.dim() > 0:
        t = op.cuda_contig(tau, "tau").to(f.dtype)
        if tuple(t.shape) != tuple(f.shape[1:]):
            raise ValueError("a tau field must have shape (nx, ny, nz)")
        return t, 0.0
    return None, float(tau)


class _Collide(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, tau, kind, flags):
        f = op.cuda_contig(f, "f")
        nx, ny, nz = op.pop_dims(f)
        tf, tv = _tau_args(tau, f)
        out = torch.empty_like(f)
        op.call("lbm_" + kind, op.dtype_code(f), op.ptr(f), op.ptr(tf), tv, op.ptr(out), nx, ny,
                nz, flags, op.stream())
        ctx.save_for_backward(f, tf if tf is not None else torch.empty(0, device=f.device))
        ctx.kind, ctx.flags, ctx.tv = kind, flags, tv
        ctx.tau_is_tensor = torch.is_tensor(tau)
        ctx.tau_field = tf is not None
        return out

    @staticmethod
    def backward(ctx, g):
        f, tf = ctx.saved_tensors
        tf = tf if ctx.tau_field else None
        g = g.contiguous()
        nx, ny, nz = op.pop_dims(f)
        gf = torch.empty_like(f)
        want_tau = ctx.tau_is_tensor and ctx.needs_input_grad[1]
        gt = torch.empty((nx, ny, nz), dtype=f.dtype, device=f.device) if want_tau else None
        op.call("lbm_" + ctx.kind + "_vjp", op.dtype_code(f), op.ptr(f), op.ptr(tf), ctx.tv,
                op.ptr(g), op.ptr(gf), op.ptr(gt), nx, ny, nz, ctx.flags, op.stream())
        g_tau = None
        if want_tau:
            g_tau = gt if ctx.tau_field else gt.sum()
        return gf, g_tau, None, None


def bgk(f, tau, exact_constants=False):
    """f - (f - f_eq) / tau; tau a scalar or an (nx, ny, nz) field (collision.py:46-100)."""
    return _Collide.apply(f, tau, "bgk", op.FLAGS_EXACT if exact_constants else 0)


def mrt(f, tau, exact_constants=False):
    """Multiple-relaxation-time collision, stress moments relaxed at 1/tau
    (collision.py:103-184)."""
    return _Collide.apply(f, tau, "mrt", op.FLAGS_EXACT if exact_constants else 0)


class _Smag(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, tau, cs, flags):
        f = op.cuda_contig(f, "f")
        nx, ny, nz = op.pop_dims(f)
        out = torch.empty((nx, ny, nz), dtype=f.dtype, device=f.device)
        op.call("lbm_smagorinsky_tau", op.dtype_code(f), op.ptr(f), float(tau), float(cs),
                op.ptr(out), nx, ny, nz, flags, op.stream())
        ctx.save_for_backward(f)
        ctx.tv, ctx.cs, ctx.flags = float(tau), float(cs), flags
        ctx.tau_is_tensor = torch.is_tensor(tau)
        return out

    @staticmethod
    def backward(ctx, g):
        (f,) = ctx.saved_tensors
        g = g.contiguous()
        nx, ny, nz = op.pop_dims(f)
        gf = torch.empty_like(f)
        want_tau = ctx.tau_is_tensor and ctx.needs_input_grad[1]
        gt = torch.empty((nx, ny, nz), dtype=f.dtype, device=f.device) if want_tau else None
        op.call("lbm_smagorinsky_tau_vjp", op.dtype_code(f), op.ptr(f), ctx.tv, ctx.cs, op.ptr(g),
                op.ptr(gf), op.ptr(gt), nx, ny, nz, ctx.flags, op.stream())
        return gf, (gt.sum() if want_tau else None), None, None


def smagorinsky_tau(f, tau, cs=0.1, exact_constants=False):
    """tau_eff = (tau + sqrt(tau^2 + 18 Cs^2 |Pi_neq| / (rho + 1e-10))) / 2
    (collision.py:187-270).  Its gradient at Pi_neq = 0 is the subgradient 0
    (jax.grad returns NaN there)."""
    return _Smag.apply(f, tau, cs, op.FLAGS_EXACT if exact_constants else 0)
