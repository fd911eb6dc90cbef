"""Momentum-exchange force, drag coefficient and projected area
(jax_lbm/core/forces.py:37-276) on the sm_103a kernels."""

import torch

from .. import _ops as op
from .equilibrium import compute_density, compute_velocity, equilibrium


class _Momentum(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f_post, f_streamed, q):
        f_post = op.cuda_contig(f_post, "f_post")
        f_streamed = op.cuda_contig(f_streamed, "f_streamed").to(f_post.dtype)
        q = op.cuda_contig(q, "q").to(f_post.dtype)
        nx, ny, nz = op.pop_dims(f_post)
        force = torch.empty(3, dtype=torch.float64, device=f_post.device)
        op.call("lbm_momentum_exchange", op.dtype_code(f_post), op.ptr(f_post), op.ptr(f_streamed),
                op.ptr(q), op.ptr(force), nx, ny, nz, op.stream())
        ctx.save_for_backward(q)
        ctx.dims = (nx, ny, nz)
        ctx.dtype = f_post.dtype
        return force.to(f_post.dtype)

    @staticmethod
    def backward(ctx, g):
        (q,) = ctx.saved_tensors
        nx, ny, nz = ctx.dims
        g64 = g.to(torch.float64).contiguous()
        gp = torch.empty((19, nx, ny, nz), dtype=ctx.dtype, device=q.device)
        gs = torch.empty_like(gp)
        op.call("lbm_momentum_exchange_vjp", op.dtype_code(gp), op.ptr(q), op.ptr(g64), op.ptr(gp),
                op.ptr(gs), nx, ny, nz, op.stream())
        return gp, gs, None


def momentum_exchange(f_post, f_streamed, q):
    """F = sum_{i>=1} sum_x [q_i(x) >= 0] e_i (f*_i(x) + f_opp(i)(x)), shape (3,)
    (forces.py:37-120).  Summed in FP64 with a fixed-order reduction."""
    return _Momentum.apply(f_post, f_streamed, q)


def momentum_exchange_decomposed(f_post, f_streamed, q):
    """(total, pressure) forces; pressure from the equilibrium of f_post on the
    same links, friction = total - pressure (forces.py:123-196)."""
    rho = compute_density(f_post)
    feq = equilibrium(rho, compute_velocity(f_post, rho))
    return momentum_exchange(f_post, f_streamed, q), momentum_exchange(feq, feq, q)


def projected_area(solid, axis=0):
    """Number of columns along ``axis`` holding a body cell (solid == 1; ground
    value 2 excluded) (forces.py:199-234)."""
    s = op.cuda_contig(solid, "solid").to(torch.int32)
    nx, ny, nz = s.shape
    area = torch.empty(1, dtype=torch.float64, device=s.device)
    op.call("lbm_projected_area", op.ptr(s), int(axis), op.ptr(area), nx, ny, nz, op.stream())
    return area[0].to(torch.float32)


class _Drag(torch.autograd.Function):
    @staticmethod
    def forward(ctx, force, u, area, rho):
        f64 = op.cuda_contig(force, "force").to(torch.float64).contiguous()
        cd = torch.empty(1, dtype=torch.float64, device=f64.device)
        op.call("lbm_drag_coefficient", op.ptr(f64), float(u), float(area), float(rho), op.ptr(cd),
                op.stream())
        ctx.save_for_backward(f64)
        ctx.u, ctx.area, ctx.rho = float(u), float(area), float(rho)
        ctx.dtype = force.dtype
        return cd[0].to(force.dtype)

    @staticmethod
    def backward(ctx, g):
        (f64,) = ctx.saved_tensors
        den = 0.5 * ctx.rho * ctx.u * ctx.u * ctx.area + 1e-10
        gf = torch.zeros(3, dtype=ctx.dtype, device=f64.device)
        gf[0] = (torch.sign(f64[0]) / den * g).to(ctx.dtype)
        return gf, None, None, None


def drag_coefficient(force, inlet_velocity, area, rho=1.0):
    """Cd = |Fx| / (0.5 rho U^2 A + 1e-10) (forces.py:237-276)."""
    return _Drag.apply(force, inlet_velocity, area, rho)
