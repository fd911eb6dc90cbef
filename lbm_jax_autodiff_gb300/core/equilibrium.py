"""Equilibrium, density and velocity (jax_lbm/core/equilibrium.py:22-151) on
the sm_103a kernels, differentiable through torch.autograd."""

import torch

from .. import _ops as op


class _Density(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f):
        f = op.cuda_contig(f, "f")
        nx, ny, nz = op.pop_dims(f)
        rho = torch.empty((nx, ny, nz), dtype=f.dtype, device=f.device)
        op.call("lbm_compute_density", op.dtype_code(f), op.ptr(f), op.ptr(rho), nx, ny, nz,
                op.stream())
        ctx.dims = (nx, ny, nz)
        return rho

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        nx, ny, nz = ctx.dims
        gf = torch.empty((19, nx, ny, nz), dtype=g.dtype, device=g.device)
        op.call("lbm_compute_density_vjp", op.dtype_code(g), op.ptr(g), op.ptr(gf), nx, ny, nz,
                op.stream())
        return gf


class _Velocity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, rho):
        f = op.cuda_contig(f, "f")
        rho = op.cuda_contig(rho, "rho").to(f.dtype)
        nx, ny, nz = op.pop_dims(f)
        u = torch.empty((3, nx, ny, nz), dtype=f.dtype, device=f.device)
        op.call("lbm_compute_velocity", op.dtype_code(f), op.ptr(f), op.ptr(rho), op.ptr(u),
                nx, ny, nz, op.stream())
        ctx.save_for_backward(f, rho)
        return u

    @staticmethod
    def backward(ctx, g):
        f, rho = ctx.saved_tensors
        g = g.contiguous()
        nx, ny, nz = op.pop_dims(f)
        gf = torch.empty_like(f)
        grho = torch.empty_like(rho)
        op.call("lbm_compute_velocity_vjp", op.dtype_code(f), op.ptr(f), op.ptr(rho), op.ptr(g),
                op.ptr(gf), op.ptr(grho), nx, ny, nz, op.stream())
        return gf, grho


class _Equilibrium(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho, u, flags):
        rho = op.cuda_contig(rho, "rho")
        u = op.cuda_contig(u, "u").to(rho.dtype)
        if u.dim() != 4 or u.shape[0] != 3 or tuple(u.shape[1:]) != tuple(rho.shape):
            raise ValueError("u must have shape (3,) + rho.shape")
        nx, ny, nz = rho.shape
        feq = torch.empty((19, nx, ny, nz), dtype=rho.dtype, device=rho.device)
        op.call("lbm_equilibrium", op.dtype_code(rho), op.ptr(rho), op.ptr(u), op.ptr(feq),
                nx, ny, nz, flags, op.stream())
        ctx.save_for_backward(rho, u)
        ctx.flags = flags
        return feq

    @staticmethod
    def backward(ctx, g):
        rho, u = ctx.saved_tensors
        g = g.contiguous()
        nx, ny, nz = rho.shape
        grho = torch.empty_like(rho)
        gu = torch.empty_like(u)
        op.call("lbm_equilibrium_vjp", op.dtype_code(rho), op.ptr(rho), op.ptr(u), op.ptr(g),
                op.ptr(grho), op.ptr(gu), nx, ny, nz, ctx.flags, op.stream())
        return grho, gu, None


def compute_density(f):
    """rho = sum_i f_i, shape (nx, ny, nz) (equilibrium.py:22-48)."""
    return _Density.apply(f)


def compute_velocity(f, rho):
    """u = sum_i f_i e_i / rho, shape (3, nx, ny, nz) (equilibrium.py:51-87)."""
    return _Velocity.apply(f, rho)


def equilibrium(rho, u, exact_constants=False):
    """f_eq = w rho (1 + 3 e.u + 4.5 (e.u)^2 - 1.5 u^2), shape (19, nx, ny, nz)
    (equilibrium.py:90-151).  Weights are the reference's float32 values unless
    exact_constants."""
    return _Equilibrium.apply(rho, u, op.FLAGS_EXACT if exact_constants else 0)
