"""Pull streaming with Bouzidi bounce-back (jax_lbm/core/streaming.py:40-185)
on the sm_103a kernels, differentiable in f and q."""

import torch

from .. import _ops as op


class _Stream(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, q, periodic_yz):
        f = op.cuda_contig(f, "f")
        q = op.cuda_contig(q, "q").to(f.dtype)
        nx, ny, nz = op.pop_dims(f)
        if tuple(q.shape) != tuple(f.shape):
            raise ValueError("q must have the shape of f")
        out = torch.empty_like(f)
        op.call("lbm_stream", op.dtype_code(f), op.ptr(f), op.ptr(q), int(bool(periodic_yz)),
                op.ptr(out), nx, ny, nz, op.stream())
        ctx.save_for_backward(f, q)
        ctx.periodic = int(bool(periodic_yz))
        return out

    @staticmethod
    def backward(ctx, g):
        f, q = ctx.saved_tensors
        g = g.contiguous()
        nx, ny, nz = op.pop_dims(f)
        gf = torch.empty_like(f)
        gq = torch.empty_like(q) if ctx.needs_input_grad[1] else None
        op.call("lbm_stream_vjp", op.dtype_code(f), op.ptr(f), op.ptr(q), ctx.periodic, op.ptr(g),
                op.ptr(gf), op.ptr(gq), nx, ny, nz, op.stream())
        return gf, gq, None


def stream(f, q, periodic_yz=True):
    """f_out[i](x) = f[i](x - e_i) (x never periodic: out-of-range sources keep
    the cell's own value; y/z periodic or clamped), Bouzidi on links with
    q[opp i](x) >= 0 (streaming.py:40-185)."""
    return _Stream.apply(f, q, periodic_yz)
