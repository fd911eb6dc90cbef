"""Sigmoid porosity, soft bounce-back and the differentiable sphere
(jax_lbm/geometry/smooth.py:34-248) on the sm_103a kernels."""

import torch

from .. import _ops as op
from .primitives import sphere_fields, sphere_struct


def signed_distance_sphere(nx, ny, nz, center, radius, dtype=torch.float32, device="cuda"):
    """r - |x - c| in the world frame (smooth.py:34-78)."""
    gx = torch.arange(nx, dtype=dtype, device=device)
    gy = torch.arange(ny, dtype=dtype, device=device)
    gz = torch.arange(nz, dtype=dtype, device=device)
    x, y, z = torch.meshgrid(gx, gy, gz, indexing="ij")
    wx = (x + 0.5) / (nx / 8.0) - 4.0
    wy = (y + 0.5) / (ny / 4.0) - 2.0
    wz = (z + 0.5) / (nz / 4.0) - 2.0
    cx, cy, cz = center
    return radius - torch.sqrt((wx - cx) ** 2 + (wy - cy) ** 2 + (wz - cz) ** 2)


def porosity_from_sdf(sdf, sharpness=20.0):
    """sigmoid(alpha sdf) (smooth.py:81-115)."""
    return torch.sigmoid(sharpness * sdf)


class _SoftBounce(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, porosity):
        f = op.cuda_contig(f, "f")
        p = op.cuda_contig(porosity, "porosity").to(f.dtype)
        nx, ny, nz = op.pop_dims(f)
        out = torch.empty_like(f)
        op.call("lbm_soft_bounce_back", op.dtype_code(f), op.ptr(f), op.ptr(p), op.ptr(out), nx, ny,
                nz, op.stream())
        ctx.save_for_backward(f, p)
        return out

    @staticmethod
    def backward(ctx, g):
        f, p = ctx.saved_tensors
        g = g.contiguous()
        nx, ny, nz = op.pop_dims(f)
        gf = torch.empty_like(f)
        gp = torch.empty_like(p) if ctx.needs_input_grad[1] else None
        op.call("lbm_soft_bounce_back_vjp", op.dtype_code(f), op.ptr(f), op.ptr(p), op.ptr(g),
                op.ptr(gf), op.ptr(gp), nx, ny, nz, op.stream())
        return gf, gp


def soft_bounce_back(f_collided, porosity):
    """(1 - p) f + p f[opp] (smooth.py:118-155)."""
    return _SoftBounce.apply(f_collided, porosity)


class _SphereGeometry(torch.autograd.Function):
    @staticmethod
    def forward(ctx, radius, nx, ny, nz, center, sharpness, q_mode, porosity_mode, dtype,
                disc_floor, denom_eps):
        s = sphere_struct(center, float(radius), sharpness, "sigmoid", q_mode, "soft", disc_floor,
                          denom_eps)
        solid, q, dq, por = sphere_fields(nx, ny, nz, s, dtype, "cuda", want_dqdr=True,
                                          want_porosity=True)
        if porosity_mode == "hard":
            por = solid.to(dtype)
            dpdr = torch.zeros_like(por)
        else:
            dpdr = sharpness * por * (1.0 - por)
        ctx.save_for_backward(dq, dpdr)
        ctx.mark_non_differentiable(solid)
        return por, solid, q

    @staticmethod
    def backward(ctx, g_por, g_solid, g_q):
        dq, dpdr = ctx.saved_tensors
        g = torch.zeros((), dtype=torch.float64, device=dq.device)
        if g_q is not None:
            g = g + (g_q.double() * dq.double()).sum()
        if g_por is not None:
            g = g + (g_por.double() * dpdr.double()).sum()
        return (g.to(dq.dtype),) + (None,) * 10


def sphere_geometry(nx, ny, nz, radius, q_mode="bouzidi", porosity_mode="soft", sharpness=20.0,
                    center=(0.0, 0.0, 0.0), dtype=torch.float32, disc_floor=1e-10,
                    denom_eps=1e-20):
    """Four-mode differentiable sphere of examples/11_optimisation_v2.py:56-119:
    (porosity, solid, q) with solid = sigmoid(alpha (r - d)) > 0.5, q from the
    ray-sphere root (q_mode "bouzidi") or 0.5 ("halfway"), porosity the sigmoid
    ("soft") or the 0/1 mask ("hard").  ``radius`` may be a tensor with
    requires_grad: q(r) and porosity(r) carry dr gradients."""
    return _SphereGeometry.apply(radius if torch.is_tensor(radius) else torch.tensor(float(radius)),
                                 nx, ny, nz, tuple(center), float(sharpness), q_mode,
                                 porosity_mode, dtype, disc_floor, denom_eps)


def smooth_sphere_geometry(nx, ny, nz, center, radius, sharpness=20.0, dtype=torch.float32):
    """(porosity, solid, q) of the differentiable sphere (smooth.py:158-248)."""
    return sphere_geometry(nx, ny, nz, radius, "bouzidi", "soft", sharpness, center, dtype)
