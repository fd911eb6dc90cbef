"""Zou-He velocity inlet and pressure outlet (jax_lbm/core/boundary.py:35-200)
on the sm_103a kernels, differentiable in f, the inlet velocity and rho_out."""

import ctypes

import torch

from .. import _ops as op


def _velocity_args(velocity, f):
    """(u_face tensor (3, ny, nz) or None, host triple or None, requires-grad inputs)."""
    comps = [velocity[k] for k in range(3)]
    any_face = any(torch.is_tensor(c) and c.dim() > 0 for c in comps)
    ny, nz = int(f.shape[2]), int(f.shape[3])
    if any_face:
        face = torch.stack([c.to(f.device, f.dtype).expand(ny, nz) if torch.is_tensor(c)
                            else torch.full((ny, nz), float(c), dtype=f.dtype, device=f.device)
                            for c in comps]).contiguous()
        return face, None
    return None, (ctypes.c_double * 3)(*[float(c.detach()) if torch.is_tensor(c) else float(c)
                                          for c in comps])


class _Inlet(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, u_face, vel_vals, rho_target):
        f = op.cuda_contig(f, "f")
        nx, ny, nz = op.pop_dims(f)
        vel = (ctypes.c_double * 3)(*vel_vals) if vel_vals is not None else None
        has_rt = rho_target is not None
        out = torch.empty_like(f)
        op.call("lbm_zou_he_inlet", op.dtype_code(f), op.ptr(f), op.ptr(u_face), vel, int(has_rt),
                float(rho_target) if has_rt else 0.0, op.ptr(out), nx, ny, nz, op.stream())
        ctx.save_for_backward(f, u_face if u_face is not None else torch.empty(0, device=f.device))
        ctx.vel_vals, ctx.rt, ctx.has_face = vel_vals, rho_target, u_face is not None
        return out

    @staticmethod
    def backward(ctx, g):
        f, uf = ctx.saved_tensors
        uf = uf if ctx.has_face else None
        g = g.contiguous()
        nx, ny, nz = op.pop_dims(f)
        gf = torch.empty_like(f)
        gu = torch.empty((3, ny, nz), dtype=f.dtype, device=f.device)
        vel = (ctypes.c_double * 3)(*ctx.vel_vals) if ctx.vel_vals is not None else None
        has_rt = ctx.rt is not None
        op.call("lbm_zou_he_inlet_vjp", op.dtype_code(f), op.ptr(f), op.ptr(uf), vel, int(has_rt),
                float(ctx.rt) if has_rt else 0.0, op.ptr(g), op.ptr(gf), op.ptr(gu), nx, ny, nz,
                op.stream())
        return gf, (gu if ctx.has_face else None), None, None


def zou_he_inlet(f, velocity, rho_target=None):
    """Zou-He velocity inlet on the x = 0 face (boundary.py:35-124).  Each of
    velocity[0..2] may be a scalar or a (ny, nz) face (broadcasting as in the
    reference); gradients flow to f and to tensor velocity components."""
    face, trip = _velocity_args(velocity, f)
    if face is not None:
        return _Inlet.apply(f, face, None, rho_target)
    comps = [velocity[k] for k in range(3)]
    needs = any(torch.is_tensor(c) and c.requires_grad for c in comps)
    if needs:
        # route scalar tensors through a (3, ny, nz) face to carry their gradient
        ny, nz = int(f.shape[2]), int(f.shape[3])
        face = torch.stack([(c if torch.is_tensor(c) else torch.tensor(float(c)))
                            .to(f.device, f.dtype).expand(ny, nz) for c in comps]).contiguous()
        return _Inlet.apply(f, face, None, rho_target)
    return _Inlet.apply(f, None, tuple(float(c.detach()) if torch.is_tensor(c) else float(c)
                                       for c in comps), rho_target)


class _Outlet(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, rho_out):
        f = op.cuda_contig(f, "f")
        nx, ny, nz = op.pop_dims(f)
        out = torch.empty_like(f)
        op.call("lbm_zou_he_outlet", op.dtype_code(f), op.ptr(f), float(rho_out), op.ptr(out),
                nx, ny, nz, op.stream())
        ctx.save_for_backward(f)
        ctx.rho_out = float(rho_out)
        ctx.rho_is_tensor = torch.is_tensor(rho_out)
        return out

    @staticmethod
    def backward(ctx, g):
        (f,) = ctx.saved_tensors
        g = g.contiguous()
        nx, ny, nz = op.pop_dims(f)
        gf = torch.empty_like(f)
        want = ctx.rho_is_tensor and ctx.needs_input_grad[1]
        gr = torch.empty((ny, nz), dtype=f.dtype, device=f.device) if want else None
        op.call("lbm_zou_he_outlet_vjp", op.dtype_code(f), op.ptr(f), ctx.rho_out, op.ptr(g),
                op.ptr(gf), op.ptr(gr), nx, ny, nz, op.stream())
        return gf, (gr.sum() if want else None)


def zou_he_outlet(f, rho_out=1.0):
    """Zou-He pressure outlet on the x = nx-1 face, u_y = u_z = 0 (boundary.py:127-200)."""
    return _Outlet.apply(f, rho_out)
