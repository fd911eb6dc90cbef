"""Sphere and box geometry (jax_lbm/geometry/primitives.py:26-255) built by
the sm_103a geometry kernels."""

import ctypes

import torch

from .. import _native as nat
from .. import _ops as op


def _grid_to_world(gx, gy, gz, nx, ny, nz):
    """Cell centre -> world coordinates, x in [-4,4], y,z in [-2,2] (primitives.py:26-53)."""
    return ((gx + 0.5) / (nx / 8.0) - 4.0, (gy + 0.5) / (ny / 4.0) - 2.0,
            (gz + 0.5) / (nz / 4.0) - 2.0)


def sphere_struct(center, radius, sharpness=20.0, kind="dist", q_mode="bouzidi",
                  porosity="hard", disc_floor=None, denom_eps=1e-20):
    s = nat.LBMSphereC()
    for k in range(3):
        s.center[k] = float(center[k])
    s.radius = float(radius)
    s.sharpness = float(sharpness)
    s.kind = nat.LBM_SPHERE_SIGMOID_MASK if kind == "sigmoid" else nat.LBM_SPHERE_DIST_MASK
    s.q_mode = nat.LBM_Q_BOUZIDI if q_mode == "bouzidi" else nat.LBM_Q_HALFWAY
    s.porosity = {"none": nat.LBM_POROSITY_NONE, "hard": nat.LBM_POROSITY_HARD,
                  "soft": nat.LBM_POROSITY_SOFT}[porosity]
    s.disc_floor = float(disc_floor if disc_floor is not None else (1e-10 if kind == "sigmoid" else 0.0))
    s.denom_eps = float(denom_eps)
    return s


def sphere_fields(nx, ny, nz, sphere, dtype=torch.float32, device="cuda", want_dqdr=False,
                  want_porosity=False):
    """Dense (solid int32, q, dq/dr or None, porosity or None) from the builder."""
    solid = torch.empty((nx, ny, nz), dtype=torch.int32, device=device)
    q = torch.empty((19, nx, ny, nz), dtype=dtype, device=device)
    dq = torch.empty_like(q) if want_dqdr else None
    por = torch.empty((nx, ny, nz), dtype=dtype, device=device) if want_porosity else None
    probe = torch.empty(0, dtype=dtype)
    op.call("lbm_sphere_fields", op.dtype_code(probe), nx, ny, nz, ctypes.byref(sphere),
            op.ptr(solid), op.ptr(q), op.ptr(dq), op.ptr(por), op.stream())
    return solid, q, dq, por


def create_sphere(nx, ny, nz, center, radius, dtype=torch.float32, device="cuda"):
    """Solid sphere (dist^2 <= r^2) with ray-sphere Bouzidi q clipped to
    [0.01, 0.99], -1 elsewhere (primitives.py:56-174).  Returns (solid, q)."""
    s = sphere_struct(center, radius, kind="dist", q_mode="bouzidi", porosity="hard")
    solid, q, _, _ = sphere_fields(nx, ny, nz, s, dtype, device)
    return solid, q


def create_box(nx, ny, nz, corner_min, corner_max, dtype=torch.float32, device="cuda"):
    """Axis-aligned box with q = 0.5 on its links (primitives.py:177-255)."""
    solid = torch.empty((nx, ny, nz), dtype=torch.int32, device=device)
    q = torch.empty((19, nx, ny, nz), dtype=dtype, device=device)
    lo = (ctypes.c_double * 3)(*[float(v) for v in corner_min])
    hi = (ctypes.c_double * 3)(*[float(v) for v in corner_max])
    probe = torch.empty(0, dtype=dtype)
    op.call("lbm_box_fields", op.dtype_code(probe), nx, ny, nz, lo, hi, op.ptr(solid), op.ptr(q),
            op.stream())
    return solid, q
