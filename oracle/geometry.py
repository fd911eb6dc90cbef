"""Sphere / wall geometry restated for the CPU oracle.

Follows:
  _grid_to_world            geometry/primitives.py:26-53
  create_sphere (hard, q)   geometry/primitives.py:56-174 (ray-sphere :145-172)
  signed_distance_sphere    geometry/smooth.py:34-78
  porosity_from_sdf         geometry/smooth.py:81-115
  smooth_sphere_geometry    geometry/smooth.py:158-248
  four-mode builder         examples/11_optimisation_v2.py:56-119
  compute_q_from_solid      geometry/bouzidi.py:32-106

``radius`` may be a tensor with requires_grad: q(r) and porosity(r) are then
differentiable exactly as in the reference's traced builders.
"""

import torch

from .lattice import E, Q
from .ops import jclip


def world_coords(nx, ny, nz, dtype):
    """Cell-centre world coordinates, x in [-4,4], y,z in [-2,2]."""
    gx = torch.arange(nx, dtype=dtype)
    gy = torch.arange(ny, dtype=dtype)
    gz = torch.arange(nz, dtype=dtype)
    gx3, gy3, gz3 = torch.meshgrid(gx, gy, gz, indexing="ij")
    sx, sy, sz = nx / 8.0, ny / 4.0, nz / 4.0
    return (gx3 + 0.5) / sx - 4.0, (gy3 + 0.5) / sy - 2.0, (gz3 + 0.5) / sz - 2.0


def _link_mask(solid, i):
    """Fluid cells whose in-bounds neighbour along e_i is a body cell."""
    nx, ny, nz = solid.shape
    ex, ey, ez = (int(v) for v in E[i])
    nb = torch.zeros_like(solid)
    xs = slice(max(0, -ex), nx - max(0, ex))
    ys = slice(max(0, -ey), ny - max(0, ey))
    zs = slice(max(0, -ez), nz - max(0, ez))
    xd = slice(xs.start + ex, xs.stop + ex)
    yd = slice(ys.start + ey, ys.stop + ey)
    zd = slice(zs.start + ez, zs.stop + ez)
    nb[xs, ys, zs] = solid[xd, yd, zd]
    return (solid == 0) & (nb == 1)


def ray_sphere_q(wx, wy, wz, center, radius, i, nx, ny, nz,
                 disc_floor=0.0, a_eps=1e-20):
    """Fraction t along link i where the ray from the cell centre meets the
    sphere; 0.5 when there is no hit in (0, 1]; clipped to [0.01, 0.99]."""
    cx, cy, cz = center
    ex, ey, ez = (int(v) for v in E[i])
    rdx, rdy, rdz = ex / (nx / 8.0), ey / (ny / 4.0), ez / (nz / 4.0)
    ox, oy, oz = wx - cx, wy - cy, wz - cz
    a = rdx * rdx + rdy * rdy + rdz * rdz
    b = 2.0 * (ox * rdx + oy * rdy + oz * rdz)
    c = ox * ox + oy * oy + oz * oz - radius * radius
    disc = b * b - 4.0 * a * c
    sq = torch.sqrt(jclip(disc, lo=disc_floor))
    t = (-b - sq) / (2.0 * a + a_eps)
    valid = (disc >= 0.0) & (t > 0.0) & (t <= 1.0)
    qv = torch.where(valid, t, torch.full_like(t, 0.5))
    return jclip(qv, 0.01, 0.99)


def create_sphere(nx, ny, nz, center, radius, dtype=torch.float32):
    """Hard sphere mask (dist^2 <= r^2) and ray-sphere q (primitives.py:56-174)."""
    wx, wy, wz = world_coords(nx, ny, nz, dtype)
    cx, cy, cz = center
    d2 = (wx - cx) ** 2 + (wy - cy) ** 2 + (wz - cz) ** 2
    solid = (d2 <= radius * radius).to(torch.int32)
    q = -torch.ones((Q, nx, ny, nz), dtype=dtype)
    qs = [q[0]]
    for i in range(1, Q):
        link = _link_mask(solid, i)
        qv = ray_sphere_q(wx, wy, wz, center, radius, i, nx, ny, nz, 0.0, 1e-20)
        qs.append(torch.where(link, qv, torch.full_like(qv, -1.0)))
    return solid, torch.stack(qs)


def signed_distance_sphere(nx, ny, nz, center, radius, dtype=torch.float32):
    """r - |x - c| (smooth.py:34-78)."""
    wx, wy, wz = world_coords(nx, ny, nz, dtype)
    cx, cy, cz = center
    dist = torch.sqrt((wx - cx) ** 2 + (wy - cy) ** 2 + (wz - cz) ** 2)
    return radius - dist


def porosity_from_sdf(sdf, sharpness=20.0):
    """sigmoid(alpha * sdf) (smooth.py:81-115)."""
    return torch.sigmoid(sharpness * sdf)


def sphere_geometry(nx, ny, nz, radius, q_mode="bouzidi", porosity_mode="soft",
                    sharpness=20.0, center=(0.0, 0.0, 0.0), dtype=torch.float32,
                    disc_floor=1e-10, a_eps=1e-20):
    """Four-mode differentiable sphere (examples/11_optimisation_v2.py:56-119).

    q_mode in {bouzidi, halfway}; porosity_mode in {soft, hard}.  The hard
    solid is porosity_soft > 0.5 in both porosity modes.  With
    q_mode='bouzidi', porosity_mode='soft' this is smooth_sphere_geometry
    (smooth.py:158-248).  Returns (porosity, solid, q).
    """
    sdf = signed_distance_sphere(nx, ny, nz, center, radius, dtype)
    p_soft = porosity_from_sdf(sdf, sharpness)
    solid = (p_soft > 0.5).to(torch.int32)
    porosity = solid.to(dtype) if porosity_mode == "hard" else p_soft
    wx, wy, wz = world_coords(nx, ny, nz, dtype)
    qs = [-torch.ones((nx, ny, nz), dtype=dtype)]
    for i in range(1, Q):
        link = _link_mask(solid, i)
        if q_mode == "bouzidi":
            qv = ray_sphere_q(wx, wy, wz, center, radius, i, nx, ny, nz, disc_floor, a_eps)
        else:
            qv = torch.full((nx, ny, nz), 0.5, dtype=dtype)
        qs.append(torch.where(link, qv, torch.full_like(qv, -1.0)))
    return porosity, solid, torch.stack(qs)


def compute_q_from_solid(solid, default_q=0.5, dtype=torch.float32):
    """q = default_q on fluid->body in-bounds links, -1 elsewhere (bouzidi.py:32-106)."""
    nx, ny, nz = solid.shape
    qs = [-torch.ones((nx, ny, nz), dtype=dtype)]
    for i in range(1, Q):
        link = _link_mask(solid, i)
        qs.append(torch.where(link, torch.full((nx, ny, nz), default_q, dtype=dtype),
                              torch.full((nx, ny, nz), -1.0, dtype=dtype)))
    return torch.stack(qs)
