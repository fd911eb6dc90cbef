"""Step orders of the reference drivers, restated on the CPU oracle.

One time step (state.py:129-171 and the examples' step_fn bodies):
  [pre-collision guard (examples/10:163-168)]
  [Smagorinsky tau from pre-collision f (state.py:134-135)]
  collide: BGK or MRT
  solid: hard where(solid, f[opp], f) (state.py:146-149) or soft blend
         (smooth.py:151-155); this is f_post
  stream with Bouzidi (streaming.py:40-185)
  Zou-He inlet, Zou-He outlet (boundary.py)
  [post-BC guard (state.py:161-169)]
The drag is momentum_exchange(f_post_last, f_final, q) (examples/11:162-165).
"""

from dataclasses import dataclass
from typing import Any, Optional

import torch

from . import ops
from .lattice import Q


@dataclass
class StepConfig:
    tau: Any
    inlet: tuple                   # (ux, uy, uz): scalars or (ny, nz) faces
    collision: str = "bgk"         # "bgk" | "mrt"
    smagorinsky_cs: Optional[float] = None
    periodic_yz: bool = True
    guard: str = "off"             # "off" | "pre" | "post"
    rho_out: float = 1.0


def step(f, q, cfg: StepConfig, solid=None, porosity=None, f_ref=None, consts=None):
    """One step; returns (f_next, f_post, guard_resets)."""
    c = consts or ops.consts_for(f.dtype)
    resets = 0
    if cfg.guard == "pre":
        f, resets = ops.guard_pre(f, f_ref)
    tau = cfg.tau
    if cfg.smagorinsky_cs is not None:
        tau = ops.smagorinsky_tau(f, tau, cfg.smagorinsky_cs, c)
    fc = ops.mrt(f, tau, c) if cfg.collision == "mrt" else ops.bgk(f, tau, c)
    if porosity is not None:
        fc = ops.soft_bounce_back(fc, porosity)
    elif solid is not None:
        fc = ops.hard_bounce_back(fc, solid)
    f_post = fc
    fs = ops.stream(fc, q, cfg.periodic_yz)
    fs = ops.zou_he_inlet(fs, cfg.inlet)
    fs = ops.zou_he_outlet(fs, cfg.rho_out)
    if cfg.guard == "post":
        fs, r2 = ops.guard_post(fs, c)
        resets += r2
    return fs, f_post, resets


def run(f, q, cfg, n_steps, solid=None, porosity=None, f_ref=None, consts=None,
        sample_every=None, on_sample=None):
    """n_steps of ``step``; optional callback(step_index, f, f_post)."""
    f_post = f
    total_resets = 0
    for k in range(n_steps):
        f, f_post, r = step(f, q, cfg, solid, porosity, f_ref, consts)
        total_resets += r
        if sample_every and on_sample and (k + 1) % sample_every == 0:
            on_sample(k + 1, f, f_post)
    return f, f_post, total_resets


def initial_state(nx, ny, nz, ux, dtype=torch.float32, consts=None):
    """f_eq(rho=1, u=(ux,0,0)) on the whole grid."""
    rho = torch.ones((nx, ny, nz), dtype=dtype)
    u = torch.zeros((3, nx, ny, nz), dtype=dtype)
    u[0] = ux
    return ops.equilibrium(rho, u, consts or ops.consts_for(dtype))


def channel_walls(nx, ny, nz):
    """Solid rows y=0 and y=ny-1 (tests/test_poiseuille.py:37-44)."""
    solid = torch.zeros((nx, ny, nz), dtype=torch.int32)
    solid[:, 0, :] = 1
    solid[:, ny - 1, :] = 1
    return solid


def parabolic_inlet(ny, nz, u_peak, dtype=torch.float32):
    """u_x(y) = u_peak * 4 s (H - s) / H^2 with s = y - 0.5, H = ny - 2, zero on
    the wall rows; (ny, nz) face."""
    H = float(ny - 2)
    y = torch.arange(ny, dtype=torch.float64)
    s = y - 0.5
    prof = u_peak * 4.0 * s * (H - s) / (H * H)
    prof[0] = 0.0
    prof[ny - 1] = 0.0
    return prof.to(dtype).unsqueeze(1).expand(ny, nz).contiguous()


def cd_from(f_post, f_final, q, u_inlet, area):
    force = ops.momentum_exchange(f_post, f_final, q)
    return ops.drag_coefficient(force, u_inlet, area), force


def cd_of_radius_bgk_f64(radius, nx=32, ny=16, nz=16, n_steps=10, u_inlet=0.05,
                         re=50.0, sharpness=20.0, consts=None):
    """The reference's FP64 Bouzidi gradient setup (tests/test_gradients_f64.py:129-207):
    soft porosity sigmoid(20 (r - d)), ray-sphere q with floors 1e-20/1e-30,
    BGK, periodic y/z, Cd from the final step."""
    from .geometry import ray_sphere_q, world_coords, _link_mask
    dtype = torch.float64
    c = consts or ops.consts_for(dtype, ref_consts=True)
    d_lat = 32 * 0.5 / 4.0
    nu = u_inlet * d_lat / re
    tau = 3.0 * nu + 0.5
    wx, wy, wz = world_coords(nx, ny, nz, dtype)
    dist = torch.sqrt(wx ** 2 + wy ** 2 + wz ** 2)
    porosity = torch.sigmoid(sharpness * (radius - dist))
    solid = (porosity > 0.5).to(torch.int32)
    qs = [-torch.ones((nx, ny, nz), dtype=dtype)]
    for i in range(1, Q):
        link = _link_mask(solid, i)
        qv = ray_sphere_q(wx, wy, wz, (0.0, 0.0, 0.0), radius, i, nx, ny, nz, 1e-20, 1e-30)
        qs.append(torch.where(link, qv, torch.full_like(qv, -1.0)))
    q = torch.stack(qs)
    f = initial_state(nx, ny, nz, u_inlet, dtype, c)
    cfg = StepConfig(tau=tau, inlet=(u_inlet, 0.0, 0.0), collision="bgk")
    f, f_post, _ = run(f, q, cfg, n_steps, porosity=porosity, consts=c)
    area = max(ops.projected_area(solid), 1.0)
    cd, _ = cd_from(f_post, f, q, u_inlet, area)
    return cd


def simulate_cd(radius, nx, ny, nz, n_steps, tau, u_inlet=0.05, q_mode="bouzidi",
                porosity_mode="soft", sharpness=20.0, collision="mrt", smagorinsky_cs=None,
                periodic_yz=True, center=(0.0, 0.0, 0.0), dtype=torch.float32,
                disc_floor=1e-10, a_eps=1e-20, q_leaf=None, consts=None, return_parts=False,
                remat_chunk=None):
    """The reference gradient drivers' simulate_cd (examples/11:139-165,
    examples/08:69-93): build the four-mode sphere from ``radius`` (a tensor
    that may require grad), run n_steps of collide -> porosity blend ->
    stream -> Zou-He, and return Cd from the final step.  ``q_leaf`` replaces
    the q buffer (to differentiate with respect to q directly).

    ``remat_chunk`` = K runs the steps in chunks of K under
    torch.utils.checkpoint, so autograd keeps one state per chunk and
    recomputes a chunk's steps in the backward pass -- the
    ``jax.checkpoint`` chunking of the reference drivers (examples/08:49-66,
    examples/12:_chunked_scan).  The gradient is the same; only the memory
    of a long run at a large grid changes."""
    from .geometry import sphere_geometry
    c = consts or ops.consts_for(dtype)
    por, solid, q = sphere_geometry(nx, ny, nz, radius, q_mode, porosity_mode, sharpness, center,
                                    dtype, disc_floor, a_eps)
    if q_leaf is not None:
        q = q_leaf
    f = initial_state(nx, ny, nz, u_inlet, dtype, c)
    cfg = StepConfig(tau=tau, inlet=(u_inlet, 0.0, 0.0), collision=collision,
                     smagorinsky_cs=smagorinsky_cs, periodic_yz=periodic_yz)
    if remat_chunk:
        from torch.utils.checkpoint import checkpoint

        def chunk(f_in, fp_in, q_in, p_in, k):
            f_out, fp_out, _ = run(f_in, q_in, cfg, k, porosity=p_in, consts=c)
            return f_out, fp_out

        f_post = f
        done = 0
        while done < n_steps:
            k = min(int(remat_chunk), n_steps - done)
            f, f_post = checkpoint(chunk, f, f_post, q, por, k, use_reentrant=False)
            done += k
    else:
        f, f_post, _ = run(f, q, cfg, n_steps, porosity=por, consts=c)
    area = max(ops.projected_area(solid), 1.0)
    cd, _ = cd_from(f_post, f, q, u_inlet, area)
    if return_parts:
        return cd, q, solid, por
    return cd
