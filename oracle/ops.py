"""Per-op restatement of jax_lbm's hot-path functions (torch, CPU).

All arrays use the reference layout: populations (19, nx, ny, nz) C-order,
fields (nx, ny, nz), velocity (3, nx, ny, nz).  Functions are pure and
autograd-differentiable; dtype follows the inputs (float32 or float64).

Reductions over directions are sequential in direction index so that the
oracle's rounding is deterministic.
"""

import torch

from .lattice import CS2, E, OPP, Q, STRESS_SLOTS, Consts, mrt_equilibrium_moments, \
    mrt_forward, mrt_inverse

_DEFAULT = {}


def consts_for(dtype, ref_consts=True):
    key = (dtype, ref_consts)
    if key not in _DEFAULT:
        _DEFAULT[key] = Consts(dtype, ref_consts)
    return _DEFAULT[key]


class _JaxClip(torch.autograd.Function):
    """clip(x, lo, hi) with jax's derivative: lax.max/lax.min pass half the
    cotangent at exact ties (jnp.clip = min(max(x, lo), hi))."""

    @staticmethod
    def forward(ctx, x, lo, hi):
        ctx.save_for_backward(x)
        ctx.lo, ctx.hi = lo, hi
        return torch.clamp(x, lo, hi)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        lo, hi = ctx.lo, ctx.hi
        w = torch.ones_like(x)
        if lo is not None:
            w = torch.where(x < lo, torch.zeros_like(w), torch.where(x == lo, 0.5 * w, w))
        if hi is not None:
            w = torch.where(x > hi, torch.zeros_like(w), torch.where(x == hi, 0.5 * w, w))
        return g * w, None, None


def jclip(x, lo=None, hi=None):
    """jnp.clip / jnp.maximum / jnp.minimum with jax's tie rule for gradients."""
    return _JaxClip.apply(x, lo, hi)


def _seq_sum(terms):
    acc = terms[0]
    for t in terms[1:]:
        acc = acc + t
    return acc


def _signed_sum(f, axis):
    """sum_i e_i[axis] * f_i with nonzero terms in index order."""
    acc = None
    for i in range(Q):
        c = int(E[i, axis])
        if c == 0:
            continue
        if acc is None:
            acc = f[i] if c > 0 else -f[i]
        else:
            acc = acc + f[i] if c > 0 else acc - f[i]
    return acc


def compute_density(f):
    """rho = sum_i f_i (equilibrium.py:22-48)."""
    return _seq_sum([f[i] for i in range(Q)])


def compute_velocity(f, rho):
    """u = sum_i f_i e_i / rho (equilibrium.py:51-87)."""
    return torch.stack([_signed_sum(f, a) / rho for a in range(3)])


def _feq_list(rho, ux, uy, uz, c):
    """Equilibrium per direction (equilibrium.py:90-151, formula :144-149)."""
    usq = ux * ux + uy * uy + uz * uz
    out = []
    for i in range(Q):
        ex, ey, ez = (int(v) for v in E[i])
        eu = None
        for comp, uc in ((ex, ux), (ey, uy), (ez, uz)):
            if comp == 0:
                continue
            t = uc if comp > 0 else -uc
            eu = t if eu is None else eu + t
        if eu is None:
            eu = ux * 0.0
        out.append(c.w_list[i] * rho * (1.0 + eu / CS2 + (eu * eu) / (2.0 * CS2 * CS2)
                                         - usq / (2.0 * CS2)))
    return out


def equilibrium(rho, u, c=None):
    c = c or consts_for(rho.dtype)
    return torch.stack(_feq_list(rho, u[0], u[1], u[2], c))


def bgk(f, tau, c=None):
    """f - (f - f_eq)/tau, tau scalar or per cell (collision.py:46-100)."""
    c = c or consts_for(f.dtype)
    rho = compute_density(f)
    u = compute_velocity(f, rho)
    feq = equilibrium(rho, u, c)
    omega = 1.0 / tau
    if torch.is_tensor(omega) and omega.dim() > 0:
        omega = omega.unsqueeze(0)
    return f - omega * (f - feq)


def mrt(f, tau, c=None):
    """Per-cell MRT collision (collision.py:103-184)."""
    c = c or consts_for(f.dtype)
    rho = compute_density(f)
    u = compute_velocity(f, rho)
    omega = 1.0 / tau
    fl = [f[i] for i in range(Q)]
    m = mrt_forward(fl)
    meq = mrt_equilibrium_moments(rho, u[0], u[1], u[2])
    mstar = []
    for k in range(Q):
        s = omega if k in STRESS_SLOTS else c.rates[k]
        mstar.append(m[k] - s * (m[k] - meq[k]))
    return torch.stack(mrt_inverse(mstar, c.norms))


def smagorinsky_tau(f, tau, cs=0.1, c=None):
    """tau_eff = (tau + sqrt(tau^2 + 18 Cs^2 |Pi_neq| / (rho+1e-10)))/2
    (collision.py:187-270)."""
    c = c or consts_for(f.dtype)
    rho = compute_density(f)
    u = compute_velocity(f, rho)
    feq = equilibrium(rho, u, c)
    fneq = f - feq

    def tens(a, b):
        acc = None
        for i in range(Q):
            w = int(E[i, a] * E[i, b])
            if w == 0:
                continue
            t = fneq[i] if w > 0 else -fneq[i]
            acc = t if acc is None else acc + t
        return acc

    sxx, syy, szz = tens(0, 0), tens(1, 1), tens(2, 2)
    sxy, sxz, syz = tens(0, 1), tens(0, 2), tens(1, 2)
    pi = torch.sqrt(sxx * sxx + syy * syy + szz * szz
                    + 2.0 * (sxy * sxy + sxz * sxz + syz * syz))
    cs2 = cs * cs
    return 0.5 * (tau + torch.sqrt(tau * tau + 18.0 * cs2 * pi / (rho + 1e-10)))


def soft_bounce_back(f, porosity):
    """(1-p) f + p f[opp] (geometry/smooth.py:118-155)."""
    p = porosity.unsqueeze(0)
    return (1.0 - p) * f + p * f[torch.as_tensor(OPP)]


def hard_bounce_back(f, solid):
    """where(solid >= 1, f[opp], f) (state.py:146-149; examples/10:171)."""
    is_solid = (solid >= 1).unsqueeze(0)
    return torch.where(is_solid, f[torch.as_tensor(OPP)], f)


def _fallback_mask(i, shape, periodic_yz, device):
    """Cells whose pull source for direction i is outside the domain.

    x is never periodic (streaming.py:123-131); y/z only when
    periodic_yz=False (streaming.py:134-142).  Such cells keep their own
    post-collision value.
    """
    nx, ny, nz = shape
    ex, ey, ez = (int(v) for v in E[i])
    m = torch.zeros(shape, dtype=torch.bool, device=device)
    if ex == 1:
        m[0] = True
    elif ex == -1:
        m[nx - 1] = True
    if not periodic_yz:
        if ey == 1:
            m[:, 0] = True
        elif ey == -1:
            m[:, ny - 1] = True
        if ez == 1:
            m[:, :, 0] = True
        elif ez == -1:
            m[:, :, nz - 1] = True
    return m


def stream(f, q, periodic_yz=True):
    """Pull streaming with Bouzidi bounce-back (streaming.py:40-185)."""
    shape = tuple(f.shape[1:])
    out = [f[0]]
    for i in range(1, Q):
        ex, ey, ez = (int(v) for v in E[i])
        io = int(OPP[i])
        shifts = [s for s in (ex, ey, ez)]
        dims = [d for d, s in zip((0, 1, 2), shifts) if s != 0]
        sh = [s for s in shifts if s != 0]
        rolled = torch.roll(f[i], shifts=sh, dims=dims)
        fb_mask = _fallback_mask(i, shape, periodic_yz, f.device)
        f_normal = torch.where(fb_mask, f[i], rolled)

        q_o = q[io]
        has_wall = q_o >= 0.0
        inv2q = 1.0 / (2.0 * jclip(q_o, 0.5, 1.0))
        high = inv2q * f[io] + (1.0 - inv2q) * f[i]
        ahead = torch.roll(f[io], shifts=[-s for s in sh], dims=dims)
        twoq = 2.0 * jclip(q_o, 0.0, 0.5)
        low = twoq * f[io] + (1.0 - twoq) * ahead
        bz = torch.where(q_o >= 0.5, high, low)
        out.append(torch.where(has_wall, bz, f_normal))
    return torch.stack(out)


def _as_face(v, like):
    if torch.is_tensor(v):
        return v.to(like.dtype)
    return torch.as_tensor(v, dtype=like.dtype)


def zou_he_inlet(f, velocity, rho_target=None):
    """Zou-He velocity inlet at x=0 (boundary.py:35-124).

    velocity = (ux, uy, uz); each component a scalar or a (ny, nz) face.
    """
    ux = _as_face(velocity[0], f)
    uy = _as_face(velocity[1], f)
    uz = _as_face(velocity[2], f)
    s = [f[i, 0] for i in range(Q)]
    k0 = _seq_sum([s[i] for i in (0, 3, 4, 5, 6, 15, 16, 17, 18)])
    kneg = _seq_sum([s[i] for i in (2, 8, 10, 12, 14)])
    rho_in = (k0 + 2.0 * kneg) / (1.0 - ux) if rho_target is None else rho_target
    c3, c6 = 1.0 / 3.0, 1.0 / 6.0
    new = {
        1: s[2] + c3 * rho_in * ux,
        7: s[10] + c6 * rho_in * (ux + uy),
        9: s[8] + c6 * rho_in * (ux - uy),
        11: s[14] + c6 * rho_in * (ux + uz),
        13: s[12] + c6 * rho_in * (ux - uz),
    }
    face = torch.stack([new.get(i, s[i]) * torch.ones_like(s[i]) for i in range(Q)])
    return torch.cat([face.unsqueeze(1), f[:, 1:]], dim=1)


def zou_he_outlet(f, rho_out=1.0):
    """Zou-He pressure outlet at x=nx-1, u_y=u_z=0 (boundary.py:127-200)."""
    s = [f[i, -1] for i in range(Q)]
    k0 = _seq_sum([s[i] for i in (0, 3, 4, 5, 6, 15, 16, 17, 18)])
    kpos = _seq_sum([s[i] for i in (1, 7, 9, 11, 13)])
    ux = -1.0 + (k0 + 2.0 * kpos) / rho_out
    c3, c6 = 1.0 / 3.0, 1.0 / 6.0
    new = {
        2: s[1] - c3 * rho_out * ux,
        10: s[7] - c6 * rho_out * ux,
        8: s[9] - c6 * rho_out * ux,
        14: s[11] - c6 * rho_out * ux,
        12: s[13] - c6 * rho_out * ux,
    }
    face = torch.stack([new.get(i, s[i]) for i in range(Q)])
    return torch.cat([f[:, :-1], face.unsqueeze(1)], dim=1)


def guard_post(f, c=None):
    """Post-BC stability guard: bad cells -> f_eq(1, 0) (state.py:161-169)."""
    c = c or consts_for(f.dtype)
    rho = compute_density(f)
    u = compute_velocity(f, rho)
    umag = torch.sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2])
    bad = (rho < 0.3) | (rho > 2.0) | (umag > 0.4) | torch.isnan(rho)
    feq = equilibrium(torch.where(bad, torch.ones_like(rho), rho),
                      torch.where(bad.unsqueeze(0), torch.zeros_like(u), u), c)
    return torch.where(bad.unsqueeze(0), feq, f), int(bad.sum())


def guard_pre(f, f_ref):
    """Pre-collision guard: bad cells -> fixed f_eq_ref (examples/10:163-168)."""
    rho = compute_density(f)
    u = compute_velocity(f, rho)
    speed = torch.sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2])
    bad = (rho < 0.3) | (rho > 2.0) | (speed > 0.4) | torch.isnan(rho)
    return torch.where(bad.unsqueeze(0), f_ref, f), int(bad.sum())


def momentum_exchange(f_post, f_streamed, q, accumulate=torch.float64):
    """F = sum_{i>=1} sum_x [q_i(x)>=0] e_i (f*_i(x) + f_opp(i)(x)) (forces.py:37-120).

    Accumulated in ``accumulate`` precision (the reference sums per direction
    in the working precision).
    """
    force = [torch.zeros((), dtype=accumulate) for _ in range(3)]
    for i in range(1, Q):
        io = int(OPP[i])
        tot = torch.where(q[i] >= 0.0, f_post[i] + f_streamed[io],
                          torch.zeros_like(f_post[i])).to(accumulate)
        s = tot.sum()
        for a in range(3):
            if E[i, a] != 0:
                force[a] = force[a] + float(E[i, a]) * s
    return torch.stack(force)


def momentum_exchange_decomposed(f_post, f_streamed, q, c=None):
    """(total, pressure) force pair (forces.py:123-196)."""
    c = c or consts_for(f_post.dtype)
    rho = compute_density(f_post)
    u = compute_velocity(f_post, rho)
    feq = equilibrium(rho, u, c)
    total = momentum_exchange(f_post, f_streamed, q)
    pres = [torch.zeros((), dtype=torch.float64) for _ in range(3)]
    for i in range(1, Q):
        io = int(OPP[i])
        tot = torch.where(q[i] >= 0.0, feq[i] + feq[io],
                          torch.zeros_like(feq[i])).double().sum()
        for a in range(3):
            if E[i, a] != 0:
                pres[a] = pres[a] + float(E[i, a]) * tot
    return total, torch.stack(pres)


def projected_area(solid, axis=0):
    """Number of columns along ``axis`` holding a body cell (forces.py:199-234)."""
    body = solid == 1
    return float(body.any(dim=axis).sum())


def drag_coefficient(force, inlet_velocity, area, rho=1.0):
    """|Fx| / (0.5 rho U^2 A + 1e-10) (forces.py:237-276)."""
    dyn = 0.5 * rho * inlet_velocity * inlet_velocity
    return torch.abs(force[0]) / (dyn * area + 1e-10)
