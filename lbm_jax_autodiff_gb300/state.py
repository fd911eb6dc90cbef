"""Solver state, parameters and the step / simulate entry points
(jax_lbm/state.py:33-230) running on the fused sm_103a step kernel.

``step`` applies, in one fused launch per time step, the order of
state.py:129-171: optional Smagorinsky tau, BGK/MRT collision, bounce-back on
solid >= 1 cells, Bouzidi streaming with ``state.q``, Zou-He inlet and outlet,
and the post-boundary stability guard.

``simulate`` is differentiable like the reference's (jax.grad through its
``fori_loop``, state.py:174-230): when ``state.f`` or ``state.q`` requires
grad, the result carries a torch autograd node whose backward runs the
hand-written adjoint kernels (lbm_vjp_run: forward with checkpoints,
recompute, adjoint) and returns the cotangents of f and q.  The guard is not
differentiated: a backward through steps in which it reset cells raises.

Each solver handle keeps its geometry between calls: ``set_mask`` runs again
only when ``state.solid`` or ``state.q`` is another tensor or was modified
in place (its version counter moved).  A call whose ``state.f`` is the
unmodified tensor the previous call returned continues from the handle's own
state instead of copying f in again.  A call writes the f it returns and
advances the handle one step further in the same launch
(``get_state_and_step``), so a loop of ``step`` calls reads the state once
per step.
"""

import ctypes
import weakref
from typing import Any, NamedTuple

import torch

from . import _native as nat
from .solver import Simulation


class LBMState(NamedTuple):
    """f (19, nx, ny, nz); solid (nx, ny, nz) int32 (0 fluid, 1 body, 2 ground);
    q (19, nx, ny, nz) Bouzidi distances, -1 where there is no wall (state.py:33-54)."""
    f: torch.Tensor
    solid: torch.Tensor
    q: torch.Tensor


class LBMParams(NamedTuple):
    """Physical parameters (state.py:57-84)."""
    tau: Any
    inlet_velocity: Any
    collision_mode: int = 0          # 0 BGK, 1 MRT
    use_smagorinsky: int = 0
    smagorinsky_cs: float = 0.1
    periodic_yz: bool = True


_CACHE = {}


def _handle(state, params):
    f = state.f
    nx, ny, nz = int(f.shape[1]), int(f.shape[2]), int(f.shape[3])
    vel = tuple(float(v) for v in torch.as_tensor(params.inlet_velocity).reshape(-1).tolist())
    key = (nx, ny, nz, f.dtype, float(params.tau), vel, int(params.collision_mode),
           int(params.use_smagorinsky), float(params.smagorinsky_cs), bool(params.periodic_yz),
           torch.cuda.current_device())
    sim = _CACHE.get(key)
    if sim is None:
        if len(_CACHE) >= 8:
            # dropped, not closed: an autograd graph may still hold it for its
            # backward; it is destroyed with its last reference
            _CACHE.pop(next(iter(_CACHE)))
        sim = Simulation(nx, ny, nz, float(params.tau),
                         collision="mrt" if int(params.collision_mode) == 1 else "bgk",
                         storage="fp64" if f.dtype == torch.float64 else "fp32",
                         use_smagorinsky=bool(params.use_smagorinsky),
                         smagorinsky_cs=float(params.smagorinsky_cs),
                         periodic_yz=bool(params.periodic_yz), guard="post", inlet_velocity=vel)
        sim._geom_key = None
        sim._geom_ref = None
        sim._f_out = None
        sim._ahead = False                 # the handle is one step past the f returned
        _CACHE[key] = sim
    return sim


def clear_handles():
    """Drop the solver handles step / simulate keep per parameter set; each is
    destroyed, with its device memory, when its last reference goes (an
    autograd graph awaiting its backward keeps its own)."""
    _CACHE.clear()


def _set_geometry(sim, solid, q):
    """set_mask unless solid and q are the tensors of the last call, unmodified.
    The handle keeps references to them, so their storage cannot be reused by
    other tensors while the key is held."""
    key = (id(solid), solid.data_ptr(), solid._version, id(q), q.data_ptr(), q._version)
    if sim._geom_key == key:
        return
    sim.set_mask(solid.detach().to(torch.int32).contiguous(),
                 q=q.detach().to(sim.dtype).contiguous())
    sim._geom_key = key
    sim._geom_ref = (solid, q)
    sim._f_out = None


def _run(sim, f0, n_steps, continue_from=False):
    """n_steps from f0, or from the handle's own state when f0 is the
    unmodified tensor the handle returned last; returns a new f tensor.  The
    handle ends one step past the returned f (its pull of the next step
    wrote it), so a continuing call has one step fewer to run."""
    last = sim._f_out
    same = (continue_from and last is not None and last[0]() is f0 and
            last[1] == f0._version)
    if not same:
        sim.set_state(f0.detach().contiguous())
        sim._ahead = False
    m = int(n_steps) - (1 if sim._ahead else 0)
    if m < 0:                              # n_steps == 0 on a handle already past f0
        return f0
    if m:
        sim.run(m)
    f = sim.get_state_and_step()
    sim._ahead = True
    sim._f_out = (weakref.ref(f), f._version)
    return f


class _SimulateFn(torch.autograd.Function):
    """f_N = simulate(f_0, q); backward: lbm_vjp_run for (g f_0, g q)."""

    @staticmethod
    def forward(ctx, f0, q, sim, solid, n_steps):
        _set_geometry(sim, solid, q)
        f = _run(sim, f0, n_steps)
        sim._f_out = None                  # the backward sets f_0 again
        ctx.sim, ctx.n_steps, ctx.solid = sim, int(n_steps), solid
        ctx.save_for_backward(f0, q)
        return f

    @staticmethod
    def backward(ctx, g):
        f0, q = ctx.saved_tensors
        sim = ctx.sim
        _set_geometry(sim, ctx.solid, q)
        sim.set_state(f0.detach().contiguous())
        g = g.contiguous().to(sim.dtype)
        g_f0 = torch.empty_like(g)
        g_q = torch.empty_like(g) if ctx.needs_input_grad[1] else None
        nat.call("lbm_vjp_run", sim._h, ctx.n_steps, 0, ctypes.c_void_p(g.data_ptr()),
                 ctypes.c_void_p(g_f0.data_ptr()),
                 ctypes.c_void_p(g_q.data_ptr() if g_q is not None else None),
                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        sim.release_workspace()
        sim._f_out = None
        g_f0 = g_f0.to(f0.dtype) if ctx.needs_input_grad[0] else None
        if g_q is not None:
            g_q = g_q.to(q.dtype)
        return g_f0, g_q, None, None, None


def simulate(state, params, n_steps, checkpoint=True):
    """Run n_steps of ``step`` (state.py:174-230).  Differentiable with respect
    to ``state.f`` and ``state.q``.  ``checkpoint`` is accepted for signature
    compatibility: the backward always recomputes from checkpoints sized to
    free device memory, as ``jax.checkpoint`` trades memory for recompute."""
    if not state.f.is_cuda:
        raise TypeError("state.f must be a CUDA tensor")
    sim = _handle(state, params)
    if torch.is_grad_enabled() and (state.f.requires_grad or state.q.requires_grad):
        f = _SimulateFn.apply(state.f, state.q, sim, state.solid, int(n_steps))
    else:
        _set_geometry(sim, state.solid, state.q)
        f = _run(sim, state.f, n_steps, continue_from=True)
    return LBMState(f=f, solid=state.solid, q=state.q)


def step(state, params):
    """One fused time step (state.py:87-171)."""
    return simulate(state, params, 1)
