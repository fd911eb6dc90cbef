"""Solver state, parameters and the step / simulate entry points
(jax_lbm/state.py:33-230) running on the fused sm_103a step kernel.

``step`` applies, in one fused launch per time step, the order of
state.py:129-171: optional Smagorinsky tau, BGK/MRT collision, bounce-back on
solid >= 1 cells, Bouzidi streaming with ``state.q``, Zou-He inlet and outlet,
and the post-boundary stability guard.  Gradients are taken either through
the per-op functions (core/*) composed by the caller, or through the fused
adjoint (``Simulation.cd_and_grad`` / ``lbm_jax_autodiff_gb300.autograd``).
"""

from typing import Any, NamedTuple

import torch

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
            _CACHE.pop(next(iter(_CACHE))).close()
        sim = Simulation(nx, ny, nz, float(params.tau),
                         collision="mrt" if int(params.collision_mode) == 1 else "bgk",
                         storage="fp64" if f.dtype == torch.float64 else "fp32",
                         use_smagorinsky=bool(params.use_smagorinsky),
                         smagorinsky_cs=float(params.smagorinsky_cs),
                         periodic_yz=bool(params.periodic_yz), guard="post", inlet_velocity=vel)
        _CACHE[key] = sim
    return sim


def simulate(state, params, n_steps, checkpoint=True):
    """Run n_steps of ``step`` (state.py:174-230).  ``checkpoint`` is accepted
    for signature compatibility; the fused kernels keep no per-step
    intermediates, so there is nothing to rematerialise in the forward."""
    if not state.f.is_cuda:
        raise TypeError("state.f must be a CUDA tensor")
    sim = _handle(state, params)
    sim.set_mask(state.solid.to(torch.int32).contiguous(),
                 q=state.q.to(state.f.dtype).contiguous())
    sim.set_state(state.f.contiguous())
    sim.run(int(n_steps))
    return LBMState(f=sim.get_state(), solid=state.solid, q=state.q)


def step(state, params):
    """One fused time step (state.py:87-171)."""
    return simulate(state, params, 1)
