"""torch.autograd entry points of the fused solver.

``cd_of_radius(radius, sim, n_steps)`` is the reference drivers'
simulate_cd(radius) (examples/11:139-165, examples/08:69-93) as one
differentiable op: the forward runs the fused steps from the state set on
``sim``, the backward returns dCd/dr from the hand-written adjoint.
"""

import torch


class _CdOfRadius(torch.autograd.Function):
    @staticmethod
    def forward(ctx, radius, sim, n_steps, checkpoint_every, sphere_kwargs):
        kw = dict(sphere_kwargs)
        sim.set_sphere(float(radius), **kw)
        cd, g = sim.cd_and_grad(int(n_steps), checkpoint_every=int(checkpoint_every))
        ctx.g = g
        return torch.tensor(cd, dtype=torch.float64, device=radius.device)

    @staticmethod
    def backward(ctx, g_cd):
        return (g_cd * ctx.g).to(torch.float64), None, None, None, None


def cd_of_radius(radius, sim, n_steps, checkpoint_every=0, **sphere_kwargs):
    """Cd(r) after n_steps; differentiable in ``radius`` (a 0-d tensor).

    ``sim`` is a ``Simulation`` with its initial state set; ``sphere_kwargs``
    go to ``Simulation.set_sphere`` (center, sharpness, kind, q_mode,
    porosity, ...)."""
    r = radius if torch.is_tensor(radius) else torch.tensor(float(radius), dtype=torch.float64)
    return _CdOfRadius.apply(r, sim, n_steps, checkpoint_every, tuple(sorted(sphere_kwargs.items())))
