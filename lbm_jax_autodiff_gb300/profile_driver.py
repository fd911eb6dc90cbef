"""Small fixed workload for profiling the fused kernels under ncu.

    python -m lbm_jax_autodiff_gb300.profile_driver NXxNYxNZ STORAGE STEPS [grad]
    python -m lbm_jax_autodiff_gb300.profile_driver batch COUNT STEPS

Builds the bench step (MRT + Smagorinsky Cs=0.1, pre-collision guard,
dist-mask Bouzidi sphere r = 0.5 world at the domain centre, Re = 100 for
D = nx/8) and runs STEPS fused steps; with ``grad`` it also evaluates one
dCd/dr over STEPS steps (forward, recompute and adjoint kernels).  ``batch``
evaluates the batched gradient (no graph) of the first COUNT instances of
the batched workload's draw over STEPS steps, checkpoint interval STEPS / 2.
"""

import sys

import torch

from .solver import Simulation


def batch_main(count, steps):
    from .batch import Batch, config5_instances
    inst, sph = config5_instances(count)
    b = Batch(inst)
    b.set_spheres(sph)
    b.set_equilibrium()
    cd, g = b.cd_and_grad(steps, checkpoint_every=max(1, steps // 2), use_graph=False)
    torch.cuda.synchronize()
    print("ok cells", b.cells, "cd[:2]", cd[:2], "g[:2]", g[:2])
    b.close()


def main(argv):
    if argv and argv[0] == "batch":
        batch_main(int(argv[1]) if len(argv) > 1 else 16, int(argv[2]) if len(argv) > 2 else 8)
        return
    nx, ny, nz = [int(v) for v in argv[0].split("x")] if argv else (192, 96, 96)
    storage = argv[1] if len(argv) > 1 else "fp32"
    steps = int(argv[2]) if len(argv) > 2 else 8
    grad = len(argv) > 3 and argv[3] == "grad"
    U = 0.05
    tau = 3 * U * (nx / 8.0) / 100.0 + 0.5
    sim = Simulation(nx, ny, nz, tau, collision="mrt", storage=storage, use_smagorinsky=True,
                     smagorinsky_cs=0.1, guard="off" if grad else "pre", inlet_velocity=(U, 0, 0))
    sim.set_sphere(0.5, kind="dist", q_mode="bouzidi", porosity="hard")
    sim.set_state(sim.equilibrium_state())
    if grad:
        cd, g = sim.cd_and_grad(steps, checkpoint_every=max(1, steps // 4))
        print("cd", cd, "dcd_dr", g)
    else:
        sim.run(steps)
    torch.cuda.synchronize()
    print("ok", sim.link_count)


if __name__ == "__main__":
    main(sys.argv[1:])
