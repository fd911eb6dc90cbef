"""The 256x128x128 sphere at the full length of its Cd study (D = 32 cells, Re 100,
MRT, Bouzidi on the dist^2 <= r^2 mask, Zou-He, periodic y/z, pre-collision
guard), 28,000 steps, Cd sampled every 500 steps and averaged over the last
30 % of the samples as examples/10_cd_convergence.py:88-106 does.

  - with Smagorinsky Cs 0.1 (the precision form): FP32, FP16 and BF16 storage
    against FP64 storage, mean Cd within 1e-5, 1e-3 and 1.5e-2 relative
    (measured 1.9e-6, 6.6e-4 and 7.4e-3);
  - without Smagorinsky (the examples/10 run): FP32 mean Cd within half a
    published standard deviation of the published 1.1854 +/- 0.0705
    (paper/make_convergence_figures.py:53-54; measured 0.05 of one).
"""

import pytest
import torch

pytestmark = pytest.mark.gpu

NX, NY, NZ = 256, 128, 128
U = 0.05
TAU = 3.0 * U * 32.0 / 100.0 + 0.5
STEPS, EVERY = 28000, 500


def _mean_cd(storage, smagorinsky):
    from lbm_jax_autodiff_gb300 import Simulation
    sim = Simulation(NX, NY, NZ, TAU, collision="mrt", storage=storage,
                     use_smagorinsky=smagorinsky, smagorinsky_cs=0.1, periodic_yz=True,
                     guard="pre", inlet_velocity=(U, 0.0, 0.0))
    try:
        sim.set_sphere(0.5, center=(0.0, 0.0, 0.0), kind="dist", q_mode="bouzidi",
                       porosity="hard")
        sim.set_state(sim.equilibrium_state())
        cd = sim.run(STEPS, sample_every=EVERY)[:, 3].double().cpu()
    finally:
        sim.close()
    assert torch.isfinite(cd).all()
    tail = cd[-max(3, int(cd.numel() * 0.3)):]
    return float(tail.mean())


def test_precision_form_28k_steps(cuda):
    ref = _mean_cd("fp64", True)
    for storage, tol in (("fp32", 1e-5), ("fp16", 1e-3), ("bf16", 1.5e-2)):
        got = _mean_cd(storage, True)
        print("%s: mean Cd %.6f, FP64 %.6f, rel %.2e" % (storage, got, ref, abs(got - ref) / ref))
        assert abs(got - ref) <= tol * abs(ref), (storage, got, ref)


def test_examples10_28k_steps_vs_published(cuda):
    got = _mean_cd("fp32", False)
    print("mean Cd %.5f against the published 1.1854 +/- 0.0705" % got)
    assert abs(got - 1.1854) <= 0.5 * 0.0705, got
