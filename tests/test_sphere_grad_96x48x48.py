"""Shape gradient of the 96x48x48 sphere and the reference's alpha sweep.

dCd/dr through 2000 MRT steps at 96x48x48 with Bouzidi ray-sphere
q(r), r = 0.5 world (6 cells) centred at cell (24, 24, 24), Re 100, for the
hard sphere and the sigmoid-soft sphere (alpha 20):
  - FP32 result identical to the bit for segment lengths K = 50, 100, 200
    and the automatic plan;
  - FP32 within 1e-4 (Cd) and 1e-3 (dCd/dr) of the FP64-storage solver;
  - FP64 adjoint within 1e-3 of central differences with dr = 1e-3 on the
    FP64 GPU forward, and within 1e-6 at dr = 1e-5 (the O(dr^2) error of the
    difference quotient shrinking);
  - on a 100-step window at the full grid, the FP64 adjoint against FP64
    autograd through the oracle (tests/golden/sphere_grad_96x48x48.json,
    made by tests/golden/make_golden.py sphere_grad_96x48x48), to 1e-8.

Alpha sweep: examples/12_sharpness_sensitivity.py:107-132 -- 96x48x48,
Re 50, 2880 MRT steps, smooth sphere (sigmoid porosity, ray-sphere q),
alpha in {5, 10, 20, 40, 80}.  The reference published Cd and the AD
gradient of an A100 FP32 run (paper/make_convergence_figures.py:86-89).
Checked here:
  - FP32 within 1e-4 (Cd) and 1e-3 (dCd/dr) of FP64 storage: ten times the
    largest FP32-vs-FP64 spread this solver shows on these runs (1.5e-5 and
    1.2e-4);
  - FP64 adjoint within 1e-4 of central differences (dr = 1e-4);
  - the published Cd and |dCd/dr| within 2 %.  The published run differs
    from this solver's FP64 result by up to 1.5 %, about a hundred times the
    FP32-vs-FP64 spread here, so the gap is the published run's own
    arithmetic, not FP32 rounding of this path; the bar is that gap with a
    margin.
"""

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.dirname(os.path.abspath(__file__)) + "/golden"

NX, NY, NZ = 96, 48, 48
TAU3 = 3.0 * 0.006 + 0.5                     # Re 100 on D = 12 cells
CENTER3 = (-2.0, 0.0, 0.0)                   # cell (24, 24, 24)
MODES3 = {
    "hard": dict(kind="sigmoid", q_mode="bouzidi", porosity="hard", sharpness=20.0),
    "soft20": dict(kind="sigmoid", q_mode="bouzidi", porosity="soft", sharpness=20.0),
}

# paper/make_convergence_figures.py:86-89 (A100, FP32): alpha -> (Cd, |dCd/dr| AD)
PUBLISHED_SWEEP = {5.0: (3.7555, 15.1634), 10.0: (1.3538, 3.6649), 20.0: (0.8745, 1.8524),
                   40.0: (0.3283, 9.4889), 80.0: (0.5414, 2.4426)}
TAU12 = float(np.float32(3.0 * (0.05 * 12.0 / 50.0) + 0.5))   # jnp.float32 as examples/12


def _sim(storage, tau, radius, center, sph):
    from lbm_jax_autodiff_gb300 import Simulation
    s = Simulation(NX, NY, NZ, tau, collision="mrt", storage=storage, periodic_yz=True,
                   guard="off", inlet_velocity=(0.05, 0.0, 0.0))
    s.set_sphere(radius, center=center, **sph)
    s.set_state(s.equilibrium_state())
    return s


def _grad(storage, tau, center, sph, n, K=0, radius=0.5):
    s = _sim(storage, tau, radius, center, sph)
    try:
        return s.cd_and_grad(n, checkpoint_every=K)
    finally:
        s.close()


def _cd(storage, tau, center, sph, n, radius):
    s = _sim(storage, tau, radius, center, sph)
    try:
        return float(s.run(n, sample_every=n)[0, 3])
    finally:
        s.close()


def _fd(tau, center, sph, n, h, radius=0.5):
    return (_cd("fp64", tau, center, sph, n, radius + h) -
            _cd("fp64", tau, center, sph, n, radius - h)) / (2.0 * h)


@pytest.mark.parametrize("mode", sorted(MODES3))
def test_sphere_gradient_2000_steps(cuda, mode):
    sph = MODES3[mode]
    base = _grad("fp32", TAU3, CENTER3, sph, 2000, K=50)
    for K in (100, 200, 0):
        assert _grad("fp32", TAU3, CENTER3, sph, 2000, K=K) == base, K
    cd32, g32 = base
    cd64, g64 = _grad("fp64", TAU3, CENTER3, sph, 2000, K=100)
    assert abs(cd32 - cd64) <= 1e-4 * abs(cd64), (cd32, cd64)
    assert abs(g32 - g64) <= 1e-3 * abs(g64), (g32, g64)
    fd3 = _fd(TAU3, CENTER3, sph, 2000, 1e-3)
    assert abs(fd3 - g64) <= 1e-3 * abs(g64), (fd3, g64)
    fd5 = _fd(TAU3, CENTER3, sph, 2000, 1e-5)
    assert abs(fd5 - g64) <= 1e-6 * abs(g64), (fd5, g64)


@pytest.mark.parametrize("mode", sorted(MODES3))
def test_sphere_grad_vs_oracle_autograd(cuda, mode):
    with open(os.path.join(GOLDEN, "sphere_grad_96x48x48.json")) as fh:
        gold = json.load(fh)
    ref = gold[mode]
    n = gold["steps"]
    cd64, g64 = _grad("fp64", TAU3, CENTER3, MODES3[mode], n, K=25)
    assert abs(cd64 - ref["cd"]) <= 1e-10 * abs(ref["cd"]), (cd64, ref["cd"])
    assert abs(g64 - ref["dcd_dr"]) <= 1e-8 * abs(ref["dcd_dr"]), (g64, ref["dcd_dr"])
    cd32, g32 = _grad("fp32", TAU3, CENTER3, MODES3[mode], n, K=25)
    assert abs(cd32 - ref["cd"]) <= 1e-4 * abs(ref["cd"]), (cd32, ref["cd"])
    assert abs(g32 - ref["dcd_dr"]) <= 1e-3 * abs(ref["dcd_dr"]), (g32, ref["dcd_dr"])


@pytest.mark.parametrize("alpha", sorted(PUBLISHED_SWEEP))
def test_alpha_sweep_examples12(cuda, alpha):
    sph = dict(kind="sigmoid", q_mode="bouzidi", porosity="soft", sharpness=alpha)
    center = (0.0, 0.0, 0.0)
    cd32, g32 = _grad("fp32", TAU12, center, sph, 2880)
    cd64, g64 = _grad("fp64", TAU12, center, sph, 2880, K=480)
    assert abs(cd32 - cd64) <= 1e-4 * abs(cd64), (cd32, cd64)
    assert abs(g32 - g64) <= 1e-3 * abs(g64), (g32, g64)
    fd = _fd(TAU12, center, sph, 2880, 1e-4)
    assert abs(fd - g64) <= 1e-4 * abs(g64), (fd, g64)
    cd_pub, g_pub = PUBLISHED_SWEEP[alpha]
    print("alpha %g: Cd %.5f (published %.4f), dCd/dr %.4f (published |.| %.4f)"
          % (alpha, cd32, cd_pub, g32, g_pub))
    assert abs(cd32 - cd_pub) <= 0.02 * cd_pub, (cd32, cd_pub)
    assert abs(abs(g32) - g_pub) <= 0.02 * g_pub, (g32, g_pub)
