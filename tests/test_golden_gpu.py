"""Full-length configurations against the committed oracle fixtures
(tests/golden/, produced by tests/golden/make_golden.py) and the reference's
published numbers."""

import json
import os

import numpy as np
import pytest
import torch

from oracle import drivers, geometry

pytestmark = pytest.mark.gpu
GOLDEN = os.path.dirname(os.path.abspath(__file__)) + "/golden"


def _load(name):
    with open(os.path.join(GOLDEN, name + ".json")) as fh:
        return json.load(fh)


def _u(f):
    rho = f.sum(dim=0)
    e = torch.tensor([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1],
                      [0, 0, -1], [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1],
                      [-1, 0, 1], [1, 0, -1], [-1, 0, -1], [0, 1, 1], [0, -1, 1], [0, 1, -1],
                      [0, -1, -1]], dtype=f.dtype, device=f.device)
    return torch.einsum("ixyz,ia->axyz", f, e) / rho


def test_channel_64x21x8_3000_steps(cuda):
    """64x21x8 BGK channel, parabolic inlet, tau 0.8, 3000 steps: whole u field
    within 1e-5 of the FP32 oracle; L2 error vs the parabola as the oracle."""
    from lbm_jax_autodiff_gb300 import Simulation
    d = _load("channel_64x21x8")
    nx, ny, nz = d["grid"]
    prof = drivers.parabolic_inlet(ny, nz, 0.05)
    sim = Simulation(nx, ny, nz, 0.8, collision="bgk", inlet_velocity=(0.05, 0.0, 0.0))
    sim.set_mask(drivers.channel_walls(nx, ny, nz).cuda())
    face = torch.stack([prof, torch.zeros_like(prof), torch.zeros_like(prof)]).contiguous()
    sim.set_inlet_profile(face.cuda())
    sim.set_state(drivers.initial_state(nx, ny, nz, 0.0).cuda())
    sim.run(d["steps"])
    u = _u(sim.get_state().double()).cpu().numpy()
    ref = np.load(os.path.join(GOLDEN, "channel_64x21x8.npz"))["u"].astype(np.float64)
    assert np.abs(u - ref).max() <= 1e-5
    prof_gpu = u[0, nx // 2].mean(axis=-1)
    assert np.abs(prof_gpu - np.array(d["profile_ux"])).max() <= 1e-6


@pytest.mark.parametrize("name,periodic", [("sphere_96x48x48_periodic", True),
                                           ("sphere_96x48x48", False)])
def test_sphere_96x48x48_2000_steps(cuda, name, periodic):
    """96x48x48 MRT Bouzidi sphere, Re 100, 2000 steps, Cd sampled every step
    over the last 30% (examples/10 step order, pre-collision guard)."""
    from lbm_jax_autodiff_gb300 import Simulation
    if not os.path.exists(os.path.join(GOLDEN, name + ".json")):
        pytest.skip("fixture missing")
    d = _load(name)
    nx, ny, nz = d["grid"]
    sim = Simulation(nx, ny, nz, d["tau"], collision="mrt", guard="pre", periodic_yz=periodic,
                     inlet_velocity=(d["U"], 0.0, 0.0))
    sim.set_sphere(0.5, center=tuple(d["center"]), kind="dist", q_mode="bouzidi", porosity="hard")
    assert sim.projected_area == d["area"]
    assert sim.link_count[0] == d["links"]
    sim.set_state(drivers.initial_state(nx, ny, nz, d["U"]).cuda())
    start = d["cd_window"][0] - 1
    sim.run(start)
    s = sim.run(d["steps"] - start, sample_every=1)
    cd = s[:, 3].cpu().numpy()
    u = _u(sim.get_state().double())[:, ::2, ::2, ::2].cpu().numpy()
    ref = np.load(os.path.join(GOLDEN, name + ".npz"))["u_sub"].astype(np.float64)
    du = np.abs(u - ref).max()
    rel = abs(cd.mean() - d["cd_mean"]) / abs(d["cd_mean"])
    print("%s: max|du| %.2e, Cd mean %.6f (oracle %.6f, rel %.2e)" % (name, du, cd.mean(),
                                                                     d["cd_mean"], rel))
    if periodic:
        assert du <= 1e-5
        assert rel <= 1e-4
    else:
        # the clamped 'free-slip' sides (streaming.py:134-142) make this flow
        # unsteady within the first flow-through time (Cd swings between ~0
        # and ~12); two FP32 trajectories separate, so only the window
        # statistics are compared here and the field is checked on a short
        # horizon in test_sphere_96x48x48_freeslip_short_horizon
        assert abs(cd.mean() - d["cd_mean"]) <= d["cd_std"]


def test_sphere_96x48x48_freeslip_short_horizon(cuda):
    """The free-slip 96x48x48 sphere for 300 steps: the whole u field within 1e-5 of the
    oracle before the unsteadiness amplifies rounding differences."""
    from lbm_jax_autodiff_gb300 import Simulation
    from oracle import ops
    nx, ny, nz, n, U = 96, 48, 48, 300, 0.05
    tau = 3 * 0.006 + 0.5
    solid, q = geometry.create_sphere(nx, ny, nz, (-2.0, 0.0, 0.0), 0.5)
    f0 = drivers.initial_state(nx, ny, nz, U)
    cfg = drivers.StepConfig(tau=tau, inlet=(U, 0.0, 0.0), collision="mrt", periodic_yz=False,
                             guard="pre")
    with torch.no_grad():
        f_or, _, _ = drivers.run(f0, q, cfg, n, solid=solid, f_ref=f0)
    sim = Simulation(nx, ny, nz, tau, collision="mrt", guard="pre", periodic_yz=False,
                     inlet_velocity=(U, 0.0, 0.0))
    sim.set_sphere(0.5, center=(-2.0, 0.0, 0.0), kind="dist", q_mode="bouzidi", porosity="hard")
    sim.set_state(f0.cuda())
    sim.run(n)
    u_g = _u(sim.get_state().double()).cpu()
    u_o = ops.compute_velocity(f_or.double(), ops.compute_density(f_or.double()))
    assert (u_g - u_o).abs().max().item() <= 1e-5


def test_sphere_96x48x48_freeslip_fp64_2000_steps(cuda):
    """The free-slip 96x48x48 sphere as written (clamped y / z edges) in FP64
    storage against the FP64 oracle (sphere_96x48x48_freeslip_fp64.json), Cd
    every 100 steps.  Measured: the two FP64 trajectories agree to ~5e-14
    through step 400 and 4e-11 at step 500; from there the difference grows
    about 5000-fold per 100 steps (the flow is chaotic) and reaches O(1) by
    step 800.  So Cd is held to 1e-12 through step 400 and 1e-9 at step 500;
    later samples, in any arithmetic, are comparable only as window
    statistics (test_sphere_96x48x48_2000_steps)."""
    from lbm_jax_autodiff_gb300 import Simulation
    from oracle import ops
    d = _load("sphere_96x48x48_freeslip_fp64")
    nx, ny, nz = d["grid"]
    dt = torch.float64
    sim = Simulation(nx, ny, nz, d["tau"], collision="mrt", storage="fp64", guard="pre",
                     periodic_yz=False, inlet_velocity=(d["U"], 0.0, 0.0))
    sim.set_sphere(0.5, center=tuple(d["center"]), kind="dist", q_mode="bouzidi", porosity="hard")
    sim.set_state(drivers.initial_state(nx, ny, nz, d["U"], dt, ops.consts_for(dt)).cuda())
    every = d["sample_every"]
    cd = sim.run(5 * every, sample_every=every)[:, 3].cpu().tolist()
    rel = [abs(a - b) / abs(b) for a, b in zip(cd, d["cd"])]
    print("rel Cd per 100 steps:", ["%.1e" % r for r in rel])
    assert max(rel[:4]) <= 1e-12, rel
    assert rel[4] <= 1e-9, rel
    sim.close()


def test_four_modes_base_cd(cuda):
    """Four-mode base Cd at r = 0.5 (examples/11, 96x48x48, MRT, Re 50, 2000
    steps): oracle fixture within 1e-3, published A100 values within 3%."""
    from lbm_jax_autodiff_gb300 import Simulation
    d = _load("modes_96x48x48")
    nx, ny, nz = d["grid"]
    published = {"halfway_hard": 1.85, "bouzidi_hard": 1.77, "halfway_soft": 0.43,
                 "bouzidi_soft": 0.45}
    for key, pub in published.items():
        qm, pm = key.split("_")
        sim = Simulation(nx, ny, nz, d["tau"], collision="mrt", inlet_velocity=(0.05, 0.0, 0.0))
        sim.set_sphere(0.5, kind="sigmoid", q_mode=qm, porosity=pm, sharpness=20.0)
        sim.set_state(drivers.initial_state(nx, ny, nz, 0.05).cuda())
        cd = float(sim.run(d["steps"], sample_every=d["steps"])[0, 3])
        sim.close()
        print(key, cd, d[key]["cd"], pub)
        assert abs(cd - d[key]["cd"]) <= 1e-3 * d[key]["cd"], (key, cd, d[key]["cd"])
        assert abs(cd - pub) <= 0.03 * pub, (key, cd, pub)
