"""State save/load and VTK export (io/vtk.py): fields read back match the
oracle's moments of the same state."""
import numpy as np
import pytest
import torch

from lbm_jax_autodiff_gb300 import Simulation, io
from oracle import ops as oops

pytestmark = pytest.mark.gpu


def test_vtk_roundtrip(cuda, tmp_path):
    sim = Simulation(24, 12, 10, 0.6, collision="mrt")
    sim.set_sphere(0.5, kind="dist", q_mode="bouzidi", porosity="hard")
    sim.set_state(sim.equilibrium_state())
    sim.run(30)
    f = sim.get_state()
    solid = torch.zeros((24, 12, 10), dtype=torch.int32)
    solid[10:14, 5:7, 4:6] = 1
    por = torch.rand((24, 12, 10), generator=torch.Generator().manual_seed(0))
    path = str(tmp_path / "flow.vtk")
    io.export_vtk(path, f, solid=solid, porosity=por)
    got = io.read_vtk(path)
    fc = f.double().cpu()
    rho = oops.compute_density(fc)
    u = oops.compute_velocity(fc, rho)
    assert np.allclose(got["density"], rho.numpy(), rtol=1e-6, atol=1e-7)
    for k, name in enumerate(("velocity_x", "velocity_y", "velocity_z")):
        assert np.allclose(got[name], u[k].numpy(), rtol=1e-5, atol=1e-7), name
    assert np.allclose(got["velocity_magnitude"], u.pow(2).sum(0).sqrt().numpy(), rtol=1e-5,
                       atol=1e-7)
    assert np.array_equal(got["solid"], solid.numpy().astype(np.float32))
    assert np.allclose(got["porosity"], por.numpy(), rtol=0, atol=0)
    sim.close()


def test_save_load_state(cuda, tmp_path):
    sim = Simulation(16, 8, 8, 0.6, collision="bgk")
    sim.set_sphere(0.5, kind="dist", q_mode="halfway", porosity="hard")
    sim.set_state(sim.equilibrium_state())
    sim.run(20)
    path = str(tmp_path / "state.npz")
    io.save_state(path, sim)
    f_saved = sim.get_state()
    sim.run(10)
    ref = sim.get_state()
    steps = io.load_state(path, sim)
    assert steps == 20
    assert torch.equal(sim.get_state(), f_saved)
    sim.run(10)
    assert torch.equal(sim.get_state(), ref)     # same trajectory from the restored state
    sim.close()
