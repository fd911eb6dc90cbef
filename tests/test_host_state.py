"""Host-pointer state entry points (lbm_set_state_host / lbm_get_state_host):
the same f as the device-pointer entry points, with and without a sample of
the final step (whose pass leaves f in the solver, so get_state_host is one
copy), and after a second set_state_host."""

import pytest
import torch

pytestmark = pytest.mark.gpu


def _sim():
    from lbm_jax_autodiff_gb300 import Simulation
    s = Simulation(48, 24, 24, 0.56, collision="mrt", use_smagorinsky=True, guard="pre")
    s.set_sphere(0.5, kind="dist", q_mode="bouzidi", porosity="hard")
    return s


@pytest.mark.parametrize("sample", [False, True])
def test_host_state_matches_device_state(cuda, sample):
    a, b = _sim(), _sim()
    f0 = a.equilibrium_state().cpu()
    host_in = f0.clone().pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    a.set_state(f0.cuda())
    b.set_state_host(host_in)
    for chunk in (7, 13):
        kw = dict(sample_every=chunk) if sample else {}
        sa = a.run(chunk, **kw)
        sb = b.run(chunk, **kw)
        ref = a.get_state().cpu()
        b.get_state_host(host_out)
        torch.cuda.synchronize()
        assert torch.equal(host_out, ref)
        if sample:
            assert torch.equal(sa, sb)
    # the state after 0 steps, then a new start from the host
    b.set_state_host(host_in)
    b.get_state_host(host_out)
    torch.cuda.synchronize()
    assert torch.equal(host_out, f0)
    b.run(5)
    a.set_state(f0.cuda())
    a.run(5)
    b.get_state_host(host_out)
    torch.cuda.synchronize()
    assert torch.equal(host_out, a.get_state().cpu())
    a.close()
    b.close()
