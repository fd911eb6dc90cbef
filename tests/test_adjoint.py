"""Hand-written adjoint (dCd/dr, dCd/dq) vs the reference's published FP64
gradient, vs torch autograd through the CPU oracle (the stand-in for
jax.grad), vs central finite differences, and the halfway_hard zero."""

import pytest
import torch

from oracle import drivers
from oracle.ops import consts_for

pytestmark = pytest.mark.gpu


def _sim(nx, ny, nz, tau, collision="mrt", storage="fp64", **kw):
    from lbm_jax_autodiff_gb300 import Simulation
    return Simulation(nx, ny, nz, tau, collision=collision, storage=storage, **kw)


def test_published_bouzidi_gradient_9333275(cuda):
    """tests/test_gradients_f64.py:129-217 of the reference: 32x16x16, 10 BGK
    steps, sigmoid porosity alpha 20, r 0.5, Re 50; published AD 93.33275."""
    nx, ny, nz = 32, 16, 16
    tau = 3.0 * (0.05 * 4.0 / 50.0) + 0.5
    sim = _sim(nx, ny, nz, tau, collision="bgk", storage="fp64")
    sim.set_sphere(0.5, kind="sigmoid", q_mode="bouzidi", porosity="soft", sharpness=20.0,
                   disc_floor=1e-20, denom_eps=1e-30)
    sim.set_state(sim.equilibrium_state())
    for K in (0, 3):
        cd, g = sim.cd_and_grad(10, checkpoint_every=K)
        assert abs(cd - 13.741894179419857) < 1e-9
        assert abs(g - 93.33275) < 1e-5 * 93.33275, g


CASES = [
    # collision, smag, q_mode, porosity, periodic
    ("mrt", None, "bouzidi", "soft", True),
    ("mrt", 0.1, "bouzidi", "hard", True),
    ("bgk", None, "bouzidi", "hard", False),
    ("bgk", 0.1, "halfway", "soft", True),
]


@pytest.mark.parametrize("collision,smag,q_mode,porosity,periodic", CASES)
def test_fp64_vs_autograd(cuda, collision, smag, q_mode, porosity, periodic):
    nx, ny, nz, n = 24, 12, 12, 8
    tau = 0.56
    dt = torch.float64
    c = consts_for(dt)
    r = torch.tensor(0.6, dtype=dt, requires_grad=True)
    cd, q, solid, por = drivers.simulate_cd(r, nx, ny, nz, n, tau, q_mode=q_mode,
                                            porosity_mode=porosity, collision=collision,
                                            smagorinsky_cs=smag, periodic_yz=periodic, dtype=dt,
                                            consts=c, return_parts=True)
    cd.backward()
    g_ref = r.grad.item()
    # dCd/dq with q as a leaf
    q_leaf = q.detach().clone().requires_grad_(True)
    cd2 = drivers.simulate_cd(torch.tensor(0.6, dtype=dt), nx, ny, nz, n, tau, q_mode=q_mode,
                              porosity_mode=porosity, collision=collision, smagorinsky_cs=smag,
                              periodic_yz=periodic, dtype=dt, consts=c, q_leaf=q_leaf)
    cd2.backward()
    gq_ref = q_leaf.grad

    sim = _sim(nx, ny, nz, tau, collision=collision, storage="fp64",
               use_smagorinsky=smag is not None, smagorinsky_cs=smag or 0.1, periodic_yz=periodic)
    sim.set_sphere(0.6, kind="sigmoid", q_mode=q_mode, porosity=porosity, sharpness=20.0)
    sim.set_state(drivers.initial_state(nx, ny, nz, 0.05, dt, c).cuda())
    cdg, gg, ex = sim.cd_and_grad(n, checkpoint_every=3, dcd_dq=True)
    assert abs(cdg - cd.item()) <= 1e-10 * abs(cd.item())
    assert abs(gg - g_ref) <= 1e-8 * max(1.0, abs(g_ref)), (gg, g_ref)
    gq = ex["dcd_dq"].cpu()
    links = q >= 0
    err = (gq[links] - gq_ref[links]).abs().max().item()
    scale = gq_ref[links].abs().max().item()
    assert err <= 1e-9 * max(scale, 1.0), (err, scale)
    assert (gq[~links] == 0).all()


def test_halfway_hard_is_exactly_zero(cuda):
    nx, ny, nz = 32, 16, 16
    sim = _sim(nx, ny, nz, 0.56, storage="fp32")
    sim.set_sphere(0.5, kind="sigmoid", q_mode="halfway", porosity="hard")
    sim.set_state(sim.equilibrium_state())
    cd, g = sim.cd_and_grad(50, checkpoint_every=10)
    assert cd > 0.0
    assert g == 0.0


@pytest.mark.parametrize("K", [1, 7, 0])
def test_checkpoint_interval_invariance(cuda, K):
    nx, ny, nz = 32, 16, 16
    sim = _sim(nx, ny, nz, 0.56, storage="fp32")
    sim.set_sphere(0.5, kind="sigmoid", q_mode="bouzidi", porosity="soft")
    sim.set_state(sim.equilibrium_state())
    base = sim.cd_and_grad(30, checkpoint_every=5)
    got = sim.cd_and_grad(30, checkpoint_every=K)
    assert got == base      # recomputation is bit-for-bit deterministic


def test_fp32_vs_fp64_oracle(cuda):
    """FP32 storage adjoint within 1e-3 relative of the FP64 oracle gradient."""
    nx, ny, nz, n = 32, 16, 16, 60
    tau = 0.56
    dt = torch.float64
    r = torch.tensor(0.5, dtype=dt, requires_grad=True)
    cd = drivers.simulate_cd(r, nx, ny, nz, n, tau, q_mode="bouzidi", porosity_mode="hard",
                             dtype=dt, consts=consts_for(dt))
    cd.backward()
    sim = _sim(nx, ny, nz, tau, storage="fp32")
    sim.set_sphere(0.5, kind="sigmoid", q_mode="bouzidi", porosity="hard")
    sim.set_state(sim.equilibrium_state())
    cdg, gg = sim.cd_and_grad(n, checkpoint_every=20)
    assert abs(cdg - cd.item()) <= 2e-4 * abs(cd.item())
    assert abs(gg - r.grad.item()) <= 1e-3 * abs(r.grad.item()), (gg, r.grad.item())


def test_central_fd_gpu(cuda):
    """dCd/dr against central differences of the GPU forward (FP64, dr = 1e-6)."""
    nx, ny, nz, n = 32, 16, 16, 40
    tau = 0.56

    def cd_at(rr):
        s = _sim(nx, ny, nz, tau, storage="fp64")
        s.set_sphere(rr, kind="sigmoid", q_mode="bouzidi", porosity="soft")
        s.set_state(s.equilibrium_state())
        return s.cd_and_grad(n, checkpoint_every=8)

    cd0, g = cd_at(0.55)
    h = 1e-6
    fd = (cd_at(0.55 + h)[0] - cd_at(0.55 - h)[0]) / (2 * h)
    assert abs(fd - g) <= 1e-5 * abs(g), (fd, g)


def test_guard_rejected(cuda):
    from lbm_jax_autodiff_gb300._native import LBMError
    sim = _sim(16, 8, 8, 0.6, storage="fp32", guard="pre")
    sim.set_sphere(0.5)
    sim.set_state(sim.equilibrium_state())
    with pytest.raises(LBMError, match="UNSUPPORTED"):
        sim.cd_and_grad(4)


@pytest.mark.parametrize("storage,cd_tol,g_tol", [("fp16", 1e-3, 1e-3), ("bf16", 3e-3, 3e-2)])
def test_low_precision_gradient_vs_fp64(cuda, storage, cd_tol, g_tol):
    """16-bit storage: Cd and dCd/dr against the FP64-storage solver on the
    same problem (MRT + Smagorinsky, Bouzidi hard sphere, 400 steps)."""
    nx, ny, nz, n = 64, 32, 32, 400
    tau = 0.56

    def run(st):
        sim = _sim(nx, ny, nz, tau, storage=st, use_smagorinsky=True, smagorinsky_cs=0.1)
        sim.set_sphere(0.5, kind="dist", q_mode="bouzidi", porosity="hard")
        sim.set_state(sim.equilibrium_state())
        out = sim.cd_and_grad(n, checkpoint_every=100)
        sim.close()
        return out

    cd64, g64 = run("fp64")
    cd, g = run(storage)
    assert abs(cd - cd64) <= cd_tol * abs(cd64), (cd, cd64)
    assert abs(g - g64) <= g_tol * abs(g64), (g, g64)


@pytest.mark.parametrize("nx,ny,nz,periodic,center", [
    (32, 16, 16, False, (0.0, 0.0, 0.0)),     # pair kernel: non-periodic edges in its list
    (33, 17, 15, True, (0.0, 0.0, 0.0)),      # odd nz: per-cell kernels
    (32, 16, 16, True, (-2.6, 0.0, 0.0)),     # links next to the inlet face
])
def test_fp32_gradient_paths_vs_fp64_oracle(cuda, nx, ny, nz, periodic, center):
    """FP32 storage dCd/dr through every adjoint path (packed interior pairs,
    listed boundary pairs, per-cell kernels) within 1e-3 of the FP64 oracle."""
    n, tau = 60, 0.56
    dt = torch.float64
    r = torch.tensor(0.5, dtype=dt, requires_grad=True)
    cd = drivers.simulate_cd(r, nx, ny, nz, n, tau, q_mode="bouzidi", porosity_mode="hard",
                             periodic_yz=periodic, center=center, dtype=dt,
                             consts=consts_for(dt))
    cd.backward()
    sim = _sim(nx, ny, nz, tau, storage="fp32", periodic_yz=periodic)
    sim.set_sphere(0.5, center=center, kind="sigmoid", q_mode="bouzidi", porosity="hard")
    sim.set_state(sim.equilibrium_state())
    cdg, gg = sim.cd_and_grad(n, checkpoint_every=20)
    sim.close()
    assert abs(cdg - cd.item()) <= 2e-4 * abs(cd.item()), (cdg, cd.item())
    assert abs(gg - r.grad.item()) <= 1e-3 * abs(r.grad.item()), (gg, r.grad.item())


@pytest.mark.parametrize("nx,ny,nz,periodic", [(48, 24, 24, False), (49, 25, 23, True)])
def test_fp16_paths_vs_fp32(cuda, nx, ny, nz, periodic):
    """FP16 storage through the pair kernels with a non-periodic box (edges
    listed) and through the per-cell kernels (odd nz): Cd and dCd/dr within
    the FP16 bar of the FP32 solver."""
    n, tau = 200, 0.56

    def run(st):
        sim = _sim(nx, ny, nz, tau, storage=st, periodic_yz=periodic)
        sim.set_sphere(0.5, kind="dist", q_mode="bouzidi", porosity="hard")
        sim.set_state(sim.equilibrium_state())
        out = sim.cd_and_grad(n, checkpoint_every=50)
        sim.close()
        return out

    cd32, g32 = run("fp32")
    cd16, g16 = run("fp16")
    assert abs(cd16 - cd32) <= 1e-3 * abs(cd32), (cd16, cd32)
    assert abs(g16 - g32) <= 1e-3 * abs(g32), (g16, g32)


@pytest.mark.parametrize("collision,smag,q_mode,periodic", [
    ("mrt", 0.1, "bouzidi", True),
    ("bgk", None, "halfway", False),     # non-periodic edges in the list
    ("mrt", None, "halfway", True),
])
def test_fp32_soft_sphere_vs_fp64(cuda, collision, smag, q_mode, periodic):
    """Sigmoid-porosity sphere: the FP32 packed adjoint (porosity-blend
    transpose and dJ/dp on the pairs) within 1e-3 of the FP64 per-cell one."""
    nx, ny, nz, n, tau = 32, 16, 16, 60, 0.56

    def run(st):
        sim = _sim(nx, ny, nz, tau, collision=collision, storage=st,
                   use_smagorinsky=smag is not None, smagorinsky_cs=smag or 0.1,
                   periodic_yz=periodic)
        sim.set_sphere(0.5, kind="sigmoid", q_mode=q_mode, porosity="soft", sharpness=20.0)
        sim.set_state(sim.equilibrium_state())
        out = sim.cd_and_grad(n, checkpoint_every=20)
        sim.close()
        return out

    cd64, g64 = run("fp64")
    cd32, g32 = run("fp32")
    assert abs(cd32 - cd64) <= 2e-4 * abs(cd64), (cd32, cd64)
    assert abs(g32 - g64) <= 1e-3 * abs(g64), (g32, g64)


def test_fp32_porosity_field_vs_fp64(cuda):
    """Porosity given as a field (mask geometry): dCd/dq of the FP32 packed
    adjoint within 1e-3 of the FP64 per-cell one."""
    from oracle import geometry
    nx, ny, nz, n, tau = 32, 16, 16, 60, 0.56

    def run(st, dt):
        por, solid, q = geometry.sphere_geometry(nx, ny, nz, 0.5, "bouzidi", "soft", 20.0)
        sim = _sim(nx, ny, nz, tau, storage=st)
        sim.set_mask(solid.to(torch.int32).cuda(), q.to(dt).cuda().contiguous(),
                     porosity=por.to(dt).cuda().contiguous())
        sim.set_state(sim.equilibrium_state())
        cd, _, ex = sim.cd_and_grad(n, checkpoint_every=20, dcd_dq=True)
        gq = ex["dcd_dq"].double().cpu()
        sim.close()
        return cd, gq

    cd64, gq64 = run("fp64", torch.float64)
    cd32, gq32 = run("fp32", torch.float32)
    assert abs(cd32 - cd64) <= 2e-4 * abs(cd64), (cd32, cd64)
    scale = gq64.abs().max().item()
    assert scale > 0.0
    assert (gq32 - gq64).abs().max().item() <= 1e-3 * scale


def test_full_size_precision_bars(cuda):
    """The 256x128x128 workload (sphere D = 32, Re 100, MRT + Smagorinsky
    Cs 0.1, Bouzidi hard sphere), dCd/dr over a 2000-step window, workspace
    sized to free HBM: FP16 storage within 1e-3 and FP32 storage within
    1e-4 (Cd) / 1e-5 (dCd/dr) of the FP64-storage solver."""
    nx, ny, nz, n = 256, 128, 128, 2000
    U = 0.05
    tau = 3.0 * (U * 32.0 / 100.0) + 0.5

    def run(st):
        torch.cuda.empty_cache()
        sim = _sim(nx, ny, nz, tau, storage=st, use_smagorinsky=True, smagorinsky_cs=0.1,
                   inlet_velocity=(U, 0.0, 0.0))
        sim.set_sphere(0.5, kind="dist", q_mode="bouzidi", porosity="hard")
        sim.set_state(sim.equilibrium_state())
        out = sim.cd_and_grad(n, checkpoint_every=0)
        sim.close()
        return out

    cd64, g64 = run("fp64")
    cd16, g16 = run("fp16")
    cd32, g32 = run("fp32")
    assert abs(cd16 - cd64) <= 1e-3 * abs(cd64), (cd16, cd64)
    assert abs(g16 - g64) <= 1e-3 * abs(g64), (g16, g64)
    assert abs(cd32 - cd64) <= 1e-4 * abs(cd64), (cd32, cd64)
    assert abs(g32 - g64) <= 1e-5 * abs(g64), (g32, g64)


def test_workspace_limit_caps_the_automatic_plan(cuda):
    """A cap on the adjoint workspace: the automatic plan stays under it and
    gives the same result as the uncapped plan; a cap below the smallest
    workspace (ceil(N/K) - 1 + K states at K ~ sqrt(N)) is refused."""
    from lbm_jax_autodiff_gb300._native import LBMError
    nx, ny, nz, n = 32, 16, 16, 64
    sim = _sim(nx, ny, nz, 0.56, storage="fp32")
    sim.set_sphere(0.5, kind="sigmoid", q_mode="bouzidi", porosity="soft")
    sim.set_state(sim.equilibrium_state())
    free = sim.cd_and_grad(n, checkpoint_every=0)
    K0, rec0, bytes0 = sim.adjoint_plan
    assert (K0, rec0) == (n, 0)
    state = 19 * nx * ny * nz * 4
    assert bytes0 == n * state                        # K stashed states, no checkpoint
    sim.release_workspace()
    sim.set_workspace_limit(20 * state)
    capped = sim.cd_and_grad(n, checkpoint_every=0)
    K, rec, wbytes = sim.adjoint_plan
    assert wbytes <= 20 * state and ((n + K - 1) // K - 1 + K) * state == wbytes
    assert rec == n - K and K < n
    assert capped == free                             # recomputation is exact
    sim.set_workspace_limit(14 * state)               # min over K of ceil(64/K) - 1 + K is 15
    with pytest.raises(LBMError, match="NOMEM"):
        sim.cd_and_grad(n, checkpoint_every=0)
    sim.set_workspace_limit(0)
    assert sim.cd_and_grad(n, checkpoint_every=0) == free
    sim.close()
