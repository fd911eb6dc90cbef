"""Batched instances (lbm_batch): one launch per step over instances of
different grids and boundary modes, the captured-graph gradient evaluation and
the device Adam step.  Each instance must reproduce the single-instance solver
on the same inputs."""
import numpy as np
import pytest
import torch

from lbm_jax_autodiff_gb300 import Batch, Simulation

pytestmark = pytest.mark.gpu

INST = [dict(nx=32, ny=16, nz=16, tau=0.56),
        dict(nx=48, ny=24, nz=24, tau=0.58),
        dict(nx=40, ny=20, nz=20, tau=0.60),
        dict(nx=32, ny=16, nz=16, tau=0.57)]
SPH = [dict(radius=0.5, kind="sigmoid", q_mode="bouzidi", porosity="hard"),
       dict(radius=0.6, kind="sigmoid", q_mode="halfway", porosity="soft", sharpness=10.0),
       dict(radius=0.55, kind="sigmoid", q_mode="bouzidi", porosity="soft", sharpness=20.0),
       dict(radius=0.5, kind="sigmoid", q_mode="halfway", porosity="hard")]


def _common(**kw):
    base = dict(collision="mrt", storage="fp32", periodic_yz=True, guard="off",
                inlet_velocity=(0.05, 0.0, 0.0))
    base.update(kw)
    return base


def _batch(inst=INST, sph=SPH, **kw):
    b = Batch([_common(**i, **kw) for i in inst])
    b.set_spheres(sph)
    b.set_equilibrium()
    return b


def _single(i, inst=INST, sph=SPH, **kw):
    s = Simulation(**_common(**inst[i], **kw))
    s.set_sphere(**sph[i])
    s.set_state(s.equilibrium_state())
    return s


def test_equilibrium_state_matches(cuda):
    """lbm_batch_set_equilibrium gives the same f_0 as Simulation.equilibrium_state."""
    b = _batch()
    for i in range(len(INST)):
        s = Simulation(**_common(**INST[i]))
        assert torch.equal(b.get_state(i), s.equilibrium_state()), i
        s.close()
    b.close()


def test_forward_matches_single(cuda):
    """Batched run (samples every 20 steps, state after 60) == each Simulation."""
    b = _batch()
    samples = b.run(60, sample_every=20)
    torch.cuda.synchronize()
    for i in range(len(INST)):
        s = _single(i)
        ref = s.run(60, sample_every=20)
        assert torch.equal(samples[:, i, :], ref), i
        assert torch.equal(b.get_state(i), s.get_state()), i
        s.close()
    b.close()


def test_gradient_matches_single(cuda):
    """Cd identical; dCd/dr equal to FP32 rounding (the single-instance
    hard-wall adjoint runs two cells per thread)."""
    n, K = 40, 10
    b = _batch()
    cd, g = b.cd_and_grad(n, checkpoint_every=K, use_graph=False)
    for i in range(len(INST)):
        s = _single(i)
        cds, gs = s.cd_and_grad(n, checkpoint_every=K)
        assert cd[i] == cds, (i, cd[i], cds)
        assert abs(g[i] - gs) <= 1e-5 * max(abs(gs), 1e-12), (i, g[i], gs)
        s.close()
    # halfway_hard: structurally zero
    assert g[3] == 0.0
    b.close()


def test_graph_replay_is_bitwise(cuda):
    b = _batch()
    cd0, g0 = b.cd_and_grad(30, checkpoint_every=10, use_graph=False)
    cd1, g1 = b.cd_and_grad(30, checkpoint_every=10, use_graph=True)    # capture + run
    cd2, g2 = b.cd_and_grad(30, checkpoint_every=10, use_graph=True)    # replay
    assert np.array_equal(cd0, cd1) and np.array_equal(cd1, cd2)
    assert np.array_equal(g0, g1) and np.array_equal(g1, g2)
    b.close()


def _adam_ref(r, g, lr, b1=0.9, b2=0.999, eps=1e-8, r_min=0.3, r_max=0.8):
    """optax.adam + clip (examples/11:182-194) over a gradient history."""
    m = v = 0.0
    out = []
    for t, gt in enumerate(g, start=1):
        out.append(r)
        m = b1 * m + (1 - b1) * gt
        v = b2 * v + (1 - b2) * gt * gt
        mh, vh = m / (1 - b1 ** t), v / (1 - b2 ** t)
        r = min(max(r - lr * mh / (np.sqrt(vh) + eps), r_min), r_max)
    return out, r


@pytest.mark.parametrize("use_graph", [False, True])
def test_optimize_adam(cuda, use_graph):
    b = _batch()
    h = b.optimize(3, 30, lr=0.05, r_min=0.3, r_max=0.8, checkpoint_every=10,
                   use_graph=use_graph)
    for i in range(len(INST)):
        rs, r_end = _adam_ref(SPH[i]["radius"], h["grad"][:, i], 0.05)
        assert np.allclose(h["r"][:, i], rs, rtol=0, atol=1e-12), (i, h["r"][:, i], rs)
        assert abs(h["r_final"][i] - r_end) <= 1e-12
        assert np.array_equal(h["loss"][:, i], h["cd"][:, i])     # loss = Cd
    # the first iteration is the plain gradient evaluation at the start radii
    cd, g = _batch().cd_and_grad(30, checkpoint_every=10, use_graph=False)
    assert np.array_equal(h["cd"][0], cd) and np.array_equal(h["grad"][0], g)
    b.close()


def test_target_loss(cuda):
    b = _batch()
    h = b.optimize(1, 20, lr=0.01, loss="target", target_cd=1.0, checkpoint_every=10,
                   use_graph=False)
    cd, g = h["cd"][0], None
    assert np.allclose(h["loss"][0], (cd - 1.0) ** 2, rtol=1e-15, atol=0)
    b2 = _batch()
    _, gcd = b2.cd_and_grad(20, checkpoint_every=10, use_graph=False)
    assert np.allclose(h["grad"][0], 2.0 * (cd - 1.0) * gcd, rtol=1e-13, atol=0)
    b.close()
    b2.close()


def test_autotune_and_block_shapes(cuda):
    b = _batch()
    cd256, g256 = b.cd_and_grad(20, checkpoint_every=10, use_graph=False)
    b.set_block(128)
    cd128, g128 = b.cd_and_grad(20, checkpoint_every=10, use_graph=False)
    # only the order of the per-block force and gradient partial sums changes
    assert np.allclose(cd128, cd256, rtol=1e-12, atol=0)
    assert np.allclose(g128, g256, rtol=1e-9, atol=1e-14)
    block, K = b.autotune(4, 200)
    assert block in (128, 256) and 1 <= K <= 200
    assert b.plan[0] == block and b.plan[1] == K
    b.close()


def test_geometry_change_between_replays(cuda):
    """New radii rebuild the instances' boundary lists and the pair-adjoint
    block maps under an already captured graph: the replay equals a fresh
    batch at the new radii, and the graph holds the planned launches."""
    n, K = 30, 10
    b = _batch()
    b.cd_and_grad(n, checkpoint_every=K, use_graph=True)      # capture
    sph2 = [dict(s, radius=s["radius"] + 0.15) for s in SPH]
    b.set_spheres(sph2)
    cd, g = b.cd_and_grad(n, checkpoint_every=K, use_graph=True)
    b2 = _batch(sph=sph2)
    cd2, g2 = b2.cd_and_grad(n, checkpoint_every=K, use_graph=False)
    assert np.array_equal(cd, cd2) and np.array_equal(g, g2)
    # n forward + stream/force + finalize + zero + seed + (n - K) recompute
    # + n adjoint steps x 2 launches (instances without / with a porosity
    # blend) + reduce
    assert b.graph_launches == n + 4 + (n - K) + 2 * n + 1
    b.close()
    b2.close()
