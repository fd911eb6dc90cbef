"""Unit properties of the reference test-suite, checked on the CPU oracle
(tests/test_equilibrium.py, test_collision.py, test_streaming.py,
test_boundary.py of the reference project)."""

import torch

from oracle import lattice, ops
from oracle.lattice import OPP, Q

c32 = ops.consts_for(torch.float32)


def _feq(nx, ny, nz, rho=1.0, u=(0.05, 0.0, 0.0)):
    r = torch.full((nx, ny, nz), rho)
    uu = torch.zeros((3, nx, ny, nz))
    for k in range(3):
        uu[k] = u[k]
    return ops.equilibrium(r, uu, c32), r, uu


def test_weights():
    w = c32.w
    assert abs(float(w.sum()) - 1.0) < 1e-7
    assert w.shape == (19,)
    assert abs(float(w[0]) - 1 / 3) < 1e-7


def test_moment_matrix_norms_and_orthogonality():
    M = lattice.M
    G = M @ M.T
    assert (G == torch.diag(torch.tensor(lattice.ROW_NORMS)).numpy()).all()
    assert list(lattice.ROW_NORMS[:3]) == [19.0, 2394.0, 252.0]


def test_equilibrium_conservation():
    f, r, u = _feq(8, 8, 8, 1.5, (0.04, -0.01, 0.02))
    rho = ops.compute_density(f)
    assert torch.allclose(rho, r, atol=1e-4)
    assert torch.allclose(ops.compute_velocity(f, rho), u, atol=1e-4)


def test_mrt_roundtrip_and_meq():
    g = torch.Generator().manual_seed(42)
    fl = list(torch.rand(19, generator=g) * 0.1)
    back = lattice.mrt_inverse(lattice.mrt_forward(fl), c32.norms)
    assert max(abs(float(a - b)) for a, b in zip(fl, back)) < 5e-6
    f, r, u = _feq(2, 2, 2, 1.1, (0.03, 0.01, -0.02))
    m = lattice.mrt_forward([f[i] for i in range(Q)])
    meq = lattice.mrt_equilibrium_moments(r, u[0], u[1], u[2])
    for a, b in zip(m, meq):
        assert torch.allclose(a, b * torch.ones_like(a), atol=5e-4)


def test_collision_fixed_points_and_conservation():
    f, _, _ = _feq(4, 4, 4, 1.0, (0.03, 0.0, 0.0))
    assert torch.allclose(ops.bgk(f, 0.8), f, atol=5e-6)
    assert torch.allclose(ops.mrt(f, 0.8), f, atol=5e-6)
    g = torch.Generator().manual_seed(0)
    p = torch.randn(f.shape, generator=g) * 1e-3
    fp = f + p - p.mean(dim=0, keepdim=True)
    for coll in (ops.bgk, ops.mrt):
        out = coll(fp, 0.8)
        assert torch.allclose(ops.compute_density(out), ops.compute_density(fp), atol=1e-6)
        r0, r1 = ops.compute_density(fp), ops.compute_density(out)
        assert torch.allclose(r0 * ops.compute_velocity(fp, r0), r1 * ops.compute_velocity(out, r1),
                              atol=1e-6)


def test_smagorinsky():
    f, _, _ = _feq(8, 8, 8)
    assert torch.allclose(ops.smagorinsky_tau(f, 0.8, 0.1), torch.tensor(0.8), atol=5e-4)
    g = torch.Generator().manual_seed(2)
    fp = f + torch.randn(f.shape, generator=g) * 0.01
    assert bool((ops.smagorinsky_tau(fp, 0.6, 0.1) >= 0.6 - 1e-6).all())


def test_stream_shift_and_bouzidi_half():
    f = torch.zeros((Q, 4, 8, 4))
    f[3, :, 3, :] = 1.0
    q = -torch.ones((Q, 4, 8, 4))
    out = ops.stream(f, q, True)
    assert torch.allclose(out[3, :, 4, :], torch.ones(4, 4))
    assert torch.allclose(out[3, :, 3, :], torch.zeros(4, 4))
    f, _, _ = _feq(8, 8, 8)
    q = -torch.ones((Q, 8, 8, 8))
    q[1, 3] = 0.5
    out = ops.stream(f, q, True)
    assert torch.allclose(out[int(OPP[1]), 3], f[1, 3], atol=1e-7)
    assert torch.allclose(out[0], f[0])


def test_zou_he():
    f, _, _ = _feq(16, 8, 8, 1.0, (0.0, 0.0, 0.0))
    fi = ops.zou_he_inlet(f, (0.05, 0.0, 0.0))
    r = ops.compute_density(fi[:, 0:1])
    assert torch.allclose(ops.compute_velocity(fi[:, 0:1], r)[0], torch.tensor(0.05), atol=1e-3)
    f, _, _ = _feq(16, 8, 8)
    fo = ops.zou_he_outlet(f, 1.0)
    assert torch.allclose(ops.compute_density(fo[:, -1:]), torch.tensor(1.0), atol=1e-2)
