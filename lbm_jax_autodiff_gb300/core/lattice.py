"""D3Q19 lattice constants (host side).

Same values and ordering as jax_lbm/core/lattice.py:29-129: velocities,
float32 weights, opposite map, cs^2 and the MRT row norms / relaxation rates.
The device kernels carry their own copy of these tables (csrc/lbm_core.cuh).
"""

import numpy as np
import torch

Q = 19
CS2 = 1.0 / 3.0
INV_CS2 = 3.0
INV_CS4 = 9.0

D3Q19_VELOCITIES = np.array([
    [0, 0, 0],
    [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
    [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0],
    [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
    [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1],
], dtype=np.int32)

D3Q19_OPPOSITE = np.array([0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15],
                          dtype=np.int32)

_W_EXACT = np.array([1.0 / 3.0] + [1.0 / 18.0] * 6 + [1.0 / 36.0] * 12)
D3Q19_WEIGHTS = _W_EXACT.astype(np.float32)

MRT_ROW_NORMS = np.array([19.0, 2394.0, 252.0, 10.0, 40.0, 10.0, 40.0, 10.0, 40.0,
                          36.0, 72.0, 12.0, 24.0, 4.0, 4.0, 4.0, 8.0, 8.0, 8.0],
                         dtype=np.float32)
MRT_RELAXATION_RATES = np.array([0.0, 1.19, 1.4, 0.0, 1.2, 0.0, 1.2, 0.0, 1.2, 0.0,
                                 1.4, 0.0, 1.4, 0.0, 0.0, 0.0, 1.98, 1.98, 1.98],
                                dtype=np.float32)
MRT_STRESS_INDICES = np.array([9, 11, 13, 14, 15], dtype=np.int32)


def weights(exact=False, dtype=np.float64):
    """Weights as used by the kernels: float32-rounded unless ``exact``."""
    w = _W_EXACT if exact else D3Q19_WEIGHTS.astype(np.float64)
    return w.astype(dtype)


def equilibrium_uniform(shape, ux, dtype=torch.float32, exact=False, device="cuda"):
    """f_eq(rho=1, u=(ux, 0, 0)) broadcast over a grid -- the reference's
    initial state (examples/10:152-154).  19 values, computed once."""
    w = weights(exact)
    e = D3Q19_VELOCITIES[:, 0].astype(np.float64)
    ux = float(ux)
    feq = w * (1.0 + 3.0 * e * ux + 4.5 * (e * ux) ** 2 - 1.5 * ux * ux)
    col = torch.tensor(feq, dtype=dtype, device=device).view(Q, 1, 1, 1)
    return col.expand((Q,) + tuple(shape)).contiguous()


def _moment_matrix():
    """19x19 d'Humieres moment matrix built from its row polynomials."""
    e = D3Q19_VELOCITIES.astype(np.int64)
    x, y, z = e[:, 0], e[:, 1], e[:, 2]
    e2 = x * x + y * y + z * z
    rows = [np.ones(Q, dtype=np.int64), 19 * e2 - 30, (21 * e2 * e2 - 53 * e2 + 24) // 2,
            x, (5 * e2 - 9) * x, y, (5 * e2 - 9) * y, z, (5 * e2 - 9) * z,
            3 * x * x - e2, (3 * e2 - 5) * (3 * x * x - e2), y * y - z * z,
            (3 * e2 - 5) * (y * y - z * z), x * y, y * z, x * z,
            (y * y - z * z) * x, (z * z - x * x) * y, (x * x - y * y) * z]
    return np.stack(rows)


MRT_MATRIX = _moment_matrix()


def mrt_forward(f_cell):
    """m = M f for one cell, shape (19,) (lattice.py:132-211)."""
    t = torch.as_tensor(f_cell)
    return torch.as_tensor(MRT_MATRIX, dtype=t.dtype, device=t.device) @ t


def mrt_inverse(m):
    """f = M^T diag(1/||M_k||^2) m (lattice.py:214-339)."""
    t = torch.as_tensor(m)
    M = torch.as_tensor(MRT_MATRIX, dtype=t.dtype, device=t.device)
    n = torch.as_tensor(MRT_ROW_NORMS, dtype=t.dtype, device=t.device)
    return M.t() @ (t / n)


def mrt_equilibrium_moments(rho, u):
    """Equilibrium moments of one cell (lattice.py:342-391)."""
    u = torch.as_tensor(u)
    ux, uy, uz = u[0], u[1], u[2]
    rho = torch.as_tensor(rho, dtype=u.dtype, device=u.device)
    u2 = ux * ux + uy * uy + uz * uz
    pxx = 2 * ux * ux - uy * uy - uz * uz
    pww = uy * uy - uz * uz
    z = rho * 0
    return torch.stack([rho, -11 * rho + 19 * rho * u2, 3 * rho - 5.5 * rho * u2,
                        rho * ux, -2.0 / 3.0 * rho * ux, rho * uy, -2.0 / 3.0 * rho * uy,
                        rho * uz, -2.0 / 3.0 * rho * uz, rho * pxx, -0.5 * rho * pxx,
                        rho * pww, -0.5 * rho * pww, rho * ux * uy, rho * uy * uz, rho * ux * uz,
                        z, z, z])
