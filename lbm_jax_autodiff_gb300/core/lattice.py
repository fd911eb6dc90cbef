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
