"""D3Q19 constants and the MRT moment basis, restated for the CPU oracle.

Follows jax_lbm/core/lattice.py:
  velocities            lattice.py:29-49
  weights (float32!)    lattice.py:53-60
  opposite map          lattice.py:68-71
  cs^2                  lattice.py:75
  MRT row norms         lattice.py:88-94
  MRT relaxation rates  lattice.py:106-126, stress slots lattice.py:129
  mrt_forward           lattice.py:132-211
  mrt_inverse           lattice.py:214-339  (M^T diag(1/||M_k||^2))
  mrt_equilibrium_moments lattice.py:342-391

The reference stores the weights and MRT rates as float32 arrays even when
JAX runs in float64, so a reference FP64 run uses 1/3 -> 0.3333333432674408.
``Consts(dtype, ref_consts=True)`` reproduces that; ``ref_consts=False``
gives the exact rationals (the FP64 "truth" variant).

The moment matrix is built here from the d'Humieres (2002) polynomial
definitions of each moment row rather than typed out; the test-suite checks
it against the row norms and the reference's sparse formulas' properties.
"""

import numpy as np
import torch

Q = 19

# Velocity ordering of lattice.py:29-49 (rest, 6 faces, 12 edges).
E = np.array([
    [0, 0, 0],
    [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
    [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0],
    [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
    [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1],
], dtype=np.int64)

OPP = np.array([int(np.nonzero((E == -E[i]).all(axis=1))[0][0]) for i in range(Q)],
               dtype=np.int64)

_W_RATIONAL = np.array([1.0 / 3.0] + [1.0 / 18.0] * 6 + [1.0 / 36.0] * 12)

CS2 = 1.0 / 3.0


def _moment_matrix():
    """19x19 integer moment matrix, rows in the reference moment order.

    Row k is a polynomial in the lattice velocity e=(x,y,z) evaluated on the
    19 velocities; the ordering is rho, e, eps, jx, qx, jy, qy, jz, qz,
    3pxx, 3pixx, pww, piww, pxy, pyz, pxz, mx, my, mz (lattice.py:115-118).
    """
    x, y, z = E[:, 0], E[:, 1], E[:, 2]
    e2 = x * x + y * y + z * z
    rows = [
        np.ones(Q, dtype=np.int64),
        19 * e2 - 30,
        (21 * e2 * e2 - 53 * e2 + 24) // 2,
        x, (5 * e2 - 9) * x,
        y, (5 * e2 - 9) * y,
        z, (5 * e2 - 9) * z,
        3 * x * x - e2,
        (3 * e2 - 5) * (3 * x * x - e2),
        y * y - z * z,
        (3 * e2 - 5) * (y * y - z * z),
        x * y, y * z, x * z,
        (y * y - z * z) * x,
        (z * z - x * x) * y,
        (x * x - y * y) * z,
    ]
    return np.stack(rows).astype(np.int64)


M = _moment_matrix()
ROW_NORMS = (M * M).sum(axis=1).astype(np.float64)   # 19, 2394, 252, 10, 40, ...

# Fixed rates of lattice.py:106-126; the stress slots are filled with omega.
_RATES = np.array([0.0, 1.19, 1.4, 0.0, 1.2, 0.0, 1.2, 0.0, 1.2,
                   0.0, 1.4, 0.0, 1.4, 0.0, 0.0, 0.0, 1.98, 1.98, 1.98])
STRESS_SLOTS = (9, 11, 13, 14, 15)


class Consts:
    """Per-dtype constant tensors.

    ref_consts=True rounds the weights and MRT rates through float32 exactly
    as the reference's ``dtype=jnp.float32`` arrays do (lattice.py:60,126).
    """

    def __init__(self, dtype=torch.float32, ref_consts=True):
        self.dtype = dtype
        w = _W_RATIONAL.copy()
        rates = _RATES.copy()
        if ref_consts:
            w = w.astype(np.float32).astype(np.float64)
            rates = rates.astype(np.float32).astype(np.float64)
        self.w = torch.tensor(w, dtype=dtype)
        self.w_list = [float(v) for v in w]
        self.rates = [float(v) for v in rates]
        self.norms = [float(v) for v in ROW_NORMS]
        self.ref_consts = ref_consts


def mrt_forward(fl):
    """m = M f for a list of 19 same-shaped tensors (lattice.py:132-211).

    Terms are summed in increasing direction index, zero entries skipped.
    """
    out = []
    for k in range(Q):
        acc = None
        for i in range(Q):
            c = int(M[k, i])
            if c == 0:
                continue
            t = fl[i] if c == 1 else (-fl[i] if c == -1 else c * fl[i])
            acc = t if acc is None else acc + t
        out.append(acc)
    return out


def mrt_inverse(ml, norms):
    """f = M^T diag(1/n) m for a list of 19 moment tensors (lattice.py:214-339).

    The moments are first divided by the row norms (lattice.py:244), then
    combined in increasing moment index.
    """
    ms = [ml[k] / norms[k] for k in range(Q)]
    out = []
    for i in range(Q):
        acc = None
        for k in range(Q):
            c = int(M[k, i])
            if c == 0:
                continue
            t = ms[k] if c == 1 else (-ms[k] if c == -1 else c * ms[k])
            acc = t if acc is None else acc + t
        out.append(acc)
    return out


def mrt_equilibrium_moments(rho, ux, uy, uz):
    """Equilibrium moments m_eq(rho, u) (lattice.py:342-391)."""
    u2 = ux * ux + uy * uy + uz * uz
    zero = rho * 0.0
    pxx = 2.0 * ux * ux - uy * uy - uz * uz
    pww = uy * uy - uz * uz
    return [
        rho,
        -11.0 * rho + 19.0 * rho * u2,
        3.0 * rho - 5.5 * rho * u2,
        rho * ux, -2.0 / 3.0 * rho * ux,
        rho * uy, -2.0 / 3.0 * rho * uy,
        rho * uz, -2.0 / 3.0 * rho * uz,
        rho * pxx, -0.5 * rho * pxx,
        rho * pww, -0.5 * rho * pww,
        rho * ux * uy, rho * uy * uz, rho * ux * uz,
        zero, zero, zero,
    ]
