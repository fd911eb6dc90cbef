"""q from a solid mask (jax_lbm/geometry/bouzidi.py:32-106)."""

import torch

from .. import _ops as op


def compute_q_from_solid(solid, nx=None, ny=None, nz=None, default_q=0.5, dtype=torch.float32):
    """q = default_q on every in-bounds fluid -> body (solid == 1) link, -1
    elsewhere; shape (19, nx, ny, nz)."""
    s = op.cuda_contig(solid, "solid").to(torch.int32)
    nx, ny, nz = s.shape
    q = torch.empty((19, nx, ny, nz), dtype=dtype, device=s.device)
    op.call("lbm_q_from_solid", op.dtype_code(q), op.ptr(s), float(default_q), op.ptr(q), nx, ny,
            nz, op.stream())
    return q
