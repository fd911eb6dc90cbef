"""Helpers shared by the per-op drop-in modules (core/*, geometry/*)."""

import ctypes

import torch

from . import _native as nat

FLAGS_EXACT = 1   # LBM_OP_EXACT_CONSTANTS


def dtype_code(t):
    if t.dtype == torch.float32:
        return nat.LBM_F32
    if t.dtype == torch.float64:
        return nat.LBM_F64
    raise TypeError("expected a float32 or float64 tensor, got %s" % t.dtype)


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr() if t is not None else None)


def cuda_contig(t, name):
    if not torch.is_tensor(t):
        raise TypeError("%s must be a torch tensor" % name)
    if not t.is_cuda:
        raise TypeError("%s must be on a CUDA device (this package has no CPU path)" % name)
    return t.contiguous()


def pop_dims(f):
    if f.dim() != 4 or f.shape[0] != 19:
        raise ValueError("populations must have shape (19, nx, ny, nz), got %s" % tuple(f.shape))
    return int(f.shape[1]), int(f.shape[2]), int(f.shape[3])


def call(name, *args):
    return nat.call(name, *args)
