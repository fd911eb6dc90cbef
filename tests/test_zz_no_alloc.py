"""lbm_momentum_exchange_noalloc: the momentum-exchange force for callers that
may not allocate device memory inside a library call (a host framework that
owns all device memory, or a fixed memory budget).  Its scratch is a fixed
array compiled into the library instead of a per-call allocation.

Called through the C ABI and compared with lbm_momentum_exchange (which
allocates its scratch) on two calls in a row.  Collected last so that a run
stopping at the first failure has already run every other test; it also
passes alone in a fresh process."""

import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _inputs(seed, nx, ny, nz):
    from oracle import drivers, geometry
    g = torch.Generator().manual_seed(seed)
    solid, q = geometry.create_sphere(nx, ny, nz, (0.0, 0.0, 0.0), 0.5)
    f0 = drivers.initial_state(nx, ny, nz, 0.05)
    fp = f0 + 1e-3 * torch.randn(f0.shape, generator=g)
    fs = f0 + 1e-3 * torch.randn(f0.shape, generator=g)
    return fp.cuda().contiguous(), fs.cuda().contiguous(), q.cuda().contiguous()


def _force(lib, name, fp, fs, q):
    from lbm_jax_autodiff_gb300 import _native as nat
    nx, ny, nz = fp.shape[1:]
    out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = getattr(lib, name)(nat.LBM_F32, ctypes.c_void_p(fp.data_ptr()),
                            ctypes.c_void_p(fs.data_ptr()), ctypes.c_void_p(q.data_ptr()),
                            ctypes.c_void_p(out.data_ptr()), nx, ny, nz, st)
    assert rc == nat.LBM_OK, lib.lbm_last_error()
    torch.cuda.synchronize()
    return out.cpu()


def test_noalloc_matches_allocating_entry_two_calls(cuda):
    from lbm_jax_autodiff_gb300 import _native as nat
    lib = nat.load()
    for seed, dims in ((0, (48, 24, 24)), (1, (64, 32, 32))):
        fp, fs, q = _inputs(seed, *dims)
        ref = _force(lib, "lbm_momentum_exchange", fp, fs, q)
        got = _force(lib, "lbm_momentum_exchange_noalloc", fp, fs, q)
        assert torch.isfinite(got).all()
        assert torch.allclose(got, ref, rtol=1e-12, atol=1e-15), (got, ref)


def test_noalloc_rejects_grids_beyond_its_scratch(cuda):
    from lbm_jax_autodiff_gb300 import _native as nat
    lib = nat.load()
    buf = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    rc = lib.lbm_momentum_exchange_noalloc(nat.LBM_F32, p, p, p, p, 256, 256, 257,
                                           ctypes.c_void_p(0))
    assert rc == nat.LBM_ERR_UNSUPPORTED
    assert b"16777216" in lib.lbm_last_error()
