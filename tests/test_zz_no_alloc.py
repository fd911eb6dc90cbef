"""lbm_momentum_exchange_noalloc: the momentum-exchange force for callers that
may not allocate device memory inside a library call (a host framework that
owns all device memory, or a fixed memory budget).  Its scratch is a fixed
array compiled into the library instead of a per-call allocation.

Called through the C ABI, in FP32 and FP64, and compared on two calls in a
row with lbm_momentum_exchange (which allocates its scratch) and with the
oracle's momentum_exchange (FP64 sums, forces.py:37-120), including a grid
at the array's limit of 16,777,216 cells.  Collected last so that a run
stopping at the first failure has already run every other test; it also
passes alone in a fresh process."""

import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_CELLS = 1 << 24


def _inputs(seed, nx, ny, nz, dtype):
    from oracle import drivers, geometry
    g = torch.Generator().manual_seed(seed)
    solid, q = geometry.create_sphere(nx, ny, nz, (0.0, 0.0, 0.0), 0.5, dtype)
    f0 = drivers.initial_state(nx, ny, nz, 0.05, dtype)
    fp = f0 + 1e-3 * torch.randn(f0.shape, generator=g, dtype=torch.float64).to(dtype)
    fs = f0 + 1e-3 * torch.randn(f0.shape, generator=g, dtype=torch.float64).to(dtype)
    return fp.contiguous(), fs.contiguous(), q.contiguous()


def _force(lib, name, dtype, fp, fs, q):
    from lbm_jax_autodiff_gb300 import _native as nat
    nx, ny, nz = fp.shape[1:]
    code = nat.LBM_F64 if dtype == torch.float64 else nat.LBM_F32
    out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = getattr(lib, name)(code, ctypes.c_void_p(fp.data_ptr()),
                            ctypes.c_void_p(fs.data_ptr()), ctypes.c_void_p(q.data_ptr()),
                            ctypes.c_void_p(out.data_ptr()), nx, ny, nz, st)
    assert rc == nat.LBM_OK, lib.lbm_last_error()
    torch.cuda.synchronize()
    return out.cpu()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64], ids=["fp32", "fp64"])
def test_noalloc_matches_allocating_entry_two_calls(cuda, dtype):
    from lbm_jax_autodiff_gb300 import _native as nat
    from oracle import ops
    lib = nat.load()
    for seed, dims in ((0, (48, 24, 24)), (1, (64, 32, 32))):
        fp, fs, q = _inputs(seed, *dims, dtype)
        want = ops.momentum_exchange(fp, fs, q).to(torch.float64)
        fpd, fsd, qd = fp.cuda(), fs.cuda(), q.cuda()
        ref = _force(lib, "lbm_momentum_exchange", dtype, fpd, fsd, qd)
        got = _force(lib, "lbm_momentum_exchange_noalloc", dtype, fpd, fsd, qd)
        assert torch.isfinite(got).all()
        # both entry points sum the same block partials in the same fixed order
        assert torch.equal(got, ref), (got, ref)
        # the oracle adds f*_i + f_opp(i) in the working precision, as the
        # reference does, and sums in FP64; the kernels add in FP64: FP32
        # inputs differ by the rounding of those additions (half an ulp of
        # ~0.1 per link term), FP64 inputs by the order of the FP64 sums
        tol = 1e-6 if dtype == torch.float32 else 1e-12
        assert torch.allclose(got, want, rtol=tol, atol=tol), (got, want)


def test_noalloc_at_its_cell_limit(cuda):
    """A 256x256x256 grid fills all 65,536 partial slots; the single-block
    total then sums the most partials it ever does."""
    from lbm_jax_autodiff_gb300 import _native as nat
    from oracle import ops
    lib = nat.load()
    nx = ny = nz = 256
    assert nx * ny * nz == MAX_CELLS
    fp, fs, q = _inputs(2, nx, ny, nz, torch.float32)
    want = ops.momentum_exchange(fp, fs, q).to(torch.float64)
    fpd, fsd, qd = fp.cuda(), fs.cuda(), q.cuda()
    del fp, fs
    for _ in range(2):
        ref = _force(lib, "lbm_momentum_exchange", torch.float32, fpd, fsd, qd)
        got = _force(lib, "lbm_momentum_exchange_noalloc", torch.float32, fpd, fsd, qd)
        assert torch.equal(got, ref), (got, ref)
        # ~10^5 link terms, each differing by the oracle's FP32 addition
        # (half an ulp of ~0.1) from the kernels' FP64 one
        assert torch.allclose(got, want, rtol=1e-5, atol=1e-5), (got, want)


def test_noalloc_rejects_grids_beyond_its_scratch(cuda):
    from lbm_jax_autodiff_gb300 import _native as nat
    lib = nat.load()
    buf = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    rc = lib.lbm_momentum_exchange_noalloc(nat.LBM_F32, p, p, p, p, 256, 256, 257,
                                           ctypes.c_void_p(0))
    assert rc == nat.LBM_ERR_UNSUPPORTED
    assert b"16777216" in lib.lbm_last_error()
