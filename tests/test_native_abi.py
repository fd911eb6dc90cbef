"""The C-ABI library builds, loads without a GPU and exports every entry
point declared in include/*.h (no compute calls)."""

import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**(lbm_[A-Za-z0-9_]+)\s*\(",
                             src, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from lbm_jax_autodiff_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = _declared()
    assert "lbm_create" in names and "lbm_run" in names
    assert len(names) >= 15


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    """ctypes prototypes for the C ABI; the XLA custom-call targets are bound
    by the jax.ffi module."""
    from lbm_jax_autodiff_gb300 import _native, jax_ffi
    declared = _declared()
    missing = [n for n in sorted(declared) if not n.startswith("lbm_xla_")
               and n not in _native.SIGNATURES]
    assert not missing, missing
    xla = {n[len("lbm_xla_"):] for n in declared if n.startswith("lbm_xla_")}
    assert xla == set(jax_ffi.TARGETS)


def test_xla_descriptor_text_roundtrip():
    from lbm_jax_autodiff_gb300 import jax_ffi
    d = jax_ffi.descriptor(7, 8, 9, 1, flags=1, periodic_yz=0, tau=0.548, cs=0.1,
                           u=(0.05, -0.01, 0.0), rho=1.02)
    parts = d.split()
    assert parts[0] == "lbm1" and parts[1:4] == ["7", "8", "9"]
    assert float.fromhex(parts[10]) == 0.548 and float.fromhex(parts[15]) == 1.02


def test_status_strings_without_gpu(lib):
    from lbm_jax_autodiff_gb300 import _native
    L = _native.load()
    assert L.lbm_status_string(0) == b"LBM_OK"
    assert L.lbm_status_string(4) == b"LBM_ERR_TIMEOUT"
    assert L.lbm_api_version() == 1


def test_create_rejects_bad_arguments_without_touching_the_gpu(lib):
    """Argument validation happens before any CUDA call."""
    from lbm_jax_autodiff_gb300 import _native as nat
    L = nat.load()
    p = nat.LBMParamsC()
    p.nx, p.ny, p.nz = 2, 4, 4          # nx < 3
    p.tau = 0.8
    p.rho_out = 1.0
    h = ctypes.c_void_p()
    assert L.lbm_create(ctypes.byref(p), ctypes.byref(h)) == nat.LBM_ERR_ARG
    p.nx = 8
    p.tau = 0.4                          # tau <= 0.5
    assert L.lbm_create(ctypes.byref(p), ctypes.byref(h)) == nat.LBM_ERR_ARG
    assert b"tau" in L.lbm_last_error()
    p.tau = 0.8
    p.storage = 9
    assert L.lbm_create(ctypes.byref(p), ctypes.byref(h)) == nat.LBM_ERR_ARG
    assert L.lbm_create(None, ctypes.byref(h)) == nat.LBM_ERR_ARG


def test_batch_entry_points_reject_null_handles(lib):
    """The batch queries validate their arguments before any CUDA call."""
    from lbm_jax_autodiff_gb300 import _native as nat
    L = nat.load()
    n = ctypes.c_longlong(-1)
    assert L.lbm_batch_graph_launches(None, ctypes.byref(n)) == nat.LBM_ERR_ARG
    assert n.value == -1
    b, k, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    w, g = ctypes.c_ulonglong(), ctypes.c_double()
    assert L.lbm_batch_get_plan(None, ctypes.byref(b), ctypes.byref(k), ctypes.byref(r),
                                ctypes.byref(w), ctypes.byref(g)) == nat.LBM_ERR_ARG


def test_workspace_limits_reject_null_handles(lib):
    from lbm_jax_autodiff_gb300 import _native as nat
    L = nat.load()
    assert L.lbm_set_workspace_limit(None, 1 << 30) == nat.LBM_ERR_ARG
    assert L.lbm_batch_set_workspace_limit(None, 1 << 30) == nat.LBM_ERR_ARG
    assert b"null handle" in L.lbm_last_error()


def test_streaming_setter_rejects_null_handles(lib):
    from lbm_jax_autodiff_gb300 import _native as nat
    L = nat.load()
    assert L.lbm_set_streaming(None, nat.LBM_STREAM_AA) == nat.LBM_ERR_ARG
    assert b"null handle" in L.lbm_last_error()


def test_ctypes_structs_match_the_library_layout(lib):
    """The Python binding's restated structs have the sizes the library was
    compiled with (lbm_struct_size), so a field added on one side only is
    caught without a GPU."""
    import ctypes

    from lbm_jax_autodiff_gb300 import _native as nat
    from lbm_jax_autodiff_gb300 import jax_ffi
    L = nat.load()
    assert L.lbm_struct_size(0) == ctypes.sizeof(nat.LBMParamsC)
    assert L.lbm_struct_size(1) == ctypes.sizeof(nat.LBMSphereC)
    assert L.lbm_struct_size(2) > 0
    assert L.lbm_struct_size(3) == ctypes.sizeof(jax_ffi.LBMXlaFusedDescC)
    assert L.lbm_struct_size(4) == ctypes.sizeof(nat.LBMAdamC)
    assert L.lbm_struct_size(99) == 0


def test_jax_wrappers_build_without_jax(monkeypatch):
    """The jax.ffi wrappers build (custom_vjp rules attached) against the
    jax stand-in of tests/jaxlike.py; the GPU test runs them."""
    import sys

    import jaxlike
    from lbm_jax_autodiff_gb300 import jax_ffi
    jax, jnp = jaxlike.make()
    monkeypatch.setitem(sys.modules, "jax", jax)
    monkeypatch.setitem(sys.modules, "jax.numpy", jnp)
    monkeypatch.setattr(jax_ffi, "_fns", None)
    fns = jax_ffi._build()
    for name in ("compute_density", "compute_velocity", "equilibrium", "smagorinsky_tau",
                 "soft_bounce_back", "stream", "zou_he_outlet", "momentum_exchange",
                 "_bgk_scalar", "_mrt_scalar", "_bgk_field", "_mrt_field", "_zi_uniform",
                 "_zi_face"):
        f = fns[name]
        assert f.fwd is not None and f.bwd is not None, name
    for name in ("bgk", "mrt", "zou_he_inlet", "fused_run", "simulate_cd"):
        assert callable(fns[name]), name


def test_checkpoint_plan_is_the_longest_segment_that_fits(lib):
    """lbm_plan_checkpoints (the automatic plan's search, host code) against
    a brute-force search over every segment length: the longest K with
    ceil(N/K) - 1 + K <= M, and LBM_ERR_NOMEM exactly when none fits."""
    import ctypes

    from lbm_jax_autodiff_gb300 import _native as nat
    L = nat.load()

    def states(n, k):
        return (n + k - 1) // k - 1 + k

    k = ctypes.c_int()
    for n in list(range(1, 120)) + [2000, 2880, 28000]:
        lo = min(states(n, j) for j in range(1, n + 1))
        for m in sorted({0, 1, 2, lo - 1, lo, lo + 1, n // 2, n - 1, n, n + 5, 10 ** 9}):
            rc = L.lbm_plan_checkpoints(n, m, ctypes.byref(k))
            fit = [j for j in range(1, n + 1) if states(n, j) <= m]
            if fit:
                assert rc == nat.LBM_OK and k.value == max(fit), (n, m, k.value)
            else:
                assert rc == nat.LBM_ERR_NOMEM, (n, m)
    assert L.lbm_plan_checkpoints(0, 10, ctypes.byref(k)) == nat.LBM_ERR_ARG
