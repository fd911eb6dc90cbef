"""A stand-in for the few parts of jax that lbm_jax_autodiff_gb300.jax_ffi
uses, so its wrappers run without JAX (absent on every machine this project
is built and tested on).  Test infrastructure only.

Arrays are torch CUDA tensors.  ``ffi.ffi_call`` does what XLA does with a
legacy (api_version 0) custom call on CUDA: it allocates the result buffers,
passes the operand and result device pointers in one ``void**`` array with
the backend-config bytes, and calls the registered target on the current
stream.  ``custom_vjp`` records the forward / backward rules, and ``vjp``
applies them as jax.vjp would (nondiff arguments first in the backward, one
cotangent per differentiable argument back)."""

import ctypes
import types

import torch


class ShapeDtypeStruct:
    def __init__(self, shape, dtype):
        self.shape = tuple(int(s) for s in shape)
        self.dtype = dtype


class _Ffi:
    def __init__(self):
        self.targets = {}

    def pycapsule(self, fn):
        return fn

    def register_ffi_target(self, name, fn, platform, api_version):
        assert platform == "CUDA" and api_version == 0
        self.targets[name] = fn

    def ffi_call(self, name, results, custom_call_api_version, legacy_backend_config):
        assert custom_call_api_version == 0
        fn = self.targets[name]
        desc = legacy_backend_config
        desc = desc.encode() if isinstance(desc, str) else bytes(desc)
        single = isinstance(results, ShapeDtypeStruct)
        specs = [results] if single else list(results)

        def call(*args):
            outs = [torch.empty(s.shape, dtype=s.dtype, device="cuda") for s in specs]
            bufs = [a.contiguous() for a in args] + outs
            arr = (ctypes.c_void_p * len(bufs))(*[b.data_ptr() for b in bufs])
            fn(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), arr, desc, len(desc))
            return outs[0] if single else tuple(outs)
        return call


class _CustomVjp:
    def __init__(self, fun, nondiff_argnums=()):
        self.fun = fun
        self.nondiff = tuple(nondiff_argnums)
        self.fwd = self.bwd = None

    def defvjp(self, fwd, bwd):
        self.fwd, self.bwd = fwd, bwd

    def __call__(self, *args):
        return self.fun(*args)


def custom_vjp(fun=None, nondiff_argnums=()):
    if fun is None:
        return lambda f: _CustomVjp(f, nondiff_argnums)
    return _CustomVjp(fun, nondiff_argnums)


def vjp(f, *args):
    """(primal out, cotangent function) through f's custom rules."""
    out, res = f.fwd(*args)

    def pullback(g):
        nd = [args[k] for k in f.nondiff]
        cts = f.bwd(*nd, res, g)
        assert len(cts) == len(args) - len(f.nondiff)
        return cts
    return out, pullback


def _asarray(x, dtype=None):
    t = x if torch.is_tensor(x) else torch.tensor(x)
    return t.to(device="cuda", dtype=dtype) if dtype is not None else t.cuda()


def make():
    """(jax, jax.numpy) stand-in modules."""
    jnp = types.ModuleType("jax.numpy")
    jnp.float32, jnp.float64, jnp.int32 = torch.float32, torch.float64, torch.int32
    jnp.asarray = _asarray
    jnp.zeros_like = torch.zeros_like
    jnp.stack = lambda xs: torch.stack(list(xs)).contiguous()
    jnp.broadcast_to = torch.broadcast_to
    jax = types.ModuleType("jax")
    jax.numpy = jnp
    jax.ffi = _Ffi()
    jax.ShapeDtypeStruct = ShapeDtypeStruct
    jax.custom_vjp = custom_vjp
    jax.vjp = vjp
    return jax, jnp
