"""jax.ffi binding of the sm_103a kernels (XLA legacy custom calls,
api_version=0) with jax.custom_vjp rules, so jnp drivers written against
jax_lbm can call the GB300 kernels inside jax.jit / jax.grad.

Import is lazy: ``register()`` needs jax (>= 0.4.35, ``jax.ffi``) and a CUDA
backend.  Each function mirrors the jax_lbm signature it replaces:

    equilibrium(rho, u)                 core/equilibrium.py:90
    compute_density(f)                  core/equilibrium.py:22
    compute_velocity(f, rho)            core/equilibrium.py:51
    bgk(f, tau) / mrt(f, tau)           core/collision.py:46,103   (scalar or per-cell tau)
    smagorinsky_tau(f, tau, cs)         core/collision.py:187
    stream(f, q, periodic_yz)           core/streaming.py:40
    zou_he_inlet(f, velocity, rho_target)  core/boundary.py:35     (uniform or face velocity)
    zou_he_outlet(f, rho_out)           core/boundary.py:127
    momentum_exchange(f_post, f_s, q)   core/forces.py:37
    soft_bounce_back(f, porosity)       geometry/smooth.py:118
"""

import ctypes
import functools

from . import _native as nat

TARGETS = [
    "compute_density", "compute_velocity", "equilibrium", "bgk", "mrt", "smagorinsky_tau",
    "soft_bounce_back", "stream", "zou_he_inlet", "zou_he_outlet", "momentum_exchange",
    "compute_density_vjp", "compute_velocity_vjp", "equilibrium_vjp", "bgk_vjp", "mrt_vjp",
    "smagorinsky_tau_vjp", "soft_bounce_back_vjp", "stream_vjp", "zou_he_inlet_vjp",
    "zou_he_outlet_vjp", "momentum_exchange_vjp",
    # fused solver: n steps with sampled Cd; Cd and dCd/dr from the adjoint
    "run", "cd_and_grad",
]

XLA_SIGNATURE = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p,
                 ctypes.c_size_t]

_registered = False


def descriptor(nx, ny, nz, dtype_code, flags=0, periodic_yz=1, tau_field=0, u_face=0,
               has_rho_target=0, tau=0.0, cs=0.0, u=(0.0, 0.0, 0.0), rho=1.0):
    """Text form of lbm_xla_desc (doubles as exact hex floats)."""
    ints = [nx, ny, nz, dtype_code, flags, int(bool(periodic_yz)), tau_field, u_face,
            has_rho_target]
    dbl = [float(tau), float(cs), float(u[0]), float(u[1]), float(u[2]), float(rho)]
    return "lbm1 " + " ".join(str(int(v)) for v in ints) + " " + " ".join(v.hex() for v in dbl)


class LBMXlaFusedDescC(ctypes.Structure):
    """lbm_xla_fused_desc (include/lbm_gb300.h)."""
    _fields_ = [
        ("params", nat.LBMParamsC),
        ("sphere", nat.LBMSphereC),
        ("n_steps", ctypes.c_int32),
        ("sample_every", ctypes.c_int32),
        ("checkpoint_every", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


def fused_descriptor(params, sphere, n_steps, sample_every=0, checkpoint_every=0):
    """Raw bytes of lbm_xla_fused_desc: params from solver.params_struct,
    sphere from solver.sphere_struct (its radius is replaced by the radius
    operand at run time)."""
    d = LBMXlaFusedDescC()
    d.params = params
    d.sphere = sphere
    d.n_steps = int(n_steps)
    d.sample_every = int(sample_every)
    d.checkpoint_every = int(checkpoint_every)
    return bytes(d)


def xla_target(name):
    """ctypes function pointer of lbm_xla_<name> (usable without jax)."""
    fn = getattr(nat.load(), "lbm_xla_" + name)
    fn.argtypes = XLA_SIGNATURE
    fn.restype = None
    return fn


def _jax():
    import jax
    ffi = getattr(jax, "ffi", None)
    if ffi is None:                                    # jax < 0.4.35
        from jax.extend import ffi                      # type: ignore
    return jax, ffi


def register():
    """Register every lbm_xla_* target with XLA for the CUDA platform."""
    global _registered
    if _registered:
        return
    jax, ffi = _jax()
    for name in TARGETS:
        ffi.register_ffi_target("lbm_" + name, ffi.pycapsule(xla_target(name)), platform="CUDA",
                                api_version=0)
    _registered = True


def _code(x):
    import jax.numpy as jnp
    if x.dtype == jnp.float32:
        return nat.LBM_F32
    if x.dtype == jnp.float64:
        return nat.LBM_F64
    raise TypeError("lbm_gb300 kernels take float32 or float64 arrays")


def _call(name, results, *args, desc):
    jax, ffi = _jax()
    register()
    return ffi.ffi_call("lbm_" + name, results, custom_call_api_version=0,
                        legacy_backend_config=desc)(*args)


def _sds(shape, dtype):
    import jax
    return jax.ShapeDtypeStruct(tuple(shape), dtype)


def _dims(f):
    return int(f.shape[1]), int(f.shape[2]), int(f.shape[3])


def _build():
    """Create the custom_vjp functions (needs jax)."""
    jax, _ = _jax()
    import jax.numpy as jnp

    @jax.custom_vjp
    def compute_density(f):
        nx, ny, nz = _dims(f)
        return _call("compute_density", _sds((nx, ny, nz), f.dtype), f,
                     desc=descriptor(nx, ny, nz, _code(f)))

    def _cd_fwd(f):
        return compute_density(f), f.shape

    def _cd_bwd(shape, g):
        nx, ny, nz = shape[1:]
        return (_call("compute_density_vjp", _sds(shape, g.dtype), g,
                      desc=descriptor(nx, ny, nz, _code(g))),)

    compute_density.defvjp(_cd_fwd, _cd_bwd)

    @jax.custom_vjp
    def compute_velocity(f, rho):
        nx, ny, nz = _dims(f)
        return _call("compute_velocity", _sds((3, nx, ny, nz), f.dtype), f, rho,
                     desc=descriptor(nx, ny, nz, _code(f)))

    def _cv_fwd(f, rho):
        return compute_velocity(f, rho), (f, rho)

    def _cv_bwd(res, g):
        f, rho = res
        nx, ny, nz = _dims(f)
        return tuple(_call("compute_velocity_vjp", (_sds(f.shape, f.dtype), _sds(rho.shape, f.dtype)),
                           f, rho, g, desc=descriptor(nx, ny, nz, _code(f))))

    compute_velocity.defvjp(_cv_fwd, _cv_bwd)

    @jax.custom_vjp
    def equilibrium(rho, u):
        nx, ny, nz = rho.shape
        return _call("equilibrium", _sds((19, nx, ny, nz), rho.dtype), rho, u,
                     desc=descriptor(nx, ny, nz, _code(rho)))

    def _eq_fwd(rho, u):
        return equilibrium(rho, u), (rho, u)

    def _eq_bwd(res, g):
        rho, u = res
        nx, ny, nz = rho.shape
        return tuple(_call("equilibrium_vjp", (_sds(rho.shape, rho.dtype), _sds(u.shape, u.dtype)),
                           rho, u, g, desc=descriptor(nx, ny, nz, _code(rho))))

    equilibrium.defvjp(_eq_fwd, _eq_bwd)

    def _collide(kind):
        # scalar tau: a static argument
        @functools.partial(jax.custom_vjp, nondiff_argnums=(1,))
        def fn(f, tau):
            nx, ny, nz = _dims(f)
            return _call(kind, _sds(f.shape, f.dtype), f,
                         desc=descriptor(nx, ny, nz, _code(f), tau=tau))

        def fwd(f, tau):
            return fn(f, tau), f

        def bwd(tau, f, g):
            nx, ny, nz = _dims(f)
            gf, _ = _call(kind + "_vjp", (_sds(f.shape, f.dtype), _sds(f.shape[1:], f.dtype)),
                          f, g, desc=descriptor(nx, ny, nz, _code(f), tau=tau))
            return (gf,)

        fn.defvjp(fwd, bwd)

        # per-cell tau (smagorinsky_tau's output, collision.py:46-100): an
        # operand, differentiable
        @jax.custom_vjp
        def fn_field(f, tau):
            nx, ny, nz = _dims(f)
            return _call(kind, _sds(f.shape, f.dtype), f, tau,
                         desc=descriptor(nx, ny, nz, _code(f), tau_field=1))

        def fwd_field(f, tau):
            return fn_field(f, tau), (f, tau)

        def bwd_field(res, g):
            f, tau = res
            nx, ny, nz = _dims(f)
            return tuple(_call(kind + "_vjp", (_sds(f.shape, f.dtype), _sds(tau.shape, f.dtype)),
                               f, tau, g, desc=descriptor(nx, ny, nz, _code(f), tau_field=1)))

        fn_field.defvjp(fwd_field, bwd_field)

        def collide(f, tau):
            return fn_field(f, tau) if getattr(tau, "ndim", 0) else fn(f, tau)

        return collide, fn, fn_field

    bgk, _bgk_scalar, _bgk_field = _collide("bgk")
    mrt, _mrt_scalar, _mrt_field = _collide("mrt")

    @functools.partial(jax.custom_vjp, nondiff_argnums=(1, 2))
    def smagorinsky_tau(f, tau, cs=0.1):
        nx, ny, nz = _dims(f)
        return _call("smagorinsky_tau", _sds((nx, ny, nz), f.dtype), f,
                     desc=descriptor(nx, ny, nz, _code(f), tau=tau, cs=cs))

    def _sm_fwd(f, tau, cs):
        return smagorinsky_tau(f, tau, cs), f

    def _sm_bwd(tau, cs, f, g):
        nx, ny, nz = _dims(f)
        gf, _ = _call("smagorinsky_tau_vjp", (_sds(f.shape, f.dtype), _sds((nx, ny, nz), f.dtype)),
                      f, g, desc=descriptor(nx, ny, nz, _code(f), tau=tau, cs=cs))
        return (gf,)

    smagorinsky_tau.defvjp(_sm_fwd, _sm_bwd)

    @jax.custom_vjp
    def soft_bounce_back(f, porosity):
        nx, ny, nz = _dims(f)
        return _call("soft_bounce_back", _sds(f.shape, f.dtype), f, porosity,
                     desc=descriptor(nx, ny, nz, _code(f)))

    def _sb_fwd(f, p):
        return soft_bounce_back(f, p), (f, p)

    def _sb_bwd(res, g):
        f, p = res
        nx, ny, nz = _dims(f)
        return tuple(_call("soft_bounce_back_vjp", (_sds(f.shape, f.dtype), _sds(p.shape, p.dtype)),
                           f, p, g, desc=descriptor(nx, ny, nz, _code(f))))

    soft_bounce_back.defvjp(_sb_fwd, _sb_bwd)

    @functools.partial(jax.custom_vjp, nondiff_argnums=(2,))
    def stream(f, q, periodic_yz=True):
        nx, ny, nz = _dims(f)
        return _call("stream", _sds(f.shape, f.dtype), f, q,
                     desc=descriptor(nx, ny, nz, _code(f), periodic_yz=periodic_yz))

    def _st_fwd(f, q, periodic_yz):
        return stream(f, q, periodic_yz), (f, q)

    def _st_bwd(periodic_yz, res, g):
        f, q = res
        nx, ny, nz = _dims(f)
        return tuple(_call("stream_vjp", (_sds(f.shape, f.dtype), _sds(q.shape, q.dtype)), f, q, g,
                           desc=descriptor(nx, ny, nz, _code(f), periodic_yz=periodic_yz)))

    stream.defvjp(_st_fwd, _st_bwd)

    def _inlet_desc(f, velocity, rho_target, face):
        nx, ny, nz = _dims(f)
        rt = rho_target is not None
        return descriptor(nx, ny, nz, _code(f), u_face=int(face), has_rho_target=int(rt),
                          u=(0.0, 0.0, 0.0) if face else tuple(float(c) for c in velocity),
                          rho=float(rho_target) if rt else 1.0)

    # uniform velocity: static arguments
    @functools.partial(jax.custom_vjp, nondiff_argnums=(1, 2))
    def _zi_uniform(f, velocity, rho_target):
        return _call("zou_he_inlet", _sds(f.shape, f.dtype), f,
                     desc=_inlet_desc(f, velocity, rho_target, False))

    def _zi_fwd(f, velocity, rho_target):
        return _zi_uniform(f, velocity, rho_target), f

    def _zi_bwd(velocity, rho_target, f, g):
        nx, ny, nz = _dims(f)
        gf, _ = _call("zou_he_inlet_vjp", (_sds(f.shape, f.dtype), _sds((3, ny, nz), f.dtype)), f, g,
                      desc=_inlet_desc(f, velocity, rho_target, False))
        return (gf,)

    _zi_uniform.defvjp(_zi_fwd, _zi_bwd)

    # a (3, ny, nz) velocity face (a parabolic profile, examples/01): an
    # operand, differentiable
    @functools.partial(jax.custom_vjp, nondiff_argnums=(2,))
    def _zi_face(f, face, rho_target):
        return _call("zou_he_inlet", _sds(f.shape, f.dtype), f, face,
                     desc=_inlet_desc(f, None, rho_target, True))

    def _zf_fwd(f, face, rho_target):
        return _zi_face(f, face, rho_target), (f, face)

    def _zf_bwd(rho_target, res, g):
        f, face = res
        return tuple(_call("zou_he_inlet_vjp", (_sds(f.shape, f.dtype), _sds(face.shape, f.dtype)),
                           f, face, g, desc=_inlet_desc(f, None, rho_target, True)))

    _zi_face.defvjp(_zf_fwd, _zf_bwd)

    def zou_he_inlet(f, velocity, rho_target=None):
        """velocity: three components, each a scalar or a (ny, nz) face, or a
        (3, ny, nz) array (boundary.py:35-124)."""
        if getattr(velocity, "ndim", 0) == 3:
            return _zi_face(f, velocity, rho_target)
        if any(getattr(c, "ndim", 0) for c in velocity):
            ny, nz = int(f.shape[2]), int(f.shape[3])
            face = jnp.stack([jnp.broadcast_to(jnp.asarray(c, f.dtype), (ny, nz))
                              for c in velocity])
            return _zi_face(f, face, rho_target)
        return _zi_uniform(f, tuple(float(c) for c in velocity), rho_target)

    @functools.partial(jax.custom_vjp, nondiff_argnums=(1,))
    def zou_he_outlet(f, rho_out=1.0):
        nx, ny, nz = _dims(f)
        return _call("zou_he_outlet", _sds(f.shape, f.dtype), f,
                     desc=descriptor(nx, ny, nz, _code(f), rho=rho_out))

    def _zo_fwd(f, rho_out):
        return zou_he_outlet(f, rho_out), f

    def _zo_bwd(rho_out, f, g):
        nx, ny, nz = _dims(f)
        gf, _ = _call("zou_he_outlet_vjp", (_sds(f.shape, f.dtype), _sds((ny, nz), f.dtype)), f, g,
                      desc=descriptor(nx, ny, nz, _code(f), rho=rho_out))
        return (gf,)

    zou_he_outlet.defvjp(_zo_fwd, _zo_bwd)

    @jax.custom_vjp
    def momentum_exchange(f_post, f_streamed, q):
        nx, ny, nz = _dims(f_post)
        out = _call("momentum_exchange", _sds((3,), jnp.float64), f_post, f_streamed, q,
                    desc=descriptor(nx, ny, nz, _code(f_post)))
        return out.astype(f_post.dtype)

    def _me_fwd(fp, fs, q):
        return momentum_exchange(fp, fs, q), (q, fp.dtype)

    def _me_bwd(res, g):
        q, dt = res
        nx, ny, nz = _dims(q)
        gp, gs = _call("momentum_exchange_vjp", (_sds(q.shape, dt), _sds(q.shape, dt)), q,
                       g.astype(jnp.float64), desc=descriptor(nx, ny, nz, _code(q)))
        return gp, gs, jnp.zeros_like(q)

    momentum_exchange.defvjp(_me_fwd, _me_bwd)

    def fused_run(f0, radius, desc, n_samples):
        """(f after the steps, samples (n_samples, 4), status) of lbm_xla_run
        (examples/10's scan of steps with a sampled Cd)."""
        return _call("run", (_sds(f0.shape, f0.dtype), _sds((max(n_samples, 1), 4), jnp.float64),
                             _sds((1,), jnp.int32)),
                     f0, jnp.asarray(radius, jnp.float64).reshape(1), desc=desc)

    def simulate_cd(desc):
        """(cd_of, cd_and_grad) on the fused solver for a fixed descriptor:
        cd_of(radius, f0) is examples/11's simulate_cd, differentiable in the
        radius through the hand-written adjoint (jax.custom_vjp over
        lbm_xla_cd_and_grad); cd_and_grad returns (cd, dcd_dr, dcd_dq,
        status) as arrays."""

        def cd_and_grad(radius, f0):
            return _call("cd_and_grad", (_sds((1,), jnp.float64), _sds((1,), jnp.float64),
                                         _sds(f0.shape, f0.dtype), _sds((1,), jnp.int32)),
                         f0, jnp.asarray(radius, jnp.float64).reshape(1), desc=desc)

        @jax.custom_vjp
        def cd_of(radius, f0):
            return cd_and_grad(radius, f0)[0][0]

        def fwd(radius, f0):
            cd, g, _, _ = cd_and_grad(radius, f0)
            return cd[0], (g[0], f0)

        def bwd(res, ct):
            g, f0 = res
            return (ct * g, jnp.zeros_like(f0))

        cd_of.defvjp(fwd, bwd)
        return cd_of, cd_and_grad

    return dict(compute_density=compute_density, compute_velocity=compute_velocity,
                equilibrium=equilibrium, bgk=bgk, mrt=mrt, smagorinsky_tau=smagorinsky_tau,
                soft_bounce_back=soft_bounce_back, stream=stream, zou_he_inlet=zou_he_inlet,
                zou_he_outlet=zou_he_outlet, momentum_exchange=momentum_exchange,
                fused_run=fused_run, simulate_cd=simulate_cd,
                _bgk_scalar=_bgk_scalar, _mrt_scalar=_mrt_scalar, _bgk_field=_bgk_field,
                _mrt_field=_mrt_field, _zi_uniform=_zi_uniform,
                _zi_face=_zi_face)


_fns = None


def __getattr__(name):
    """Module-level access to the jax functions, built on first use."""
    global _fns
    if name in ("compute_density", "compute_velocity", "equilibrium", "bgk", "mrt",
                "smagorinsky_tau", "soft_bounce_back", "stream", "zou_he_inlet", "zou_he_outlet",
                "momentum_exchange", "fused_run", "simulate_cd"):
        if _fns is None:
            _fns = _build()
        return _fns[name]
    raise AttributeError(name)
