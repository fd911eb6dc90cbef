"""ctypes binding of ``lib/liblbm_gb300.so`` (C ABI: ``include/lbm_gb300.h``).

The library is the only compute path of this package: there is no CPU
fallback.  If it is missing, every call raises :class:`NativeLibraryMissing`
telling the user to build it.
"""

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "liblbm_gb300.so")

LBM_OK = 0
LBM_ERR_ARG = 1
LBM_ERR_ALIGN = 2
LBM_ERR_UNSUPPORTED = 3
LBM_ERR_TIMEOUT = 4
LBM_ERR_CUDA = 5
LBM_ERR_NOMEM = 6
LBM_ERR_STATE = 7

LBM_F32, LBM_F64, LBM_F16, LBM_BF16 = 0, 1, 2, 3
LBM_BGK, LBM_MRT = 0, 1
LBM_GUARD_OFF, LBM_GUARD_PRE, LBM_GUARD_POST = 0, 1, 2
LBM_POROSITY_NONE, LBM_POROSITY_HARD, LBM_POROSITY_SOFT = 0, 1, 2
LBM_Q_HALFWAY, LBM_Q_BOUZIDI = 0, 1
LBM_SPHERE_DIST_MASK, LBM_SPHERE_SIGMOID_MASK = 0, 1
LBM_LOSS_CD, LBM_LOSS_TARGET_CD = 0, 1
LBM_STREAM_AB, LBM_STREAM_AA = 0, 1


class NativeLibraryMissing(RuntimeError):
    pass


class LBMError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


STATUS_NAMES = {
    LBM_OK: "LBM_OK", LBM_ERR_ARG: "LBM_ERR_ARG", LBM_ERR_ALIGN: "LBM_ERR_ALIGN",
    LBM_ERR_UNSUPPORTED: "LBM_ERR_UNSUPPORTED", LBM_ERR_TIMEOUT: "LBM_ERR_TIMEOUT",
    LBM_ERR_CUDA: "LBM_ERR_CUDA", LBM_ERR_NOMEM: "LBM_ERR_NOMEM", LBM_ERR_STATE: "LBM_ERR_STATE",
}


class LBMParamsC(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("storage", ctypes.c_int),
        ("collision", ctypes.c_int),
        ("tau", ctypes.c_double),
        ("use_smagorinsky", ctypes.c_int),
        ("smagorinsky_cs", ctypes.c_double),
        ("periodic_yz", ctypes.c_int),
        ("guard", ctypes.c_int),
        ("inlet_velocity", ctypes.c_double * 3),
        ("rho_out", ctypes.c_double),
        ("u_ref", ctypes.c_double),
        ("area_min", ctypes.c_double),
        ("exact_constants", ctypes.c_int),
    ]


class LBMSphereC(ctypes.Structure):
    _fields_ = [
        ("center", ctypes.c_double * 3),
        ("radius", ctypes.c_double),
        ("sharpness", ctypes.c_double),
        ("kind", ctypes.c_int),
        ("q_mode", ctypes.c_int),
        ("porosity", ctypes.c_int),
        ("disc_floor", ctypes.c_double),
        ("denom_eps", ctypes.c_double),
    ]


class LBMAdamC(ctypes.Structure):
    _fields_ = [
        ("lr", ctypes.c_double),
        ("b1", ctypes.c_double),
        ("b2", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("r_min", ctypes.c_double),
        ("r_max", ctypes.c_double),
        ("loss", ctypes.c_int),
        ("target_cd", ctypes.c_double),
    ]


_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_ll = ctypes.c_longlong

# name -> argtypes (restype is int for every entry unless listed in _RESTYPES)
SIGNATURES = {
    "lbm_api_version": [],
    "lbm_status_string": [_i],
    "lbm_last_error": [],
    "lbm_struct_size": [_i],
    "lbm_create": [ctypes.POINTER(LBMParamsC), ctypes.POINTER(_vp)],
    "lbm_destroy": [_vp],
    "lbm_set_geometry_sphere": [_vp, ctypes.POINTER(LBMSphereC), _vp],
    "lbm_set_geometry_mask": [_vp, _vp, _vp, _d, _vp, _vp],
    "lbm_set_inlet_profile": [_vp, _vp, _vp],
    "lbm_set_state": [_vp, _vp, _vp],
    "lbm_get_state": [_vp, _vp, _vp],
    "lbm_get_state_and_step": [_vp, _vp, _vp],
    "lbm_set_state_host": [_vp, _vp, _vp],
    "lbm_get_state_host": [_vp, _vp, _vp],
    "lbm_run": [_vp, _i, _i, _vp, _vp],
    "lbm_set_streaming": [_vp, _i],
    "lbm_cd_and_grad": [_vp, _i, _i, ctypes.POINTER(_d), ctypes.POINTER(_d), _vp, _vp, _vp],
    "lbm_get_projected_area": [_vp, ctypes.POINTER(_d)],
    "lbm_get_link_count": [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i)],
    "lbm_get_guard_resets": [_vp, ctypes.POINTER(ctypes.c_ulonglong), _vp],
    "lbm_get_steps": [_vp, ctypes.POINTER(_ll)],
    "lbm_plan_checkpoints": [_i, ctypes.c_longlong, ctypes.POINTER(_i)],
    "lbm_get_adjoint_plan": [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i),
                             ctypes.POINTER(ctypes.c_ulonglong)],
    "lbm_release_workspace": [_vp],
    "lbm_vjp_run": [_vp, _i, _i, _vp, _vp, _vp, _vp],
    "lbm_set_workspace_limit": [_vp, ctypes.c_ulonglong],
    # geometry builders
    "lbm_sphere_fields": [_i, _i, _i, _i, ctypes.POINTER(LBMSphereC), _vp, _vp, _vp, _vp, _vp],
    "lbm_box_fields": [_i, _i, _i, _i, ctypes.POINTER(_d), ctypes.POINTER(_d), _vp, _vp, _vp],
    "lbm_q_from_solid": [_i, _vp, _d, _vp, _i, _i, _i, _vp],
    # per-op drop-ins
    "lbm_compute_density": [_i, _vp, _vp, _i, _i, _i, _vp],
    "lbm_compute_velocity": [_i, _vp, _vp, _vp, _i, _i, _i, _vp],
    "lbm_equilibrium": [_i, _vp, _vp, _vp, _i, _i, _i, _i, _vp],
    "lbm_bgk": [_i, _vp, _vp, _d, _vp, _i, _i, _i, _i, _vp],
    "lbm_mrt": [_i, _vp, _vp, _d, _vp, _i, _i, _i, _i, _vp],
    "lbm_smagorinsky_tau": [_i, _vp, _d, _d, _vp, _i, _i, _i, _i, _vp],
    "lbm_soft_bounce_back": [_i, _vp, _vp, _vp, _i, _i, _i, _vp],
    "lbm_stream": [_i, _vp, _vp, _i, _vp, _i, _i, _i, _vp],
    "lbm_zou_he_inlet": [_i, _vp, _vp, ctypes.POINTER(_d), _i, _d, _vp, _i, _i, _i, _vp],
    "lbm_zou_he_outlet": [_i, _vp, _d, _vp, _i, _i, _i, _vp],
    "lbm_momentum_exchange": [_i, _vp, _vp, _vp, _vp, _i, _i, _i, _vp],
    "lbm_drag_coefficient": [_vp, _d, _d, _d, _vp, _vp],
    "lbm_projected_area": [_vp, _i, _vp, _i, _i, _i, _vp],
    "lbm_compute_density_vjp": [_i, _vp, _vp, _i, _i, _i, _vp],
    "lbm_compute_velocity_vjp": [_i, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp],
    "lbm_equilibrium_vjp": [_i, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp],
    "lbm_bgk_vjp": [_i, _vp, _vp, _d, _vp, _vp, _vp, _i, _i, _i, _i, _vp],
    "lbm_mrt_vjp": [_i, _vp, _vp, _d, _vp, _vp, _vp, _i, _i, _i, _i, _vp],
    "lbm_smagorinsky_tau_vjp": [_i, _vp, _d, _d, _vp, _vp, _vp, _i, _i, _i, _i, _vp],
    "lbm_soft_bounce_back_vjp": [_i, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp],
    "lbm_stream_vjp": [_i, _vp, _vp, _i, _vp, _vp, _vp, _i, _i, _i, _vp],
    "lbm_zou_he_inlet_vjp": [_i, _vp, _vp, ctypes.POINTER(_d), _i, _d, _vp, _vp, _vp, _i, _i,
                             _i, _vp],
    "lbm_zou_he_outlet_vjp": [_i, _vp, _d, _vp, _vp, _vp, _i, _i, _i, _vp],
    "lbm_momentum_exchange_vjp": [_i, _vp, _vp, _vp, _vp, _i, _i, _i, _vp],
    "lbm_momentum_exchange_noalloc": [_i, _vp, _vp, _vp, _vp, _i, _i, _i, _vp],
    # batched instances
    "lbm_batch_create": [ctypes.POINTER(LBMParamsC), _i, ctypes.POINTER(_vp)],
    "lbm_batch_destroy": [_vp],
    "lbm_batch_size": [_vp, ctypes.POINTER(_i), ctypes.POINTER(_ll)],
    "lbm_batch_instance": [_vp, _i, ctypes.POINTER(_vp)],
    "lbm_batch_set_spheres": [_vp, ctypes.POINTER(LBMSphereC), _vp],
    "lbm_batch_set_equilibrium": [_vp, _vp],
    "lbm_batch_set_state": [_vp, _i, _vp, _vp],
    "lbm_batched_run": [_vp, _i, _i, _vp, _vp],
    "lbm_batch_cd_and_grad": [_vp, _i, _i, _i, ctypes.POINTER(_d), ctypes.POINTER(_d), _vp],
    "lbm_batch_optimize": [_vp, _i, _i, _i, ctypes.POINTER(LBMAdamC), _i, ctypes.POINTER(_d),
                           ctypes.POINTER(_d), ctypes.POINTER(_d), ctypes.POINTER(_d), _vp],
    "lbm_batch_get_radii": [_vp, ctypes.POINTER(_d)],
    "lbm_batch_set_block": [_vp, _i],
    "lbm_batch_autotune": [_vp, _i, _i, ctypes.POINTER(_i), ctypes.POINTER(_i), _vp],
    "lbm_batch_get_plan": [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i),
                           ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(_d)],
    "lbm_batch_graph_launches": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "lbm_batch_set_workspace_limit": [_vp, ctypes.c_ulonglong],
}
_RESTYPES = {"lbm_status_string": ctypes.c_char_p, "lbm_last_error": ctypes.c_char_p,
             "lbm_struct_size": ctypes.c_size_t}

_lock = threading.Lock()
_lib = None


def load(path=LIB_PATH):
    """Load the library once and attach the prototypes."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise NativeLibraryMissing(
                "CUDA library %s not found; build it with "
                "`python -c \"import __graft_entry__ as g; g.build()\"` or "
                "`python -m lbm_jax_autodiff_gb300.build`" % path)
        lib = ctypes.CDLL(path)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = lib
        return lib


def check(status):
    if status != LBM_OK:
        msg = load().lbm_last_error()
        raise LBMError(status, msg.decode() if msg else "")
    return status


def call(name, *args):
    return check(getattr(load(), name)(*args))
