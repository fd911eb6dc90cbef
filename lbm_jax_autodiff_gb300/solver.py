"""Fused GB300 solver handle: the hot path of jax_lbm as one object.

``Simulation`` owns an ``lbm_sim`` (include/lbm_gb300.h).  It replaces the
reference's ``step``/``simulate`` loops and the examples' ``lax.scan`` drivers
(state.py:87-230, examples/10:162-193, examples/11:139-165): geometry,
state, time stepping with sampled momentum-exchange Cd, and (see
``cd_and_grad``) the shape gradient.

Tensors crossing this API are torch CUDA tensors in the reference layout:
populations (19, nx, ny, nz), fields (nx, ny, nz).
"""

import ctypes

import torch

from . import _native as nat

_STORAGE = {"fp32": nat.LBM_F32, "fp64": nat.LBM_F64, "fp16": nat.LBM_F16, "bf16": nat.LBM_BF16}
_GUARD = {"off": nat.LBM_GUARD_OFF, "pre": nat.LBM_GUARD_PRE, "post": nat.LBM_GUARD_POST}


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(None)


def _require_cuda(t, name, dtype=None, numel=None):
    if not (torch.is_tensor(t) and t.is_cuda):
        raise TypeError("%s must be a CUDA tensor" % name)
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    if dtype is not None and t.dtype != dtype:
        raise TypeError("%s must have dtype %s, got %s" % (name, dtype, t.dtype))
    if numel is not None and t.numel() != numel:
        raise ValueError("%s must have %d elements, got %d" % (name, numel, t.numel()))


def params_struct(nx, ny, nz, tau, collision="mrt", storage="fp32", use_smagorinsky=False,
                  smagorinsky_cs=0.1, periodic_yz=True, guard="off",
                  inlet_velocity=(0.05, 0.0, 0.0), rho_out=1.0, u_ref=None, area_min=1.0,
                  exact_constants=False):
    """lbm_params of one domain (validated)."""
    if storage not in _STORAGE:
        raise ValueError("storage must be one of %s" % sorted(_STORAGE))
    if collision not in ("bgk", "mrt"):
        raise ValueError("collision must be 'bgk' or 'mrt'")
    if guard not in _GUARD:
        raise ValueError("guard must be one of %s" % sorted(_GUARD))
    inlet_velocity = tuple(float(v) for v in inlet_velocity)
    p = nat.LBMParamsC()
    p.nx, p.ny, p.nz = int(nx), int(ny), int(nz)
    p.storage = _STORAGE[storage]
    p.collision = nat.LBM_MRT if collision == "mrt" else nat.LBM_BGK
    p.tau = float(tau)
    p.use_smagorinsky = int(bool(use_smagorinsky))
    p.smagorinsky_cs = float(smagorinsky_cs)
    p.periodic_yz = int(bool(periodic_yz))
    p.guard = _GUARD[guard]
    for k in range(3):
        p.inlet_velocity[k] = inlet_velocity[k]
    p.rho_out = float(rho_out)
    p.u_ref = float(u_ref if u_ref is not None else inlet_velocity[0])
    p.area_min = float(area_min)
    p.exact_constants = int(bool(exact_constants))
    return p


def sphere_struct(radius, center=(0.0, 0.0, 0.0), sharpness=20.0, kind="sigmoid",
                  q_mode="bouzidi", porosity="hard", disc_floor=None, denom_eps=1e-20):
    """lbm_sphere in the reference world frame (see Simulation.set_sphere)."""
    s = nat.LBMSphereC()
    for k in range(3):
        s.center[k] = float(center[k])
    s.radius = float(radius)
    s.sharpness = float(sharpness)
    s.kind = nat.LBM_SPHERE_SIGMOID_MASK if kind == "sigmoid" else nat.LBM_SPHERE_DIST_MASK
    s.q_mode = nat.LBM_Q_BOUZIDI if q_mode == "bouzidi" else nat.LBM_Q_HALFWAY
    s.porosity = {"none": nat.LBM_POROSITY_NONE, "hard": nat.LBM_POROSITY_HARD,
                  "soft": nat.LBM_POROSITY_SOFT}[porosity]
    if disc_floor is None:
        disc_floor = 1e-10 if kind == "sigmoid" else 0.0
    s.disc_floor = float(disc_floor)
    s.denom_eps = float(denom_eps)
    return s


class Simulation:
    """One D3Q19 domain on the current CUDA device.

    collision: "bgk" | "mrt"; storage: "fp32" | "fp64" | "fp16" | "bf16"
    (16-bit storage keeps f_i - f_eq,i(1, (U, 0, 0)), arithmetic in fp32); guard: "off" |
    "pre" (examples/10:163-168) | "post" (state.py:161-169).
    """

    def __init__(self, nx, ny, nz, tau, collision="mrt", storage="fp32",
                 use_smagorinsky=False, smagorinsky_cs=0.1, periodic_yz=True, guard="off",
                 inlet_velocity=(0.05, 0.0, 0.0), rho_out=1.0, u_ref=None, area_min=1.0,
                 exact_constants=False):
        nat.load()
        p = params_struct(nx, ny, nz, tau, collision, storage, use_smagorinsky, smagorinsky_cs,
                          periodic_yz, guard, inlet_velocity, rho_out, u_ref, area_min,
                          exact_constants)
        self.shape = (int(nx), int(ny), int(nz))
        self.n = nx * ny * nz
        self.storage = storage
        self.dtype = torch.float64 if storage == "fp64" else torch.float32
        self.collision = collision
        self.tau = float(tau)
        self.inlet_velocity = tuple(float(v) for v in inlet_velocity)
        self._params = p
        self._h = ctypes.c_void_p()
        nat.call("lbm_create", ctypes.byref(p), ctypes.byref(self._h))
        self._keep = {}

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            torch.cuda.synchronize()
            nat.load().lbm_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- geometry -----------------------------------------------------------
    def set_sphere(self, radius, center=(0.0, 0.0, 0.0), sharpness=20.0, kind="sigmoid",
                   q_mode="bouzidi", porosity="hard", disc_floor=None, denom_eps=1e-20):
        """Sphere in the reference world frame.

        kind="dist": solid = dist^2 <= r^2, q floor 0 (create_sphere,
        primitives.py:56-174).  kind="sigmoid": solid = sigmoid(alpha (r-d)) > 0.5,
        q floor 1e-10 (smooth_sphere_geometry / examples/11:56-119).
        q_mode: "bouzidi" (ray-sphere q(r)) | "halfway" (q = 0.5).
        porosity: "hard" (bounce-back on solid cells) | "soft" (sigmoid blend).
        """
        s = sphere_struct(radius, center, sharpness, kind, q_mode, porosity, disc_floor,
                          denom_eps)
        self.sphere = dict(radius=float(radius), center=tuple(center), sharpness=float(sharpness),
                           kind=kind, q_mode=q_mode, porosity=porosity)
        nat.call("lbm_set_geometry_sphere", self._h, ctypes.byref(s), _stream())

    def set_mask(self, solid, q=None, default_q=0.5, porosity=None):
        """Mask geometry: solid int32 (nx,ny,nz) (0 fluid, 1 body, 2 ground); q
        (19,nx,ny,nz) or None for compute_q_from_solid(default_q); porosity
        (nx,ny,nz) or None for hard bounce-back on solid >= 1."""
        _require_cuda(solid, "solid", torch.int32, self.n)
        if q is not None:
            _require_cuda(q, "q", self.dtype, 19 * self.n)
        if porosity is not None:
            _require_cuda(porosity, "porosity", self.dtype, self.n)
        nat.call("lbm_set_geometry_mask", self._h, _ptr(solid), _ptr(q), float(default_q),
                 _ptr(porosity), _stream())

    def set_inlet_profile(self, u_face):
        """Per-(y, z) inlet velocity (3, ny, nz); None restores the uniform inlet."""
        if u_face is not None:
            _require_cuda(u_face, "u_face", self.dtype, 3 * self.shape[1] * self.shape[2])
        self._keep["u_face"] = u_face
        nat.call("lbm_set_inlet_profile", self._h, _ptr(u_face), _stream())

    # -- state --------------------------------------------------------------
    def set_state(self, f):
        _require_cuda(f, "f", self.dtype, 19 * self.n)
        nat.call("lbm_set_state", self._h, _ptr(f), _stream())

    def set_state_host(self, f):
        """set_state from a host (CPU) tensor, pinned for an asynchronous
        copy: one host-to-device copy into the solver's own buffer."""
        if not (torch.is_tensor(f) and not f.is_cuda and f.is_contiguous()):
            raise TypeError("f must be a contiguous CPU tensor")
        if f.dtype != self.dtype or f.numel() != 19 * self.n:
            raise ValueError("f must be a %s tensor of %d elements" % (self.dtype, 19 * self.n))
        self._keep["f_host_in"] = f
        nat.call("lbm_set_state_host", self._h, _ptr(f), _stream())

    def get_state_host(self, out):
        """The reference f after the steps run so far, into a host (CPU)
        tensor (pinned for an asynchronous copy); asynchronous on the current
        stream -- synchronise before reading ``out``."""
        if not (torch.is_tensor(out) and not out.is_cuda and out.is_contiguous()):
            raise TypeError("out must be a contiguous CPU tensor")
        if out.dtype != self.dtype or out.numel() != 19 * self.n:
            raise ValueError("out must be a %s tensor of %d elements" % (self.dtype, 19 * self.n))
        nat.call("lbm_get_state_host", self._h, _ptr(out), _stream())
        return out

    def get_state(self, out=None):
        if out is None:
            out = torch.empty((19,) + self.shape, dtype=self.dtype, device="cuda")
        _require_cuda(out, "out", self.dtype, 19 * self.n)
        nat.call("lbm_get_state", self._h, _ptr(out), _stream())
        return out

    def get_state_and_step(self, out=None):
        """get_state(), then run(1), in one launch that reads the state once
        (lbm_get_state_and_step): returns f of the current step and leaves the
        handle one step further on."""
        if out is None:
            out = torch.empty((19,) + self.shape, dtype=self.dtype, device="cuda")
        _require_cuda(out, "out", self.dtype, 19 * self.n)
        nat.call("lbm_get_state_and_step", self._h, _ptr(out), _stream())
        return out

    def equilibrium_state(self, ux=None):
        """f_eq(rho=1, u=(ux,0,0)) built on the host in the reference formula."""
        from .core.lattice import equilibrium_uniform
        ux = self.inlet_velocity[0] if ux is None else ux
        return equilibrium_uniform(self.shape, ux, self.dtype,
                                   exact=bool(self._params.exact_constants))

    # -- stepping -----------------------------------------------------------
    def set_streaming(self, mode):
        """"ab" (two population buffers, the default) or "aa" (one buffer
        updated in place: half the state memory of a forward run; periodic
        y/z, FP32 / FP64 storage).  Set the state again after switching."""
        nat.call("lbm_set_streaming", self._h,
                 {"ab": nat.LBM_STREAM_AB, "aa": nat.LBM_STREAM_AA}[mode])

    def run(self, n_steps, sample_every=0, samples=None):
        """Advance n_steps.  With sample_every > 0 returns a (n_samples, 4)
        float64 CUDA tensor of (Fx, Fy, Fz, Cd) after every sample_every-th step."""
        n_steps = int(n_steps)
        if sample_every:
            ns = n_steps // int(sample_every)
            if samples is None:
                samples = torch.zeros((max(ns, 1), 4), dtype=torch.float64, device="cuda")
            _require_cuda(samples, "samples", torch.float64)
            if samples.numel() < 4 * ns:
                raise ValueError("samples buffer too small")
        nat.call("lbm_run", self._h, n_steps, int(sample_every), _ptr(samples), _stream())
        return samples

    def cd_and_grad(self, n_steps, checkpoint_every=0, dcd_dq=False, dcd_df0=False):
        """Cd after n_steps from the state set by set_state, and dCd/dr.

        The shape gradient flows through the ray-sphere q(r) (q_mode
        "bouzidi") and the sigmoid porosity (porosity "soft"); with
        q_mode "halfway" and porosity "hard" it is exactly 0.0, as in the
        reference's halfway_hard mode.  checkpoint_every=K stores the
        last K steps' populations from the forward pass and recomputes earlier
        segments of K steps from checkpoints (0: the longest K that fits in
        free HBM).
        Returns (cd, dcd_dr) or (cd, dcd_dr, extras) when dcd_dq / dcd_df0 are
        requested (dense (19, nx, ny, nz) CUDA tensors).
        """
        cd, gr = ctypes.c_double(), ctypes.c_double()
        extras = {}
        dq = df0 = None
        if dcd_dq:
            dq = extras["dcd_dq"] = torch.empty((19,) + self.shape, dtype=self.dtype, device="cuda")
        if dcd_df0:
            df0 = extras["dcd_df0"] = torch.empty((19,) + self.shape, dtype=self.dtype,
                                                  device="cuda")
        nat.call("lbm_cd_and_grad", self._h, int(n_steps), int(checkpoint_every),
                 ctypes.byref(cd), ctypes.byref(gr), _ptr(dq), _ptr(df0), _stream())
        if extras:
            return cd.value, gr.value, extras
        return cd.value, gr.value

    @property
    def adjoint_plan(self):
        """(segment steps, recomputed steps, workspace bytes) of the last cd_and_grad."""
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_ulonglong()
        nat.call("lbm_get_adjoint_plan", self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def release_workspace(self):
        nat.call("lbm_release_workspace", self._h)

    def set_workspace_limit(self, max_bytes):
        """Cap the adjoint population workspace that cd_and_grad's automatic
        plan (checkpoint_every=0) may take; 0 removes the cap (free device
        memory minus a reserve).  Use it beside a framework that holds a
        memory pool."""
        nat.call("lbm_set_workspace_limit", self._h, int(max_bytes))

    # -- queries ------------------------------------------------------------
    @property
    def projected_area(self):
        a = ctypes.c_double()
        nat.call("lbm_get_projected_area", self._h, ctypes.byref(a))
        return a.value

    @property
    def link_count(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        nat.call("lbm_get_link_count", self._h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    @property
    def guard_resets(self):
        c = ctypes.c_ulonglong()
        nat.call("lbm_get_guard_resets", self._h, ctypes.byref(c), _stream())
        return c.value

    @property
    def steps(self):
        c = ctypes.c_longlong()
        nat.call("lbm_get_steps", self._h, ctypes.byref(c))
        return c.value
