"""Batched instances: many independent sphere domains advanced together.

``Batch`` owns an ``lbm_batch`` (include/lbm_gb300.h): instances of
different grid sizes, radii and boundary modes share one kernel launch per
step, the gradient evaluation of all of them can run as one captured CUDA
graph, and ``optimize`` adds the Adam step on every radius inside it.  It is
the batched form of the reference's optimisation driver
(examples/11:168-195, optax.adam + clip on r) with the losses of
optim/losses.py (minimize_cd_loss, target_cd_loss).
"""

import ctypes

import numpy as np
import torch

from . import _native as nat
from .solver import _ptr, _require_cuda, _stream, params_struct, sphere_struct


class Batch:
    """instances: list of dicts of Simulation keyword arguments (nx, ny, nz,
    tau required; storage must be fp32; collision and guard shared)."""

    def __init__(self, instances):
        nat.load()
        if not instances:
            raise ValueError("a batch needs at least one instance")
        params = []
        for kw in instances:
            kw = dict(kw)
            if kw.get("storage", "fp32") != "fp32":
                raise ValueError("batched instances use fp32 storage")
            params.append(params_struct(**kw))
        self.count = len(params)
        self.shapes = [(p.nx, p.ny, p.nz) for p in params]
        self.inlet_velocity = [float(p.inlet_velocity[0]) for p in params]
        arr = (nat.LBMParamsC * self.count)(*params)
        self._h = ctypes.c_void_p()
        nat.call("lbm_batch_create", arr, self.count, ctypes.byref(self._h))
        c, cells = ctypes.c_int(), ctypes.c_longlong()
        nat.call("lbm_batch_size", self._h, ctypes.byref(c), ctypes.byref(cells))
        self.cells = cells.value
        self.spheres = [None] * self.count

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            torch.cuda.synchronize()
            nat.load().lbm_batch_destroy(self._h)
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

    # -- setup --------------------------------------------------------------
    def set_spheres(self, spheres):
        """One dict of Simulation.set_sphere arguments per instance."""
        if len(spheres) != self.count:
            raise ValueError("need %d spheres" % self.count)
        arr = (nat.LBMSphereC * self.count)(*[sphere_struct(**sp) for sp in spheres])
        nat.call("lbm_batch_set_spheres", self._h, arr, _stream())
        self.spheres = [dict(sp) for sp in spheres]

    def set_equilibrium(self):
        """f_0 = f_eq(1, (U, 0, 0)) on every instance."""
        nat.call("lbm_batch_set_equilibrium", self._h, _stream())

    def set_state(self, i, f):
        nx, ny, nz = self.shapes[i]
        _require_cuda(f, "f", torch.float32, 19 * nx * ny * nz)
        nat.call("lbm_batch_set_state", self._h, int(i), _ptr(f), _stream())

    def get_state(self, i):
        """f of instance i after the steps run so far, (19, nx, ny, nz)."""
        sim = ctypes.c_void_p()
        nat.call("lbm_batch_instance", self._h, int(i), ctypes.byref(sim))
        out = torch.empty((19,) + tuple(self.shapes[i]), dtype=torch.float32, device="cuda")
        nat.call("lbm_get_state", sim, _ptr(out), _stream())
        return out

    def projected_area(self, i):
        sim = ctypes.c_void_p()
        nat.call("lbm_batch_instance", self._h, int(i), ctypes.byref(sim))
        a = ctypes.c_double()
        nat.call("lbm_get_projected_area", sim, ctypes.byref(a))
        return a.value

    # -- stepping -----------------------------------------------------------
    def run(self, n_steps, sample_every=0):
        """Advance every instance; with sample_every > 0 returns a
        (n_samples, count, 4) float64 CUDA tensor of (Fx, Fy, Fz, Cd)."""
        n_steps = int(n_steps)
        samples = None
        if sample_every:
            ns = n_steps // int(sample_every)
            samples = torch.zeros((max(ns, 1), self.count, 4), dtype=torch.float64,
                                  device="cuda")
        nat.call("lbm_batched_run", self._h, n_steps, int(sample_every), _ptr(samples), _stream())
        return samples

    def cd_and_grad(self, n_steps, checkpoint_every=0, use_graph=True):
        """(Cd, dCd/dr) per instance after n_steps from the initial state."""
        cd = (ctypes.c_double * self.count)()
        g = (ctypes.c_double * self.count)()
        nat.call("lbm_batch_cd_and_grad", self._h, int(n_steps), int(checkpoint_every),
                 int(bool(use_graph)), cd, g, _stream())
        return np.array(cd[:]), np.array(g[:])

    def optimize(self, n_iters, n_steps, lr, r_min=0.3, r_max=0.8, loss="cd", target_cd=0.0,
                 b1=0.9, b2=0.999, eps=1e-8, checkpoint_every=0, use_graph=True):
        """n_iters Adam iterations on every radius (examples/11:182-194);
        loss "cd" (minimize_cd_loss) or "target" ((Cd - target_cd)^2).
        Returns histories (n_iters, count): r, loss, cd, grad (dloss/dr)."""
        o = nat.LBMAdamC()
        o.lr, o.b1, o.b2, o.eps = float(lr), float(b1), float(b2), float(eps)
        o.r_min, o.r_max = float(r_min), float(r_max)
        o.loss = nat.LBM_LOSS_TARGET_CD if loss == "target" else nat.LBM_LOSS_CD
        o.target_cd = float(target_cd)
        size = int(n_iters) * self.count
        hist = {k: (ctypes.c_double * max(size, 1))() for k in ("r", "loss", "cd", "grad")}
        nat.call("lbm_batch_optimize", self._h, int(n_iters), int(n_steps),
                 int(checkpoint_every), ctypes.byref(o), int(bool(use_graph)), hist["r"],
                 hist["loss"], hist["cd"], hist["grad"], _stream())
        out = {k: np.array(v[:size]).reshape(int(n_iters), self.count) for k, v in hist.items()}
        r = (ctypes.c_double * self.count)()
        nat.call("lbm_batch_get_radii", self._h, r)
        for i in range(self.count):
            self.spheres[i]["radius"] = r[i]
        out["r_final"] = np.array(r[:])
        return out

    # -- tuning -------------------------------------------------------------
    def set_workspace_limit(self, max_bytes):
        """Cap the population workspace of all instances under the automatic
        plan (checkpoint_every=0, autotune); 0 removes the cap."""
        nat.call("lbm_batch_set_workspace_limit", self._h, int(max_bytes))

    def set_block(self, block):
        nat.call("lbm_batch_set_block", self._h, int(block))

    def autotune(self, probe_steps, n_steps):
        """Pick the block shape by timing a probe_steps gradient evaluation at
        each, and the checkpoint interval for n_steps; returns (block, K)."""
        b, k = ctypes.c_int(), ctypes.c_int()
        nat.call("lbm_batch_autotune", self._h, int(probe_steps), int(n_steps), ctypes.byref(b),
                 ctypes.byref(k), _stream())
        return b.value, k.value

    @property
    def plan(self):
        """(block, segment steps, recomputed steps, workspace bytes, graph build s)."""
        b, k, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        w, g = ctypes.c_ulonglong(), ctypes.c_double()
        nat.call("lbm_batch_get_plan", self._h, ctypes.byref(b), ctypes.byref(k),
                 ctypes.byref(r), ctypes.byref(w), ctypes.byref(g))
        return b.value, k.value, r.value, w.value, g.value

    @property
    def graph_launches(self):
        """Kernel launches in the last captured gradient-evaluation graph."""
        n = ctypes.c_longlong()
        nat.call("lbm_batch_graph_launches", self._h, ctypes.byref(n))
        return n.value


def mixed_sphere_instances(count=64, seed=0, n_alpha=(5.0, 10.0, 20.0), re=50.0):
    """The batched workload: grids uniform over {64x32x32, 96x48x48,
    128x64x64}, radius uniform in [4, 8] * (ny / 32) cells, modes split evenly
    over {halfway, bouzidi} x {hard, sigmoid-soft} with alpha from n_alpha,
    drawn with numpy default_rng(seed).  As the reference's optimisation
    driver (examples/11:56-60, 218-230): MRT, sphere centred at the world
    origin, u_in = 0.05, tau from Re (default 50) on the sphere diameter.
    Returns (instances, spheres) for Batch and Batch.set_spheres."""
    rng = np.random.default_rng(seed)
    grids = [(64, 32, 32), (96, 48, 48), (128, 64, 64)]
    modes = [("halfway", "hard"), ("bouzidi", "hard"), ("halfway", "soft"), ("bouzidi", "soft")]
    U = 0.05
    instances, spheres = [], []
    for i in range(count):
        nx, ny, nz = grids[int(rng.integers(0, 3))]
        r_cells = float(rng.uniform(4.0, 8.0)) * ny / 32.0
        r_world = r_cells / (ny / 4.0)          # world units: ny/4 cells per unit
        q_mode, porosity = modes[i % 4]
        alpha = float(n_alpha[int(rng.integers(0, len(n_alpha)))])
        tau = 3.0 * U * (2.0 * r_cells) / re + 0.5
        instances.append(dict(nx=nx, ny=ny, nz=nz, tau=tau, collision="mrt", storage="fp32",
                              periodic_yz=True, guard="off", inlet_velocity=(U, 0.0, 0.0)))
        spheres.append(dict(radius=r_world, center=(0.0, 0.0, 0.0), sharpness=alpha,
                            kind="sigmoid", q_mode=q_mode, porosity=porosity))
    return instances, spheres
