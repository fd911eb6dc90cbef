"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

The reference (JAX) cannot run here, so the fixtures come from the oracle,
which tests/test_oracle_pins.py pins to the reference's published numbers.
Each fixture records the configuration it was produced with.

    python tests/golden/make_golden.py pins channel sphere modes
"""

import json
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import drivers, geometry, ops  # noqa: E402
from oracle.ops import consts_for  # noqa: E402


def _save_json(name, d):
    with open(os.path.join(HERE, name), "w") as fh:
        json.dump(d, fh, indent=1, sort_keys=True)


def pins():
    dt = torch.float64
    c = consts_for(dt, True)
    r = torch.tensor(0.5, dtype=dt, requires_grad=True)
    cd = drivers.cd_of_radius_bgk_f64(r)
    cd.backward()

    def sim(ux):
        f = drivers.initial_state(8, 4, 4, 0.0, dt, c)
        q = -torch.ones((19, 8, 4, 4), dtype=dt)
        for _ in range(5):
            f = ops.zou_he_outlet(ops.zou_he_inlet(ops.stream(ops.bgk(f, 0.8, c), q, True),
                                                   (ux, 0.0, 0.0)), 1.0)
        return ops.compute_density(f[:, 2:-2]).mean()

    u = torch.tensor(0.05, dtype=dt, requires_grad=True)
    sim(u).backward()
    _save_json("pins.json", {
        "bouzidi_cd_f64": float(cd), "bouzidi_dcd_dr_f64": float(r.grad),
        "inlet_grad_f64": float(u.grad),
        "setup": "tests/test_gradients_f64.py of the reference (32x16x16, 10 BGK steps, alpha 20, r 0.5)",
    })


def channel():
    """Channel: 64x21x8 BGK, parabolic inlet peak 0.05, tau 0.8, 3000 steps."""
    nx, ny, nz, n = 64, 21, 8, 3000
    prof = drivers.parabolic_inlet(ny, nz, 0.05)
    solid = drivers.channel_walls(nx, ny, nz)
    q = geometry.compute_q_from_solid(solid, 0.5)
    f = drivers.initial_state(nx, ny, nz, 0.0)
    cfg = drivers.StepConfig(tau=0.8, inlet=(prof, 0.0, 0.0), collision="bgk")
    t0 = time.time()
    with torch.no_grad():
        f, _, _ = drivers.run(f, q, cfg, n, solid=solid)
    u = ops.compute_velocity(f, ops.compute_density(f))
    ux = u[0, nx // 2].mean(dim=-1).double()
    H = float(ny - 2)
    s = torch.arange(ny, dtype=torch.float64) - 0.5
    ana = ux[1:-1].max() * 4 * s * (H - s) / (H * H)
    ana[0] = ana[-1] = 0.0
    l2 = float(torch.sqrt(((ux[1:-1] - ana[1:-1]) ** 2).sum() / (ana[1:-1] ** 2).sum()))
    np.savez_compressed(os.path.join(HERE, "channel_64x21x8.npz"), u=u.numpy().astype(np.float32))
    _save_json("channel_64x21x8.json", {
        "grid": [nx, ny, nz], "steps": n, "tau": 0.8, "u_peak": 0.05,
        "profile_ux": ux.tolist(), "l2_vs_parabola": l2, "seconds": time.time() - t0})


def sphere(periodic=False):
    """Sphere: 96x48x48 MRT, Bouzidi hard sphere r=0.5 world (6 cells) at
    world (-2,0,0) = lattice (24,24,24), U 0.05, nu 0.006 (Re 100), free-slip
    sides (periodic_yz=False; with periodic=True the examples/10 periodic
    sides), pre-collision guard, 2000 steps, Cd every step of the last 30%."""
    nx, ny, nz, n = 96, 48, 48, 2000
    U, nu = 0.05, 0.006
    tau = 3 * nu + 0.5
    center = (-2.0, 0.0, 0.0)
    solid, q = geometry.create_sphere(nx, ny, nz, center, 0.5)
    f = drivers.initial_state(nx, ny, nz, U)
    cfg = drivers.StepConfig(tau=tau, inlet=(U, 0.0, 0.0), collision="mrt",
                             periodic_yz=periodic, guard="pre")
    area = max(ops.projected_area(solid), 1.0)
    start = n - int(0.3 * n)
    hist = []

    def cb(k, fs, fp):
        if k > start:
            hist.append(float(drivers.cd_from(fp, fs, q, U, area)[0]))

    t0 = time.time()
    with torch.no_grad():
        f, _, _ = drivers.run(f, q, cfg, n, solid=solid, f_ref=f, sample_every=1, on_sample=cb)
    u = ops.compute_velocity(f, ops.compute_density(f))
    tag = "sphere_96x48x48" + ("_periodic" if periodic else "")
    np.savez_compressed(os.path.join(HERE, tag + ".npz"),
                        u_sub=u[:, ::2, ::2, ::2].numpy().astype(np.float32))
    _save_json(tag + ".json", {"periodic_yz": periodic,
        "grid": [nx, ny, nz], "steps": n, "tau": tau, "U": U, "center": center, "radius": 0.5,
        "area": area, "cd_window": [start + 1, n], "cd_mean": float(np.mean(hist)),
        "cd_std": float(np.std(hist)), "cd_last": hist[-1], "cd_hist_every10": hist[::10],
        "links": int((q[1:] >= 0).sum()), "seconds": time.time() - t0})


def sphere_periodic():
    sphere(periodic=True)


def sphere_freeslip_fp64():
    """The free-slip 96x48x48 sphere of sphere() in FP64 (the oracle's FP64
    constants, those of the fused solver's FP64 storage mode): Cd every 100
    steps over the 2000 steps and u at a few fixed cells at the end."""
    dt = torch.float64
    c = ops.consts_for(dt)
    nx, ny, nz, n, every = 96, 48, 48, 2000, 100
    U, nu = 0.05, 0.006
    tau = 3 * nu + 0.5
    center = (-2.0, 0.0, 0.0)
    solid, q = geometry.create_sphere(nx, ny, nz, center, 0.5, dt)
    f = drivers.initial_state(nx, ny, nz, U, dt, c)
    cfg = drivers.StepConfig(tau=tau, inlet=(U, 0.0, 0.0), collision="mrt",
                             periodic_yz=False, guard="pre")
    area = max(ops.projected_area(solid), 1.0)
    cds = []

    def cb(k, fs, fp):
        if k % every == 0:
            cds.append(float(drivers.cd_from(fp, fs, q, U, area)[0]))

    t0 = time.time()
    with torch.no_grad():
        f, _, _ = drivers.run(f, q, cfg, n, solid=solid, f_ref=f, sample_every=1, on_sample=cb,
                              consts=c)
    u = ops.compute_velocity(f, ops.compute_density(f))
    probes = [(40, 24, 24), (30, 10, 40), (60, 24, 5), (90, 40, 40), (10, 0, 0)]
    _save_json("sphere_96x48x48_freeslip_fp64.json", {
        "grid": [nx, ny, nz], "steps": n, "tau": tau, "U": U, "center": center, "radius": 0.5,
        "sample_every": every, "cd": cds, "probes": probes,
        "u_probes": [[float(u[a, x, y, z]) for a in range(3)] for x, y, z in probes],
        "seconds": time.time() - t0})


def modes():
    """Four-mode base Cd, 96x48x48 MRT, Re 50, 2000 steps (examples/11:56-165);
    published (A100): halfway_hard 1.85, bouzidi_hard 1.77, halfway_soft 0.43,
    bouzidi_soft 0.45 (README.md:33-38)."""
    nx, ny, nz, n = 96, 48, 48, 2000
    U = 0.05
    d_lat = nx * 0.5 / 4.0
    tau = float(np.float32(3.0 * (U * d_lat / 50.0) + 0.5))
    out = {"grid": [nx, ny, nz], "steps": n, "tau": tau}
    for qm, pm in (("halfway", "hard"), ("bouzidi", "hard"), ("halfway", "soft"), ("bouzidi", "soft")):
        por, solid, q = geometry.sphere_geometry(nx, ny, nz, 0.5, qm, pm, 20.0)
        f = drivers.initial_state(nx, ny, nz, U)
        cfg = drivers.StepConfig(tau=tau, inlet=(U, 0.0, 0.0), collision="mrt")
        t0 = time.time()
        with torch.no_grad():
            f, fp, _ = drivers.run(f, q, cfg, n, porosity=por)
        cd, _ = drivers.cd_from(fp, f, q, U, max(ops.projected_area(solid), 1.0))
        out["%s_%s" % (qm, pm)] = {"cd": float(cd), "seconds": time.time() - t0}
        _save_json("modes_96x48x48.json", out)


def sphere_grad_96x48x48():
    """dCd/dr at 96x48x48, MRT, Bouzidi ray-sphere q(r),
    r = 0.5 world (6 cells) centred at cell (24, 24, 24) = world (-2, 0, 0),
    Re 100 (nu 0.006, tau 0.518); FP64 autograd through the oracle (the
    jax.grad stand-in) over a 100-step window, for the hard sphere and the
    sigmoid-soft sphere (alpha 20).  Rematerialised in chunks of 10 steps."""
    nx, ny, nz, n = 96, 48, 48, 100
    tau = 3.0 * 0.006 + 0.5
    dt = torch.float64
    out = {"grid": [nx, ny, nz], "steps": n, "tau": tau, "center": [-2.0, 0.0, 0.0],
           "radius": 0.5}
    torch.set_num_threads(os.cpu_count() or 1)
    for name, kw in (("hard", dict(q_mode="bouzidi", porosity_mode="hard")),
                     ("soft20", dict(q_mode="bouzidi", porosity_mode="soft", sharpness=20.0))):
        r = torch.tensor(0.5, dtype=dt, requires_grad=True)
        t0 = time.time()
        cd = drivers.simulate_cd(r, nx, ny, nz, n, tau, center=(-2.0, 0.0, 0.0), dtype=dt,
                                 consts=consts_for(dt), remat_chunk=10, **kw)
        cd.backward()
        out[name] = {"cd": float(cd.detach()), "dcd_dr": float(r.grad), "seconds": time.time() - t0,
                     "porosity": kw["porosity_mode"], "sharpness": kw.get("sharpness")}
        _save_json("sphere_grad_96x48x48.json", out)


if __name__ == "__main__":
    for name in sys.argv[1:] or ["pins", "channel", "sphere", "sphere_periodic", "modes"]:
        globals()[name]()
        print("done", name, flush=True)
