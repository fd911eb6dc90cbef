"""The batched workload generator (no GPU): 64 instances over three grids,
radii in [4, 8] * ny / 32 cells, modes split evenly, reproducible seed."""
import numpy as np

from lbm_jax_autodiff_gb300.batch import mixed_sphere_instances


def test_mixed_sphere_draw():
    inst, sph = mixed_sphere_instances()
    assert len(inst) == 64 and len(sph) == 64
    grids = {(i["nx"], i["ny"], i["nz"]) for i in inst}
    assert grids <= {(64, 32, 32), (96, 48, 48), (128, 64, 64)} and len(grids) == 3
    for i, s in zip(inst, sph):
        r_cells = s["radius"] * i["ny"] / 4.0
        assert 4.0 * i["ny"] / 32 <= r_cells <= 8.0 * i["ny"] / 32
        assert s["sharpness"] in (5.0, 10.0, 20.0)
        assert i["collision"] == "mrt" and i["storage"] == "fp32"
        # tau from Re = 50 on the diameter (examples/11:229-230)
        assert abs(i["tau"] - (0.5 + 3 * 0.05 * 2 * r_cells / 50.0)) < 1e-15
    modes = [(s["q_mode"], s["porosity"]) for s in sph]
    for m in [("halfway", "hard"), ("bouzidi", "hard"), ("halfway", "soft"), ("bouzidi", "soft")]:
        assert modes.count(m) == 16
    inst2, sph2 = mixed_sphere_instances()
    assert inst == inst2 and sph == sph2
    cells = sum(i["nx"] * i["ny"] * i["nz"] for i in inst)
    assert 64 * 65536 <= cells <= 64 * 524288
