"""State I/O and VTK export (jax_lbm io/vtk.py).

``export_vtk`` has the reference's signature and fields: density, velocity
components and magnitude, and the optional solid mask and porosity, as cell
data of an nx x ny x nz grid of unit cells (io/vtk.py:14-104).  The reference
goes through meshio, which is not a dependency here; this writes the legacy
VTK format (STRUCTURED_POINTS, binary big-endian float32) that ParaView reads
directly.  Density and velocity come from the CUDA moment kernels, so f must
be a CUDA tensor.

``save_state`` / ``load_state`` keep a Simulation's populations (reference
layout, compute dtype) and its step count in an .npz file.
"""

import numpy as np
import torch

from .core.equilibrium import compute_density, compute_velocity


def _cells_x_fastest(a):
    """(nx, ny, nz) array -> flat in VTK cell order (x fastest, then y, z)."""
    return np.ascontiguousarray(np.transpose(np.asarray(a), (2, 1, 0))).ravel()


def export_vtk(filename, f, solid=None, porosity=None):
    """Write density, velocity and the optional solid / porosity of the state
    f (19, nx, ny, nz) to a legacy .vtk file (io/vtk.py:14-104)."""
    if not (torch.is_tensor(f) and f.is_cuda):
        raise TypeError("f must be a CUDA tensor (19, nx, ny, nz)")
    rho = compute_density(f)
    u = compute_velocity(f, rho)
    rho = rho.detach().cpu().numpy()
    u = u.detach().cpu().numpy()
    nx, ny, nz = rho.shape
    fields = [("density", rho), ("velocity_x", u[0]), ("velocity_y", u[1]),
              ("velocity_z", u[2]), ("velocity_magnitude", np.sqrt((u ** 2).sum(axis=0)))]
    if solid is not None:
        fields.append(("solid", torch.as_tensor(solid).detach().cpu().numpy()))
    if porosity is not None:
        fields.append(("porosity", torch.as_tensor(porosity).detach().cpu().numpy()))
    with open(filename, "wb") as fh:
        head = ("# vtk DataFile Version 3.0\njax_lbm state\nBINARY\nDATASET STRUCTURED_POINTS\n"
                "DIMENSIONS %d %d %d\nORIGIN 0 0 0\nSPACING 1 1 1\nCELL_DATA %d\n"
                % (nx + 1, ny + 1, nz + 1, nx * ny * nz))
        fh.write(head.encode("ascii"))
        for name, a in fields:
            fh.write(("SCALARS %s float 1\nLOOKUP_TABLE default\n" % name).encode("ascii"))
            fh.write(_cells_x_fastest(a).astype(">f4").tobytes())
            fh.write(b"\n")


def read_vtk(filename):
    """Read back a file written by export_vtk: {field: (nx, ny, nz) float32 array}."""
    with open(filename, "rb") as fh:
        data = fh.read()
    pos = 0

    def line():
        nonlocal pos
        end = data.index(b"\n", pos)
        out = data[pos:end].decode("ascii")
        pos = end + 1
        return out

    dims = None
    ncell = None
    fields = {}
    while pos < len(data):
        ln = line().strip()
        if ln.startswith("DIMENSIONS"):
            dims = [int(v) - 1 for v in ln.split()[1:4]]
        elif ln.startswith("CELL_DATA"):
            ncell = int(ln.split()[1])
        elif ln.startswith("SCALARS"):
            name = ln.split()[1]
            line()                                   # LOOKUP_TABLE default
            a = np.frombuffer(data, dtype=">f4", count=ncell, offset=pos).astype(np.float32)
            pos += 4 * ncell + 1
            nx, ny, nz = dims
            fields[name] = np.transpose(a.reshape(nz, ny, nx), (2, 1, 0))
    return fields


def save_state(path, sim):
    """Write sim's populations (reference layout) and step count to an .npz."""
    f = sim.get_state().cpu().numpy()
    np.savez(path, f=f, steps=np.int64(sim.steps), shape=np.array(sim.shape))


def load_state(path, sim):
    """Load populations saved by save_state into sim (the step count restarts)."""
    d = np.load(path)
    if tuple(d["shape"]) != tuple(sim.shape):
        raise ValueError("state shape %s does not match the simulation %s"
                         % (tuple(d["shape"]), sim.shape))
    sim.set_state(torch.as_tensor(d["f"], dtype=sim.dtype, device="cuda"))
    return int(d["steps"])
