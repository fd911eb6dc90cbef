"""The index arithmetic of the fused kernels, restated on the CPU and checked
against the physical neighbour (x - e_i for a pull, x + e_i for a push; y and
z periodic, x in range) on grids whose y / z wraps land on the cell itself or
its pair partner:

  - k_step / pull_post_bc with pointer tables (csrc/step.cu, csrc/sim.cuh):
    tab[i] + idx + wrap corrections;
  - k_step_pair, the 16-bit pair pull (csrc/step.cu): pair_pull(i) + b with
    the y rows iym / iyp and the per-lane z wraps zw0 / zw1;
  - k_adjoint_pair's gather of nu_{k+1} (csrc/adjoint.cu): adj_push(j) + b;
  - k_step_aa's tables (csrc/step_aa.cu): rd[i] / wr[i] + idx + wy / wz.

The GPU tests hold the kernels to the oracle and to each other; this pins
the arithmetic itself, including every index staying inside its direction's
plane of the population array."""

import itertools

import pytest

E = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
     (1, 1, 0), (-1, 1, 0), (1, -1, 0), (-1, -1, 0), (1, 0, 1), (-1, 0, 1), (1, 0, -1),
     (-1, 0, -1), (0, 1, 1), (0, -1, 1), (0, 1, -1), (0, -1, -1)]
OPP = [E.index(tuple(-c for c in e)) for e in E]
Q = 19
GRIDS = [(3, 1, 2), (4, 2, 2), (5, 3, 4), (6, 4, 6), (4, 5, 8)]


def cell(g, x, y, z):
    nx, ny, nz = g
    return (x * ny + y % ny) * nz + z % nz


def interior(g):
    nx, ny, nz = g
    return [(x, y, z) for x, y, z in itertools.product(range(1, nx - 1), range(ny), range(nz))]


def off(g, i):
    nx, ny, nz = g
    ex, ey, ez = E[i]
    return ex * ny * nz + ey * nz + ez


@pytest.mark.parametrize("g", GRIDS)
def test_per_cell_pull_tables(g):
    nx, ny, nz = g
    N, nyz = nx * ny * nz, ny * nz
    for x, y, z in interior(g):
        idx = cell(g, x, y, z)
        wym = nyz if y == 0 else 0
        wyp = -nyz if y == ny - 1 else 0
        wzm = nz if z == 0 else 0
        wzp = -nz if z == nz - 1 else 0
        for i in range(Q):
            ex, ey, ez = E[i]
            b = idx + {1: wym, -1: wyp, 0: 0}[ey] + {1: wzm, -1: wzp, 0: 0}[ez]
            got = i * N - off(g, i) + b
            assert got == i * N + cell(g, x - ex, y - ey, z - ez), (g, x, y, z, i)


@pytest.mark.parametrize("g", [g for g in GRIDS if g[2] % 2 == 0])
def test_pair_pull_and_adjoint_gather(g):
    nx, ny, nz = g
    N, nyz = nx * ny * nz, ny * nz
    for x, y, z in interior(g):
        if z % 2:
            continue
        idx = cell(g, x, y, z)
        iym = idx + (nyz if y == 0 else 0)
        iyp = idx - (nyz if y == ny - 1 else 0)
        zw0 = nz if z == 0 else 0
        zw1 = -nz if z + 2 == nz else 0
        for i in range(Q):
            ex, ey, ez = E[i]
            # forward pull (step_pair_interior)
            b = iym if ey == 1 else (iyp if ey == -1 else idx)
            p = i * N - off(g, i) + b
            lanes = {0: (p, p + 1), 1: (p + zw0, p + 1), -1: (p, p + 1 + zw1)}[ez]
            for lane, e in enumerate(lanes):
                assert e == i * N + cell(g, x - ex, y - ey, z + lane - ez), ("pull", g, i, lane)
            # adjoint gather nu_{k+1}(x + e_j) (adjoint_pair_interior)
            b = iyp if ey == 1 else (iym if ey == -1 else idx)
            p = i * N + off(g, i) + b
            lanes = {0: (p, p + 1), 1: (p, p + 1 + zw1), -1: (p + zw0, p + 1)}[ez]
            for lane, e in enumerate(lanes):
                assert e == i * N + cell(g, x + ex, y + ey, z + lane + ez), ("push", g, i, lane)


@pytest.mark.parametrize("g", GRIDS)
def test_in_place_tables(g):
    nx, ny, nz = g
    N, nyz = nx * ny * nz, ny * nz
    for x, y, z in interior(g):
        idx = cell(g, x, y, z)

        def wy(d):
            return (nyz if y == 0 else 0) if d < 0 else ((-nyz if y == ny - 1 else 0) if d > 0 else 0)

        def wz(d):
            return (nz if z == 0 else 0) if d < 0 else ((-nz if z == nz - 1 else 0) if d > 0 else 0)

        for i in range(Q):
            ex, ey, ez = E[i]
            # layout-L launch: read A[opp(i)][x - e_i], write A[i][x + e_i]
            rd = OPP[i] * N - off(g, i) + idx + wy(-ey) + wz(-ez)
            wr = i * N + off(g, i) + idx + wy(ey) + wz(ez)
            assert rd == OPP[i] * N + cell(g, x - ex, y - ey, z - ez), ("read", g, i)
            assert wr == i * N + cell(g, x + ex, y + ey, z + ez), ("write", g, i)
            assert OPP[i] * N <= rd < (OPP[i] + 1) * N and i * N <= wr < (i + 1) * N
