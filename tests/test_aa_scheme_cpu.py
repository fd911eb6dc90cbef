"""The in-place (AA) streaming scheme of csrc/step_aa.cu, restated on the CPU
with a stand-in collision, against the two-buffer pull it replaces:

  layout L: S_i(x) at A[opp(i)][x];  layout P: S_i(x) at A[i][x + e_i]
  (y, z periodic; x never), record and x-face cells also keeping their S
  vector in a side buffer (two copies) for the reads beyond the plain pull:
  the Bouzidi terms (q < 0.5 reads the second fluid cell's vector), the
  fallback of out-of-range x sources.

Checked over several launches of both layouts: every A location a launch
touches is read and written by one cell only (no races), no read finds an
unwritten location, and the states equal the two-buffer scheme's.  The GPU
tests hold the kernel itself to the two-buffer kernel to the bit."""

import numpy as np
import pytest

E = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
              [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1],
              [-1, 0, -1], [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]])
OPP = [int(np.where((E == -E[i]).all(axis=1))[0][0]) for i in range(19)]
Q = 19


class Grid:
    def __init__(self, nx, ny, nz, n_records, seed):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.n = nx * ny * nz
        rng = np.random.default_rng(seed)
        # boundary records: cells with random wall links (q in (0, 1)), and
        # every q < 0.5 link's second fluid cell a record too
        self.links = {int(c): {} for c in rng.choice(self.n, n_records, replace=False)}
        for c in list(self.links):
            for i in range(1, Q):
                if rng.random() < 0.3:
                    self.links[c][OPP[i]] = float(rng.choice([rng.uniform(0.02, 0.49), 0.5,
                                                              rng.uniform(0.51, 0.98)]))
        todo = list(self.links)
        while todo:
            c = todo.pop()
            for io, q in self.links[c].items():
                nb = self.ahead(c, OPP[io])
                if q < 0.5 and nb not in self.links:
                    self.links[nb] = {}
                    todo.append(nb)
        self.records = sorted(self.links)
        self.rec_index = {c: k for k, c in enumerate(self.records)}

    def xyz(self, c):
        return c // (self.ny * self.nz), (c // self.nz) % self.ny, c % self.nz

    def cell(self, x, y, z):
        return (x * self.ny + y % self.ny) * self.nz + z % self.nz

    def ahead(self, c, i):
        x, y, z = self.xyz(c)
        return self.cell((x + E[i, 0]) % self.nx, y + E[i, 1], z + E[i, 2])

    def slot(self, c):
        """Side-buffer slot: the record, else the x-face slot, else None."""
        if c in self.rec_index:
            return self.rec_index[c]
        x, y, z = self.xyz(c)
        base = len(self.records)
        if x == 0:
            return base + y * self.nz + z
        if x == self.nx - 1:
            return base + self.ny * self.nz + y * self.nz + z
        return None

    def slots(self):
        return len(self.records) + 2 * self.ny * self.nz


def collide(f, c):
    """A cell-dependent stand-in for the collision (the scheme does not care)."""
    return f * 1.01 + 0.001 * np.arange(Q) + 1e-4 * (c % 7)


def bouzidi(g, c, f, own, second):
    """streaming.py:148-183 on cell c: own(j) = S_j(c), second(io, nb) = S_io(nb)."""
    for io, q in g.links.get(c, {}).items():
        i = OPP[io]
        if q >= 0.5:
            a = 1.0 / (2.0 * min(q, 1.0))
            f[i] = a * own(io) + (1.0 - a) * own(i)
        else:
            b = 2.0 * max(q, 0.0)
            f[i] = b * own(io) + (1.0 - b) * second(io, g.ahead(c, i))
    return f


def step_ab(g, S):
    out = np.empty_like(S)
    for c in range(g.n):
        x, y, z = g.xyz(c)
        f = np.empty(Q)
        for i in range(Q):
            sx = x - E[i, 0]
            f[i] = S[i, c] if not 0 <= sx < g.nx else S[i, g.cell(sx, y - E[i, 1], z - E[i, 2])]
        f = bouzidi(g, c, f, lambda j: S[j, c], lambda io, nb: S[io, nb])
        out[:, c] = collide(f, c)
    return out


def state_of(g, A, sb, layout_l):
    """S recovered from the buffer and the side buffer."""
    S = np.empty((Q, g.n))
    for c in range(g.n):
        x, y, z = g.xyz(c)
        for i in range(Q):
            if layout_l:
                S[i, c] = A[OPP[i], c]
            else:
                tx = x + E[i, 0]
                S[i, c] = (A[i, g.cell(tx, y + E[i, 1], z + E[i, 2])] if 0 <= tx < g.nx
                           else sb[g.slot(c)][i])
    return S


@pytest.mark.parametrize("grid", [(7, 4, 6, 12, 0), (5, 3, 2, 6, 1), (4, 1, 3, 3, 2)])
def test_aa_scheme_equals_the_pull_and_is_race_free(grid):
    g = Grid(*grid)
    rng = np.random.default_rng(9)
    f0 = rng.random((Q, g.n))
    S = np.stack([collide(f0[:, c], c) for c in range(g.n)], axis=1)
    # the collide-only launch writes layout L and the side buffer
    A = np.full((Q, g.n), np.nan)
    sb = [np.full((g.slots(), Q), np.nan) for _ in range(2)]
    cur = 1
    for c in range(g.n):
        for i in range(Q):
            A[OPP[i], c] = S[i, c]
        if g.slot(c) is not None:
            sb[cur][g.slot(c)] = S[:, c]
    layout_l = True
    assert np.array_equal(state_of(g, A, sb[cur], layout_l), S)
    for k in range(6):
        S = step_ab(g, S)
        new, owner = A.copy(), {}
        sin, sout = sb[cur], sb[1 - cur]
        for c in range(g.n):
            x, y, z = g.xyz(c)
            sl = g.slot(c)
            f, reads = np.empty(Q), []
            for i in range(Q):
                sx = x - E[i, 0]
                if not 0 <= sx < g.nx:
                    f[i] = sin[sl][i]
                else:
                    loc = ((OPP[i], g.cell(sx, y - E[i, 1], z - E[i, 2])) if layout_l else (i, c))
                    f[i] = A[loc]
                    reads.append(loc)
            f = bouzidi(g, c, f, lambda j: sin[sl][j], lambda io, nb: sin[g.slot(nb)][io])
            s = collide(f, c)
            writes = []
            for i in range(Q):
                if layout_l:
                    tx = x + E[i, 0]
                    if 0 <= tx < g.nx:
                        writes.append((i, g.cell(tx, y + E[i, 1], z + E[i, 2])))
                        new[writes[-1]] = s[i]
                else:
                    writes.append((OPP[i], c))
                    new[writes[-1]] = s[i]
            if sl is not None:
                sout[sl] = s
            for loc in reads + writes:
                assert owner.setdefault(loc, c) == c, ("two cells touch", loc, k)
            for loc in reads:
                assert not np.isnan(A[loc]), ("read of an unwritten location", loc, k)
        A, cur, layout_l = new, 1 - cur, not layout_l
        assert np.allclose(state_of(g, A, sb[cur], layout_l), S, rtol=0, atol=1e-12), k
