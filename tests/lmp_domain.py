"""An MD engine's view of a periodic structure, as LAMMPS hands it to a pair style: the atoms of
the cell (local, wrapped into the cell) followed by ghost atoms (periodic images within a
communication cutoff of some local atom), and a FULL neighbour list over local + ghost atoms built
with a skin (rc + skin), rows in a shuffled order. Test infrastructure for the caller-list entry
point (ann_compute_list)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Domain:
    x: np.ndarray          # (nall, 3) local atoms then ghosts
    type: np.ndarray       # (nall,)
    owner: np.ndarray      # (nall,) local atom each atom is an image of (itself for local atoms)
    image: np.ndarray      # (nall, 3) integer lattice translation of each atom
    nlocal: int
    numneigh: np.ndarray   # (nlocal,) in local atom order
    neigh: np.ndarray      # rows back to back

    @property
    def nall(self) -> int:
        return len(self.x)

    def rows(self, ilist):
        """numneigh / neigh reordered for the rows of ilist (centre atoms, a subset or permutation)."""
        off = np.concatenate([[0], np.cumsum(self.numneigh)])
        nn = self.numneigh[ilist]
        nb = np.concatenate([self.neigh[off[i]:off[i + 1]] for i in ilist]) if len(ilist) else np.zeros(0, np.int32)
        return nn.astype(np.int32), nb.astype(np.int32)

    def fold(self, F: np.ndarray) -> np.ndarray:
        """Ghost forces added to their owners (LAMMPS reverse communication with newton_pair on)."""
        out = np.zeros((self.nlocal, 3))
        np.add.at(out, self.owner, F)
        return out


def _heights(R: np.ndarray) -> np.ndarray:
    a = [R[:, 0], R[:, 1], R[:, 2]]
    vol = abs(np.linalg.det(R))
    return np.array([vol / np.linalg.norm(np.cross(a[(d + 1) % 3], a[(d + 2) % 3])) for d in range(3)])


def build_domain(x, types, R, rcomm, seed=0, shuffle=True) -> Domain:
    """Local atoms = x wrapped into the cell R (lattice vectors as columns); ghosts = every image
    x_j + R n (n != 0) closer than rcomm to some local atom; full lists of every local atom within
    rcomm (self excluded), each row in a random order."""
    R = np.asarray(R, np.float64)
    s = np.linalg.solve(R, np.asarray(x, np.float64).T).T
    s -= np.floor(s)
    s[s >= 1.0] = 0.0
    xl = s @ R.T
    n = len(xl)
    k = np.ceil(rcomm / _heights(R)).astype(int) + 1
    gx, gt, go, gi = [], [], [], []
    for n0 in range(-k[0], k[0] + 1):
        for n1 in range(-k[1], k[1] + 1):
            for n2 in range(-k[2], k[2] + 1):
                if n0 == n1 == n2 == 0:
                    continue
                sh = R @ np.array([n0, n1, n2], np.float64)
                xi = xl + sh
                d = np.linalg.norm(xi[:, None, :] - xl[None, :, :], axis=2).min(axis=1)
                keep = np.nonzero(d < rcomm)[0]
                if len(keep):
                    gx.append(xi[keep]); gt.append(np.asarray(types)[keep]); go.append(keep)
                    gi.append(np.tile([n0, n1, n2], (len(keep), 1)))
    X = np.concatenate([xl] + gx) if gx else xl
    T = np.concatenate([np.asarray(types, np.int32)] + gt).astype(np.int32) if gt else np.asarray(types, np.int32)
    O = np.concatenate([np.arange(n)] + go).astype(np.int64) if go else np.arange(n)
    I = np.concatenate([np.zeros((n, 3), int)] + gi) if gi else np.zeros((n, 3), int)
    rng = np.random.default_rng(seed)
    numneigh, rows = [], []
    for i in range(n):
        d = np.linalg.norm(X - xl[i], axis=1)
        j = np.nonzero((d < rcomm) & (np.arange(len(X)) != i))[0]
        if shuffle:
            j = rng.permutation(j)
        numneigh.append(len(j)); rows.append(j)
    neigh = np.concatenate(rows).astype(np.int32) if rows else np.zeros(0, np.int32)
    return Domain(X, T, O, I, n, np.array(numneigh, np.int32), neigh)
