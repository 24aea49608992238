"""Structure files: the extended-XYZ reader and writer of the reference (XYZ::read / XYZ::write,
src/format/xyz_struc.cpp:38-266), in metal units, and packing of read structures into a batch
for the library (types resolved by the potential's type names).

Reader, as XYZ::read: line 1 is the atom count; line 2 is searched case-insensitively for
Properties=species:S:1:pos:R:3[:forces:R:3], potential_energy=<E> and Lattice="<a1> <a2> <a3>"
(nine numbers, the lattice vectors one after the other: the columns of R); then one line per atom
(name, x, y, z[, fx, fy, fz]). With a lattice the positions are wrapped into the cell
(fractional coordinates in [0, 1), as Cell::returnToCell).

Writer, as XYZ::write, but with the lattice vectors written in order (the reference writes R(1,2)
in place of R(2,1) and R(0,2), which matters only for non-orthogonal cells).
"""
from __future__ import annotations

import re
from dataclasses import dataclass
from pathlib import Path

import numpy as np


@dataclass
class XYZStructure:
    names: list
    posn: np.ndarray                 # (N, 3) Angstrom
    cell: np.ndarray | None          # (3, 3), lattice vectors as columns; None without a lattice
    energy: float                    # potential_energy (eV), 0 when absent
    forces: np.ndarray | None        # (N, 3) eV/Angstrom when the file has them


def _wrap(x: np.ndarray, R: np.ndarray) -> np.ndarray:
    s = np.linalg.solve(R, x.T).T
    s -= np.floor(s)
    s[s >= 1.0] = 0.0
    return s @ R.T


def read_xyz(path) -> XYZStructure:
    lines = Path(path).read_text().splitlines()
    if len(lines) < 2:
        raise ValueError(f"{path}: not an XYZ file")
    try:
        n = int(lines[0].split()[0])
    except (ValueError, IndexError):
        n = 0
    if n <= 0:
        raise ValueError(f"{path}: found zero atoms")
    head = lines[1].upper()
    cols = {"species": 0, "pos": (1, 2, 3), "forces": None}
    m = re.search(r"PROPERTIES\s*=\s*(\S+)", head)
    if m:
        tok = m.group(1).split(":")
        index, k = 0, 0
        while k + 2 < len(tok):
            tag, typ, cnt = tok[k], tok[k + 1], int(tok[k + 2])
            if tag == "SPECIES":
                if typ != "S" or cnt != 1:
                    raise ValueError(f"{path}: invalid species column")
                cols["species"] = index
            elif tag == "POS":
                if typ != "R" or cnt != 3:
                    raise ValueError(f"{path}: invalid position columns")
                cols["pos"] = (index, index + 1, index + 2)
            elif tag == "FORCES":
                if typ != "R" or cnt != 3:
                    raise ValueError(f"{path}: invalid force columns")
                cols["forces"] = (index, index + 1, index + 2)
            index += cnt
            k += 3
    energy = 0.0
    m = re.search(r"POTENTIAL_ENERGY\s*=\s*([-+0-9.EeDd]+)", head)
    if m:
        energy = float(m.group(1).replace("D", "E"))
    R = None
    m = re.search(r'LATTICE\s*=\s*"([^"]*)"', head)
    if m:
        v = [float(t) for t in m.group(1).split()]
        if len(v) != 9:
            raise ValueError(f"{path}: the lattice needs nine numbers")
        R = np.array(v).reshape(3, 3).T          # vectors as columns
        if not np.linalg.norm(R) > 0:
            R = None
    if len(lines) < 2 + n:
        raise ValueError(f"{path}: {n} atoms announced, {len(lines) - 2} lines found")
    names, x, f = [], np.zeros((n, 3)), np.zeros((n, 3)) if cols["forces"] else None
    for i in range(n):
        t = lines[2 + i].split()
        names.append(t[cols["species"]])
        x[i] = [float(t[c]) for c in cols["pos"]]
        if f is not None:
            f[i] = [float(t[c]) for c in cols["forces"]]
    if R is not None:
        x = _wrap(x, R)
    return XYZStructure(names, x, R, energy, f)


def write_xyz(path, s: XYZStructure) -> None:
    R = s.cell if s.cell is not None else np.zeros((3, 3))
    lat = " ".join(f"{v:f}" for v in R.T.reshape(9))
    props = "species:S:1:pos:R:3" + (":forces:R:3" if s.forces is not None else "")
    out = [f"{len(s.names)}", f'Properties={props} potential_energy={s.energy:f} pbc="T T T" Lattice="{lat}"']
    for i, nm in enumerate(s.names):
        row = f"{nm:<2s} " + " ".join(f"{v:19.10f}" for v in s.posn[i])
        if s.forces is not None:
            row += " " + " ".join(f"{v:19.10f}" for v in s.forces[i])
        out.append(row)
    Path(path).write_text("\n".join(out) + "\n")


def batch_from_xyz(ctx, structures):
    """(atom_offsets, posn, types, cell) for ann_compute from read structures; the atom names are
    mapped to the loaded potential's type indices (NNP::index). Every structure needs a lattice."""
    from .api import pack_batch
    packed = []
    for s in structures:
        if s.cell is None:
            raise ValueError("a structure without a lattice cannot be computed periodically")
        t = np.array([ctx.type_index(nm) for nm in s.names], np.int32)
        packed.append((s.posn, t, s.cell))
    return pack_batch(packed)
