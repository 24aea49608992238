"""Structure files: the extended-XYZ reader and writer of the reference (XYZ::read / XYZ::write,
src/format/xyz_struc.cpp:38-266) and its Quantum ESPRESSO pw.x output reader (QE::OUT::read,
src/format/qe_struc.cpp:69-334), in metal units, and packing of read structures into a batch for
the library (types resolved by the potential's type names).

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


# ------------------------------------------------------------------------ Quantum ESPRESSO output
BOHR2ANG = 0.529177210903          # chem/units.hpp:30
EH2EV = 27.211386245988            # chem/units.hpp:24
RY2EV = 0.5 * EH2EV                # pw.x energies are in Rydberg


@dataclass
class QEStructure(XYZStructure):
    types: np.ndarray | None = None      # index into species, in the file's species order
    species: list | None = None
    stress: np.ndarray | None = None     # (3, 3) eV/A^3 when the file has a stress block
    qtot: float = 0.0                    # sum of Zval over atoms minus the number of electrons


_NUM = re.compile(r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eEdD][-+]?\d+)?")


def _after_eq(line: str) -> float:
    m = _NUM.search(line.split("=", 1)[1])
    if m is None:
        raise ValueError(f"no number in {line!r}")
    return float(m.group(0).replace("d", "e").replace("D", "E"))


def read_qe_out(path, with_forces: bool = True) -> QEStructure:
    """One pw.x output file as QE::OUT::read reads it (metal units): the last '!    total energy'
    (Ry -> eV), 'lattice parameter' alat (bohr -> A), 'crystal axes' (alat units, the lattice
    vectors as columns), 'number of atoms/cell', 'number of atomic types', the 'atomic species'
    names, the last 'site n.' block (alat units, wrapped into the cell as Cell::returnToCell), the
    last 'Forces' block (Ry/bohr -> eV/A) and the last 'total   stress' block (Ry/bohr^3 -> eV/A^3)."""
    lines = Path(path).read_text().splitlines()
    energy, alat, nat, nsp = 0.0, 0.0, 0, 0
    lv = np.zeros((3, 3))
    species, zval, nelect = [], [], 0
    pos_at = force_at = stress_at = -1
    for k, ln in enumerate(lines):
        if "!    total energy" in ln:
            energy = RY2EV * _after_eq(ln)
        elif "crystal axes" in ln:
            for c in range(3):
                t = lines[k + 1 + c].replace("(", " ").replace(")", " ").split()
                lv[:, c] = [float(v) for v in t[3:6]]
        elif "lattice parameter" in ln:
            alat = BOHR2ANG * _after_eq(ln)
        elif "number of atoms/cell" in ln:
            nat = int(_after_eq(ln))
        elif "number of atomic types" in ln:
            nsp = int(_after_eq(ln))
        elif "atomic species  " in ln:
            species = [lines[k + 1 + q].split()[0] for q in range(nsp)]
        elif "Zval" in ln:
            zval.append(round(_after_eq(ln)))
        elif "number of electrons" in ln:
            nelect = round(_after_eq(ln))
        elif "site n." in ln:
            pos_at = k
        elif "Forces" in ln:
            force_at = k
        elif "total   stress" in ln:
            stress_at = k
    if nsp <= 0:
        raise ValueError(f"{path}: number of species not found")
    if nat <= 0:
        raise ValueError(f"{path}: number of atoms not found")
    if len(species) != nsp:
        raise ValueError(f"{path}: species names not found")
    if alat <= 0 or not np.linalg.norm(lv) > 0:
        raise ValueError(f"{path}: alat / crystal axes not found")
    R = alat * lv
    if abs(np.linalg.det(R)) < 1e-12:
        raise ValueError(f"{path}: invalid lattice vector matrix")
    if pos_at < 0:
        raise ValueError(f"{path}: no atomic positions")
    names, x = [], np.zeros((nat, 3))
    for i in range(nat):
        t = lines[pos_at + 1 + i].replace("(", " ").replace(")", " ").split()
        names.append(t[1])
        x[i] = [float(v) for v in t[5:8]]
    if any(nm not in species for nm in names):
        raise ValueError(f"{path}: invalid species name in atomic positions")
    types = np.array([species.index(nm) for nm in names], np.int32)
    x = _wrap(x * alat, R)
    F = None
    if with_forces and force_at >= 0:
        F = np.zeros((nat, 3))
        for i in range(nat):
            t = lines[force_at + 2 + i].split()
            F[i] = [float(v) for v in t[6:9]]
        F *= RY2EV / BOHR2ANG
    S = None
    if stress_at >= 0:
        S = np.array([[float(v) for v in lines[stress_at + 1 + r].split()[:3]] for r in range(3)]) * (RY2EV / BOHR2ANG ** 3)
    counts = [names.count(sp) for sp in species]
    qtot = float(sum(z * n for z, n in zip(zval, counts)) - nelect) if len(zval) == nsp else 0.0
    return QEStructure(names, x, R, energy, F, types=types, species=species, stress=S, qtot=qtot)
