"""Builds tests/golden/ar_qe.npz from the reference's argon example: the files its trainer input
lists (examples/Ar/nn_pot_train_init.txt: data_train = data_deform_iso_train.txt, isotropic
deformations of a one-atom FCC cell; data_val = data_md_nve.txt, NVE MD frames of 32 atoms), read
from examples/Ar/deform_iso.zip and md_nve.zip (pw.x outputs). Every file is read with ann_gb300.io.read_qe_out
(the reference's QE::OUT::read) into metal units and stored as arrays: positions (A, wrapped),
cells (lattice vectors as columns), energies (eV), forces (eV/A).

Usage: python tests/golden/make_ar_qe_fixture.py [reference root]   (default: the root that
tests/oracle_lib.py uses for the reference sources)."""
import sys
import tempfile
import zipfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE.parent))

from ann_gb300.io import read_qe_out  # noqa: E402


def read_set(zpath, listfile):
    z = zipfile.ZipFile(zpath)
    want = [ln.strip().lstrip("./") for ln in listfile.read_text().splitlines() if ln.strip()]
    names = [n for n in want if n in z.namelist()]
    if len(names) != len(want):
        raise FileNotFoundError(f"{zpath}: files of {listfile.name} missing")
    X, C, E, F = [], [], [], []
    with tempfile.TemporaryDirectory() as d:
        for n in names:
            p = Path(d) / Path(n).name
            p.write_bytes(z.read(n))
            s = read_qe_out(p)
            X.append(s.posn); C.append(s.cell); E.append(s.energy); F.append(s.forces)
    return np.array(X), np.array(C), np.array(E), np.array(F), names


def main():
    if len(sys.argv) > 1:
        root = Path(sys.argv[1])
    else:
        from oracle_lib import REF_SRC
        root = REF_SRC.parent
    ex = root / "examples" / "Ar"
    tx, tc, te, tf, tn = read_set(ex / "deform_iso.zip", ex / "data_deform_iso_train.txt")
    vx, vc, ve, vf, vn = read_set(ex / "md_nve.zip", ex / "data_md_nve.txt")
    np.savez_compressed(HERE / "ar_qe.npz", train_posn=tx, train_cell=tc, train_energy=te, train_forces=tf,
                        val_posn=vx, val_cell=vc, val_energy=ve, val_forces=vf,
                        train_files=np.array(tn), val_files=np.array(vn))
    print(f"train {len(te)} structures, validation {len(ve)} structures -> {HERE / 'ar_qe.npz'}")


if __name__ == "__main__":
    main()
