"""The pw.x output reader (ann_gb300.io.read_qe_out, the reference's QE::OUT::read of
src/format/qe_struc.cpp:69-334): keys, unit conversions (Ry, bohr), wrapping, last-block rules,
on a synthetic output; and, where the reference's own example outputs are readable
(examples/Ar/md_nve.zip), on those."""
import zipfile
from pathlib import Path

import numpy as np
import pytest

from ann_gb300.io import BOHR2ANG, RY2EV, read_qe_out
from oracle_lib import REF_SRC

AR_ZIP = REF_SRC.parent / "examples" / "Ar" / "md_nve.zip"


def _pw_output(alat, axes, species, atoms, energies, forces_blocks, stress=None):
    """Text in the layout of a pw.x output, holding the lines the reader keys on."""
    out = ["     Program PWSCF", f"     lattice parameter (alat)  =      {alat:.4f}  a.u.",
           f"     number of atoms/cell      =           {len(atoms)}",
           f"     number of atomic types    =            {len(species)}",
           f"     number of electrons       =       {8.0 * len(atoms):.2f}", "",
           "     crystal axes: (cart. coord. in units of alat)"]
    out += [f"               a({c + 1}) = (  {axes[c][0]:10.6f} {axes[c][1]:10.6f} {axes[c][2]:10.6f} )  " for c in range(3)]
    out += ["", "     Pseudo is Norm-conserving, Zval =  8.0"] * len(species)
    out += ["", "     atomic species   valence    mass     pseudopotential"]
    out += [f"        {sp:<4s}           8.00    39.94800     {sp}( 1.00)" for sp in species]
    out += ["", "     site n.     atom                  positions (alat units)"]
    out += [f"         {i + 1}           {nm}  tau(   {i + 1}) = (  {x[0]:11.7f} {x[1]:11.7f} {x[2]:11.7f}  )" for i, (nm, x) in enumerate(atoms)]
    for e, F in zip(energies, forces_blocks):
        out += ["", f"!    total energy              =   {e:.8f} Ry", "", "     Forces acting on atoms (cartesian axes, Ry/au):", ""]
        out += [f"     atom    {i + 1} type  1   force =  {f[0]:13.8f} {f[1]:13.8f} {f[2]:13.8f}" for i, f in enumerate(F)]
    if stress is not None:
        out += ["", "     total   stress  (Ry/bohr**3)                   (kbar)     P=   1.00"]
        out += [f"   {s[0]:13.8f} {s[1]:13.8f} {s[2]:13.8f}          0.00        0.00        0.00" for s in stress]
    return "\n".join(out) + "\n"


def test_synthetic_output(tmp_path):
    axes = [[1.0, 0.0, 0.0], [0.1, 0.9, 0.0], [0.0, 0.2, 1.1]]
    atoms = [("Ar", [0.1, 0.2, 0.3]), ("Ne", [1.05, -0.1, 0.5]), ("Ar", [0.5, 0.5, 0.5])]
    F1 = np.array([[0.1, 0.0, 0.0], [0.0, 0.2, 0.0], [-0.1, -0.2, 0.0]])
    F2 = np.array([[0.01, 0.02, 0.03], [-0.01, 0.0, -0.02], [0.0, -0.02, -0.01]])
    stress = np.array([[1e-4, 2e-5, 0.0], [2e-5, 3e-4, 0.0], [0.0, 0.0, -1e-4]])
    p = tmp_path / "pw.out"
    p.write_text(_pw_output(12.5, axes, ["Ar", "Ne"], atoms, [-100.25, -100.5], [F1, F2], stress))
    s = read_qe_out(p)
    alat = 12.5 * BOHR2ANG
    R = alat * np.array(axes).T
    assert np.allclose(s.cell, R, rtol=1e-15)
    assert s.names == ["Ar", "Ne", "Ar"] and s.species == ["Ar", "Ne"] and list(s.types) == [0, 1, 0]
    assert s.energy == pytest.approx(-100.5 * RY2EV, rel=1e-15)            # the last energy
    assert np.allclose(s.forces, F2 * RY2EV / BOHR2ANG, rtol=1e-15)       # the last force block
    assert np.allclose(s.stress, stress * RY2EV / BOHR2ANG ** 3, rtol=1e-15)
    # positions: alat units -> A, wrapped into the cell (the second atom lies outside it)
    frac = np.linalg.solve(R, s.posn.T).T
    assert np.all(frac >= 0) and np.all(frac < 1)
    raw = alat * np.array([a[1] for a in atoms])
    d = np.linalg.solve(R, (s.posn - raw).T).T
    assert np.allclose(d, np.round(d), atol=1e-9)
    assert s.qtot == 0.0


def test_missing_keys_raise(tmp_path):
    p = tmp_path / "bad.out"
    p.write_text("     Program PWSCF\n     number of atoms/cell      =           2\n")
    with pytest.raises(ValueError, match="species"):
        read_qe_out(p)


@pytest.mark.skipif(not AR_ZIP.exists(), reason="the reference's example outputs are not readable here")
def test_reference_argon_outputs(tmp_path):
    z = zipfile.ZipFile(AR_ZIP)
    names = [n for n in z.namelist() if n.endswith(".out")][:4]
    for n in names:
        p = tmp_path / Path(n).name
        p.write_bytes(z.read(n))
        s = read_qe_out(p)
        text = p.read_text()
        e_ry = [float(ln.split("=")[1].split()[0]) for ln in text.splitlines() if ln.startswith("!    total energy")][-1]
        assert len(s.names) == 32 and set(s.names) == {"Ar"}
        assert s.energy == pytest.approx(e_ry * RY2EV, rel=1e-15)
        assert np.max(np.abs(s.forces.sum(axis=0))) < 1e-4
        frac = np.linalg.solve(s.cell, s.posn.T).T
        assert np.all(frac >= 0) and np.all(frac < 1)
