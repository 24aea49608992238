"""Generate the golden fixtures of tests/golden/ (run here, where the reference sources are).

ref_basis.npz : outputs of the reference's OWN cutoff / radial / angular basis code and special
                functions (src/nnp/cutoff.cpp, basis_radial.cpp, basis_angular.cpp,
                src/math/special.cpp compiled unmodified by oracle/Makefile into
                oracle/_ref/libref_basis.so) at seeded sample points: Cutoff::cutf/cutg,
                BasisR::symm/force/symmd, BasisA::symm/force/symmd, fmexp, coscut, sincut.
                The reference keeps no golden vectors of its own (its tests print, seeded from
                the clock), so these are the pins of the oracle's restatement.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from oracle_lib import RefBasis, eval_basisA, eval_basisR  # noqa: E402

SEED = 20261203


def main():
    ref = RefBasis()
    L = ref.L
    rng = np.random.default_rng(SEED)
    out = {}
    x = np.concatenate([rng.uniform(-745.0, 709.0, 400), rng.uniform(-5, 5, 200), [0.0, -1e-300, 1e-300]])
    out["fmexp_x"] = x
    out["fmexp_y"] = np.array([L.ref_fmexp(float(v)) for v in x])
    t = rng.uniform(0.0, np.pi, 200)
    out["cut_x"] = t
    out["coscut_y"] = np.array([L.ref_coscut(float(v)) for v in t])
    out["sincut_y"] = np.array([L.ref_sincut(float(v)) for v in t])
    # cutoffs
    rows = []
    for name in range(1, 5):
        for dr in rng.uniform(0.0, 7.0, 60):
            import ctypes as C
            f, g = C.c_double(), C.c_double()
            assert L.ref_cutoff(name, 6.0, float(dr), C.byref(f), C.byref(g)) == 0
            rows.append((name, 6.0, dr, f.value, g.value))
    out["cutoff"] = np.array(rows)
    # radial: per (function, cutoff) 30 points of 4 functions
    R_in, R_out = [], []
    for name in range(1, 7):
        for cut in range(1, 5):
            for _ in range(30):
                rs = rng.uniform(0.0, 3.0, 4); eta = rng.uniform(0.1, 2.0, 4)
                dr = float(rng.uniform(0.5, 7.0)); dE = rng.normal(size=4)
                s, amp, sd = eval_basisR(L, "ref_", cut, 6.0, name, rs, eta, dr, dE)
                R_in.append(np.concatenate([[name, cut, 6.0, dr], rs, eta, dE]))
                R_out.append(np.concatenate([s, [amp], sd]))
    out["radial_in"] = np.array(R_in)
    out["radial_out"] = np.array(R_out)
    # angular: eta in two groups (exercises the rflag grouping), integer and real zeta
    A_in, A_out = [], []
    for name in range(1, 7):
        for cut in range(1, 5):
            for _ in range(30):
                e = rng.uniform(1.0, 12.0, 2)
                eta = np.array([e[0], e[0], e[1], e[1]])
                zeta = rng.choice([1.0, 2.0, 4.0, 8.0, 1.5, 3.3], 4)
                lam = rng.choice([-1, 1], 4).astype(np.int32)
                dij, dik = rng.uniform(0.5, 7.0, 2); cs = float(rng.uniform(-1.0, 1.0)); dE = rng.normal(size=4)
                s, phi, e2, sd = eval_basisA(L, "ref_", cut, 6.0, name, eta, zeta, lam, float(dij), float(dik), cs, dE)
                A_in.append(np.concatenate([[name, cut, 6.0, dij, dik, cs], eta, zeta, lam, dE]))
                A_out.append(np.concatenate([s, [phi], e2, sd]))
    out["angular_in"] = np.array(A_in)
    out["angular_out"] = np.array(A_out)
    np.savez_compressed(HERE / "ref_basis.npz", **out)
    print("wrote", HERE / "ref_basis.npz", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
