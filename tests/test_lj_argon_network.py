"""The MD workload's potential: tanh networks whose weights hold a Lennard-Jones argon pair
potential (workloads.lj_argon_text), checked on the oracle. The network is linear in its radial
inputs to 1e-5, its pair curve follows LJ (eps 10.4 meV, sigma 3.405 A, shifted at rc) to within
0.5 meV on [3, 6] A, and an FCC crystal under it stays a crystal in velocity-Verlet MD
(integrator.cpp:177-200, restated in the oracle) with bounded energy drift."""
import numpy as np
import pytest

from ann_gb300 import workloads as W
from ann_gb300.api import pack_batch

EPS, SIG, RC = 0.0104, 3.405, 6.0
KB = 8.617333262e-5


def _lj(r):
    return 4 * EPS * ((SIG / r) ** 12 - (SIG / r) ** 6) - 4 * EPS * ((SIG / RC) ** 12 - (SIG / RC) ** 6)


@pytest.fixture(scope="module")
def pot(oracle):
    return oracle.load_text(W.lj_argon_text(5))


def _energy(pot, structs):
    offs, posn, types, cell = pack_batch(structs)
    return pot.compute(offs, posn, types, cell, forces=False)[0]


def test_pair_curve(pot):
    L = np.eye(3) * 30.0
    e1 = _energy(pot, [(np.full((1, 3), 5.0), np.zeros(1, np.int32), L)])[0]
    assert abs(e1) < 1e-6                        # an isolated atom: G = 0, energy c.G = 0
    eta = W.radial_eta(8)
    c = W.lj_pair_coefficients(RC, eta)
    rs = np.linspace(3.0, 5.9, 30)
    structs = [(np.array([[5.0, 5, 5], [5.0 + r, 5, 5]]), np.zeros(2, np.int32), L) for r in rs]
    e = _energy(pot, structs) - 2 * e1
    lin = 2 * W._radial_g(rs, RC, eta)[0] @ c
    assert np.abs(e - lin).max() < 1e-5 * np.abs(lin).max() + 1e-7     # the network is linear in G
    assert np.abs(e - _lj(rs)).max() < 5e-4


def test_fcc_crystal_stays_in_md(pot):
    x, v, t, R = W.config5(cells=(3, 3, 3))
    offs, _, _, cell = pack_batch([(x, t, R)])
    F = pot.compute(offs, x, t, cell)[1]
    x, v = x.copy(), v.copy()
    masses = np.array([W.MASS["Ar"]])
    e0 = None
    for _ in range(300):
        pe, ke = pot.md_step(x, v, t, R, masses, 2.0, F)
        e0 = pe + ke if e0 is None else e0
    T = 2 * ke / (3 * len(x) * KB)
    assert 15.0 < T < 70.0, T                   # 80 K start relaxes toward equipartition (~40 K)
    d = x[:, None] - x[None]
    Ls = np.diag(R)
    d -= Ls * np.round(d / Ls)
    dd = np.linalg.norm(d, axis=2)
    np.fill_diagonal(dd, np.inf)
    assert dd.min() > 3.0
    assert abs(pe + ke - e0) / len(x) < 1e-5    # eV/atom over 0.6 ps
