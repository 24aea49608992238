"""The oracle's cell-binned neighbour search against its all-pairs definition, and one structure
split over threads against the serial pass (CPU only).

The binned search serves structures of more than 512 atoms whose cell holds three or more bins of
height rc along every lattice direction; it must give the same (i, j, image) set, the same pair
vectors bit for bit and the same row order as the brute force over all atoms and images.
"""
import numpy as np
import pytest

from ann_gb300 import workloads as W
from ann_gb300.api import pack_batch


def _cases():
    rng = np.random.default_rng(17)
    out = []
    x, t, R = W.config4(dims=(12, 12, 8))[0]                  # 1,152 atoms, orthorhombic
    out.append((x, R, 6.0))
    R = np.array([[22.0, 3.0, 1.5], [0.0, 20.5, 2.0], [0.0, 0.0, 21.0]])   # triclinic, 700 atoms
    out.append((rng.uniform(0, 1, (700, 3)) @ R.T, R, 6.5))
    x, t, R = W.random_binary(1, 600, 700, seed=3)[0]       # one binary structure at the workload's density
    out.append((x, R, 6.5))
    x = rng.uniform(-30, 50, (600, 3))                       # unwrapped coordinates in a cubic cell
    out.append((x, np.eye(3) * 19.0, 6.0))
    return out


@pytest.mark.parametrize("case", range(4))
def test_binned_equals_brute_force(oracle, case):
    cs = _cases()
    if case >= len(cs):
        pytest.skip("case not generated")
    x, R, rc = cs[case]
    a = oracle.neighbors(x, R, rc)
    b = oracle.neighbors(x, R, rc, brute=True)
    assert len(a[0]) == len(b[0]) > 0
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def test_one_structure_over_threads(oracle):
    pot = oracle.load_text(W.config_potential_text(4))
    x, t, R = W.config4(dims=(10, 10, 8))[0]
    offs, posn, types, cell = pack_batch([(x, t, R)])
    E1, F1, W1, G1, D1 = pot.compute(offs, posn, types, cell, symm=True, dedg=True, nthreads=1)
    E4, F4, W4, G4, D4 = pot.compute(offs, posn, types, cell, symm=True, dedg=True, nthreads=4)
    assert np.array_equal(G4, G1) and np.array_equal(D4, D1)
    assert abs(E4[0] - E1[0]) <= 1e-12 * abs(E1[0])
    assert np.max(np.abs(F4 - F1)) <= 1e-12 * np.max(np.abs(F1))
    assert np.max(np.abs(W4 - W1)) <= 1e-12 * np.max(np.abs(W1))
