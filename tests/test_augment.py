"""Taylor-perturbed training structures (ann_gb300.augment.taylor_perturb, the reference's
nnptefr2.cpp:2409-2479) vs the oracle's restatement on std::mt19937: bit-identical positions and
energies for every radial distribution, with and without covalent scaling; structures without
forces get no copies; the energy shift is the first-order Taylor term."""
import numpy as np
import pytest

from ann_gb300.augment import DIST, taylor_perturb


def _data(seed=1):
    rng = np.random.default_rng(seed)
    n = [5, 3, 7, 4]
    offs = np.concatenate([[0], np.cumsum(n)]).astype(np.int64)
    x = rng.uniform(0, 10, (offs[-1], 3))
    F = rng.normal(0, 0.5, (offs[-1], 3))
    F[offs[1]:offs[2]] = 0.0                  # a structure without forces: kept, not copied
    E = rng.normal(-100, 5, len(n))
    return offs, x, F, E


@pytest.mark.parametrize("dist", sorted(DIST))
@pytest.mark.parametrize("covalent", [False, True])
def test_matches_oracle_bit_for_bit(oracle, dist, covalent):
    offs, x, F, E = _data()
    rcov = np.linspace(0.8, 1.6, offs[-1]) if covalent else None
    a = taylor_perturb(offs, x, F, E, nadd=3, dist=dist, rdelta=0.05, seed=12345, rcov=rcov)
    b = oracle.taylor_perturb(offs, x, F, E, 3, DIST[dist], 0.05, 12345, rcov)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    assert len(a[3]) == 4 + 3 * 3 and list(a[3][:4]) == [0, 0, 0, 0]


def test_structure_rules_and_taylor_energy():
    offs, x, F, E = _data(2)
    o, X, Ee, src = taylor_perturb(offs, x, F, E, nadd=2, dist="NORMAL", rdelta=0.1, seed=7)
    assert list(src) == [0, 0, 0, 1, 2, 2, 2, 3, 3, 3]
    for k, s in enumerate(src):
        a0, a1 = offs[s], offs[s + 1]
        dx = X[o[k]:o[k + 1]] - x[a0:a1]
        assert np.isclose(Ee[k], E[s] - np.sum(dx * F[a0:a1]), rtol=0, atol=1e-12)
    with pytest.raises(ValueError):
        taylor_perturb(offs, x, F, E, nadd=1, dist=4)
