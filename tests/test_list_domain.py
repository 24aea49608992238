"""The ghost-atom domain used by the caller-list tests (tests/lmp_domain.py), checked on the CPU:
within the cutoff, its full rows name exactly the oracle's periodic neighbours (atom, image), so a
list call on the domain computes the periodic structure."""
import numpy as np
import pytest

import cases
from lmp_domain import build_domain


def _pairs_domain(dom, rc):
    out = set()
    off = np.concatenate([[0], np.cumsum(dom.numneigh)])
    for i in range(dom.nlocal):
        for j in dom.neigh[off[i]:off[i + 1]]:
            if np.linalg.norm(dom.x[i] - dom.x[j]) < rc:
                out.add((i, int(dom.owner[j]), *map(int, dom.image[j])))
    return out


@pytest.mark.parametrize("case", ["binary", "tiny"])
def test_domain_rows_are_the_periodic_neighbours(oracle, case):
    structs = cases.small_binary(n_struc=1, seed=23) if case == "binary" else cases.tiny_cells()
    rc = 5.0
    for x, t, R in structs:
        dom = build_domain(x, t, R, rc + 1.0, seed=1)
        i, j, img, _, _ = oracle.neighbors(dom.x[:dom.nlocal], R, rc)
        ref = {(int(a), int(b), *map(int, n)) for a, b, n in zip(i, j, img)}
        assert _pairs_domain(dom, rc) == ref
        # rows hold the skin shell too, and every ghost is in some row
        assert dom.numneigh.sum() > len(ref)
        assert set(range(dom.nlocal, dom.nall)) <= set(dom.neigh.tolist())
        # folding a ghost force onto its owner
        F = np.zeros((dom.nall, 3))
        F[dom.nall - 1] = [1.0, 2.0, 3.0]
        assert np.array_equal(dom.fold(F)[dom.owner[-1]], [1.0, 2.0, 3.0])


@pytest.mark.parametrize("case", ["binary", "tiny"])
def test_fast_ghost_domain_matches(case):
    """ann_gb300.workloads.ghost_domain (k-d tree, the bench's LAMMPS-shaped domain) gives every
    local atom the same neighbours, by position, as the brute-force builder above."""
    pytest.importorskip("scipy")
    from ann_gb300 import workloads as W
    structs = cases.small_binary(n_struc=1, seed=23) if case == "binary" else cases.tiny_cells()
    for x, t, R in structs:
        X, T, owner, nn, nb = W.ghost_domain(x, t, R, 6.0)
        dom = build_domain(x, t, R, 6.0, shuffle=False)
        assert np.allclose(X[:len(t)], dom.x[:dom.nlocal], rtol=0, atol=1e-12) and np.array_equal(T, np.asarray(t)[owner])
        o1 = np.concatenate([[0], np.cumsum(nn)])
        o2 = np.concatenate([[0], np.cumsum(dom.numneigh)])
        for i in range(len(t)):
            a = sorted(map(tuple, np.round(X[nb[o1[i]:o1[i + 1]]], 9)))
            b = sorted(map(tuple, np.round(dom.x[dom.neigh[o2[i]:o2[i + 1]]], 9)))
            assert a == b, i
