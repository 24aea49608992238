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


@pytest.mark.skipif(not __import__("oracle_lib").REF_SRC.exists(), reason="reference sources not present on this machine")
def test_reference_on_domain_is_the_periodic_structure(oracle, tmp_path):
    """The reference's own NNP (nnp.cpp compiled with the struc stand-ins) on an MD engine's
    domain: local atoms as the centres, ghosts only as neighbours, the full rows cut to rc, the
    Newton's-third-law reaction on every entry. Its energy is the periodic structure's, and its
    local + ghost forces, folded onto the owners, are the oracle's periodic forces: the semantics
    of the caller-list entry point, ann_compute_list, held to the reference's code."""
    from pathlib import Path
    from ann_gb300.api import pack_batch
    from oracle_lib import RefNNP
    ref = RefNNP()
    gold = np.load(Path(__file__).resolve().parent / "golden" / "ref_nnp.npz")
    for name in [str(n) for n in gold["pot_names"]]:
        text = str(gold[f"pot_{name}"])
        p = tmp_path / f"{name}.ann"
        p.write_text(text)
        h = ref.read(p)
        try:
            pot = oracle.load_text(text)
            nt, rc = pot.ntypes, ref.L.ref_nnp_rc(h)
            for x, t, R in cases.small_binary(n_struc=1, seed=23) + cases.tiny_cells()[:2]:
                t = (np.asarray(t) % nt).astype(np.int32)
                dom = build_domain(x, t, R, rc + 1.0, seed=2)
                off = np.concatenate([[0], np.cumsum(dom.numneigh)])
                ei = np.repeat(np.arange(dom.nlocal), dom.numneigh)
                ej = dom.neigh
                keep = np.linalg.norm(dom.x[ei] - dom.x[ej], axis=1) < rc
                assert off[-1] == len(ej)
                E, F = ref.domain(h, dom.nlocal, dom.type, dom.x, ei[keep], ej[keep])
                offs, posn, types, cell = pack_batch([(dom.x[:dom.nlocal], dom.type[:dom.nlocal], R)])
                E0, F0, _, _, _ = pot.compute(offs, posn, types, cell)
                assert abs(E - E0[0]) <= 1e-12 * max(1.0, abs(E0[0])), name
                assert np.abs(dom.fold(F) - F0).max() <= 1e-12 * max(1.0, np.abs(F0).max()), name
                assert np.abs(F[dom.nlocal:]).max() > 0.0      # the ghosts carry force for the owners
        finally:
            ref.L.ref_nnp_free(h)
