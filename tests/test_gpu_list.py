"""ann_compute_list: energies and forces from the caller's full neighbour list over local and ghost
atoms (the LAMMPS pair style shape) vs the CPU oracle on the same periodic structures.

The domain is what LAMMPS passes a pair style: wrapped local atoms, ghost images, full rows built
with a skin and shuffled. After the ghost forces are added to their owners (reverse
communication), the result must be the periodic structure's: FP64 within 1e-10 relative of the
oracle, mixed within 1 meV/atom and 10 meV/A of it."""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, AnnError, Context
from lmp_domain import build_domain

pytestmark = pytest.mark.gpu

REL = 1e-10
E_MEV_ATOM = 1.0
F_MEV_A = 10.0


def _rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300)


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = Context()
    yield c
    c.close()


def _oracle(pot, x, t, R):
    offs, posn, types, cell = cases.batch([(x, t, R)])
    E, F, Wv, _, _ = pot.compute(offs, posn, types, cell)
    return E[0], F, Wv[0]


def _check(ctx, dom, Eo, Fo, Wo, prec, skin_rows=True):
    E, F, Wv, ea = ctx.compute_list(dom.x, dom.type, dom.numneigh, dom.neigh, eatom=True, precision=prec)
    Fl = dom.fold(F)
    n = dom.nlocal
    if prec == FP64:
        assert _rel(E, Eo) < REL, (E, Eo)
        assert _rel(Fl, Fo) < REL
        assert _rel(Wv, Wo) < REL
        assert abs(ea.sum() - E) <= 1e-12 * max(abs(E), 1.0)
    else:
        assert abs(E - Eo) / n * 1e3 < E_MEV_ATOM
        assert np.max(np.abs(Fl - Fo)) * 1e3 < F_MEV_A
    return E, F, Wv, ea


@pytest.mark.parametrize("skin", [0.0, 1.5])
def test_binary_domain_matches_oracle(ctx, oracle, tmp_path, skin):
    structs = cases.small_binary(n_struc=2, seed=23)
    offs, posn, types, cell = cases.batch(structs)
    text = cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    pot = oracle.load_text(text)
    for x, t, R in structs:
        dom = build_domain(x, t, R, ctx.rc + skin, seed=1)
        Eo, Fo, Wo = _oracle(pot, dom.x[:dom.nlocal], t, R)
        _check(ctx, dom, Eo, Fo, Wo, FP64)
        _check(ctx, dom, Eo, Fo, Wo, MIXED)


def test_small_cells_and_generic_basis(ctx, oracle):
    """Cells smaller than the cutoff (an atom's own images are its neighbours), a triclinic cell,
    and the generic basis variants / cutoffs."""
    text = cases.generic_potential_text()
    ctx.load_text(text)
    pot = oracle.load_text(text)
    for x, t, R in cases.tiny_cells():
        dom = build_domain(x, t, R, ctx.rc + 0.7, seed=4)
        Eo, Fo, Wo = _oracle(pot, dom.x[:dom.nlocal], t, R)
        _check(ctx, dom, Eo, Fo, Wo, FP64)


def test_ilist_permutation_and_subset(ctx, oracle, tmp_path):
    """Rows in any order (ilist) give per-row energies of their atoms; a subset of rows (a group)
    gives the energy of those atoms and the forces of their energy alone."""
    structs = cases.small_binary(n_struc=1, seed=31)
    offs, posn, types, cell = cases.batch(structs)
    cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    x, t, R = structs[0]
    dom = build_domain(x, t, R, ctx.rc + 1.0, seed=2)
    E0, F0, W0, ea0 = ctx.compute_list(dom.x, dom.type, dom.numneigh, dom.neigh, eatom=True, precision=FP64)
    rng = np.random.default_rng(7)
    perm = rng.permutation(dom.nlocal).astype(np.int32)
    nn, nb = dom.rows(perm)
    E1, F1, W1, ea1 = ctx.compute_list(dom.x, dom.type, nn, nb, ilist=perm, eatom=True, precision=FP64)
    assert abs(E1 - E0) <= 1e-12 * abs(E0)
    assert np.max(np.abs(ea1 - ea0[perm])) <= 1e-12 * np.max(np.abs(ea0))
    assert _rel(F1, F0) < 1e-12 and _rel(W1, W0) < 1e-12
    sub = perm[: dom.nlocal // 3]
    nn, nb = dom.rows(sub)
    E2, F2, _, ea2 = ctx.compute_list(dom.x, dom.type, nn, nb, ilist=sub, eatom=True, precision=FP64)
    assert abs(E2 - ea0[sub].sum()) <= 1e-12 * max(abs(E2), 1.0)
    # the group's forces: F = -d(sum of the group's energies)/dx; their total vanishes (translation)
    assert np.max(np.abs(F2.sum(axis=0))) < 1e-9 * max(np.max(np.abs(F2)), 1.0)
    assert not np.allclose(F2, F0)


def test_capacity_grows_with_denser_rows(gpu_lib, oracle, tmp_path):
    """A sparse domain first (short rows set the capacity hint), then a denser one whose rows
    overflow that capacity: the call regrows and recomputes."""
    c = Context()
    try:
        sparse = cases.W.random_binary(1, 40, 40, seed=3, rho=0.02)[0]
        dense = cases.small_binary(n_struc=1, seed=5)[0]
        text = cases.config_potential(c, 2, tmp_path)
        pot = oracle.load_text(text)
        for x, t, R in (sparse, dense):
            dom = build_domain(x, t, R, c.rc + 2.0, seed=3)
            Eo, Fo, Wo = _oracle(pot, dom.x[:dom.nlocal], t, R)
            _check(c, dom, Eo, Fo, Wo, FP64)
    finally:
        c.close()


def test_list_errors_leave_the_context_usable(ctx, oracle, tmp_path):
    structs = cases.small_binary(n_struc=1, seed=9)
    offs, posn, types, cell = cases.batch(structs)
    text = cases.config_potential(ctx, 2, tmp_path)
    pot = oracle.load_text(text)
    x, t, R = structs[0]
    dom = build_domain(x, t, R, ctx.rc + 0.5, seed=5)
    bad = dom.neigh.copy()
    bad[len(bad) // 2] = dom.nall                      # index past the last ghost
    with pytest.raises(AnnError, match="outside"):
        ctx.compute_list(dom.x, dom.type, dom.numneigh, bad, precision=FP64)
    bt = dom.type.copy()
    bt[-1] = 7                                         # a ghost with a type the potential lacks
    with pytest.raises(AnnError, match="type"):
        ctx.compute_list(dom.x, bt, dom.numneigh, dom.neigh, precision=FP64)
    nn = dom.numneigh.copy()
    nn[0] = -1
    with pytest.raises(AnnError, match="numneigh"):
        ctx.compute_list(dom.x, dom.type, nn, dom.neigh, precision=FP64)
    bx = dom.x.copy()
    bx[dom.neigh[0]] = np.nan
    with pytest.raises(AnnError, match="non-finite"):
        ctx.compute_list(bx, dom.type, dom.numneigh, dom.neigh, precision=FP64)
    Eo, Fo, Wo = _oracle(pot, dom.x[:dom.nlocal], t, R)
    _check(ctx, dom, Eo, Fo, Wo, FP64)
    # an empty call
    E, F, Wv, _ = ctx.compute_list(np.zeros((0, 3)), np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32),
                                   precision=FP64)
    assert E == 0.0 and F.shape == (0, 3) and np.all(Wv == 0)


def test_list_and_batch_paths_interleave(ctx, oracle, tmp_path):
    """A list call between a staged batch and its download leaves the batch's results alone."""
    structs = cases.small_binary(n_struc=3, seed=13)
    offs, posn, types, cell = cases.batch(structs)
    cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    E0, F0, _ = ctx.compute(offs, posn, types, cell, precision=MIXED)
    ctx.upload(offs, posn, types, cell)
    ctx.compute_resident(precision=MIXED)
    x, t, R = structs[1]
    dom = build_domain(x, t, R, ctx.rc + 1.0, seed=8)
    El, Fl, _, _ = ctx.compute_list(dom.x, dom.type, dom.numneigh, dom.neigh, precision=MIXED)
    E1, F1, _ = ctx.download()
    assert np.array_equal(E1, E0)
    assert abs(El - E0[1]) / len(t) * 1e3 < E_MEV_ATOM


def test_keep_list_between_reneighbourings(ctx, oracle, tmp_path):
    """ANN_LIST_KEEP: the list of the previous call with new positions (atoms moved by less than
    half the skin, as between two reneighbourings) equals a full call and the oracle."""
    structs = cases.small_binary(n_struc=1, seed=19)
    offs, posn, types, cell = cases.batch(structs)
    text = cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    pot = oracle.load_text(text)
    x, t, R = structs[0]
    skin = 1.0
    dom = build_domain(x, t, R, ctx.rc + skin, seed=3)
    ctx.compute_list(dom.x, dom.type, dom.numneigh, dom.neigh, precision=FP64)
    rng = np.random.default_rng(5)
    d = rng.normal(0.0, 1.0, (dom.nlocal, 3))
    d *= (0.45 * skin / 2) / np.linalg.norm(d, axis=1, keepdims=True)   # < skin / 2 per atom
    x1 = dom.x + d[dom.owner]                                         # ghosts move with their owners
    E1, F1, W1, _ = ctx.compute_list(x1, None, None, None, precision=FP64, keep=True, inum=dom.nlocal)
    E2, F2, W2, _ = ctx.compute_list(x1, dom.type, dom.numneigh, dom.neigh, precision=FP64)
    assert abs(E1 - E2) <= 1e-13 * abs(E2) and _rel(F1, F2) < 1e-12 and _rel(W1, W2) < 1e-12
    Eo, Fo, Wo = _oracle(pot, x1[:dom.nlocal], t, R)
    assert _rel(E1, Eo) < REL and _rel(dom.fold(F1), Fo) < REL and _rel(W1, Wo) < REL
    Em, Fm, _, _ = ctx.compute_list(x1, None, None, None, precision=MIXED, keep=True, inum=dom.nlocal)
    assert abs(Em - Eo) / dom.nlocal * 1e3 < E_MEV_ATOM and np.max(np.abs(dom.fold(Fm) - Fo)) * 1e3 < F_MEV_A
    with pytest.raises(AnnError, match="differ"):
        ctx.compute_list(x1[:-1], None, None, None, precision=FP64, keep=True, inum=dom.nlocal)
    c2 = Context()
    try:
        c2.load_text(text)
        with pytest.raises(AnnError, match="staged"):
            c2.compute_list(x1, None, None, None, precision=FP64, keep=True, inum=dom.nlocal)
    finally:
        c2.close()


def test_large_domain_matches_periodic_batch(gpu_lib, tmp_path):
    """A 16,384-atom FCC box as an MD engine's domain (k-d tree ghosts, full list with a 2 A skin,
    as the LAMMPS-shaped bench leg builds it): the list call gives the periodic box's energy and,
    after folding the ghost forces, its forces, in FP64 and in mixed precision."""
    pytest.importorskip("scipy")
    c = Context()
    try:
        cases.W.make_potential(c, 5)
        x, R = cases.W.fcc(16, 16, 16, 5.26)
        rng = np.random.default_rng(12)
        x = x + rng.normal(0.0, 0.05, x.shape)
        t = np.zeros(len(x), np.int32)
        X, T, owner, nn, nb = cases.W.ghost_domain(x, t, R, c.rc + 2.0)
        offs, posn, types, cell = cases.batch([(X[:len(t)], t, R)])
        for prec, tol_e, tol_f in ((FP64, 1e-11, 1e-9), (MIXED, 1e-6, 2e-3)):
            E0, F0, W0 = c.compute(offs, posn, types, cell, precision=prec)
            E, F, Wv, _ = c.compute_list(X, T, nn, nb, precision=prec)
            Ff = np.zeros((len(t), 3))
            np.add.at(Ff, owner, F)
            assert abs(E - E0[0]) <= tol_e * abs(E0[0]), (prec, E, E0[0])
            assert np.max(np.abs(Ff - F0)) <= tol_f * max(np.max(np.abs(F0)), 1.0), prec
            assert np.max(np.abs(Wv - W0[0])) <= tol_f * np.max(np.abs(W0[0])), prec
    finally:
        c.close()
