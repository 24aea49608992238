"""GPU path vs the CPU oracle on the same seeded inputs, through the C ABI.

Bars (the benchmark spec): the FP64 pipeline matches the oracle with neighbour lists bit-exact and
energies / forces / virials within 1e-10 relative; the mixed pipeline (FP32 basis and forces,
FP32-accumulated networks, FP64 energy sums) stays within 1 meV/atom and 10 meV/A of FP64.
"""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, Context

pytestmark = pytest.mark.gpu

REL = 1e-10          # FP64 pipeline vs oracle, relative to the largest magnitude
E_MEV_ATOM = 1.0     # mixed vs FP64
F_MEV_A = 10.0


def _rel_err(a, b):
    scale = max(np.max(np.abs(b)), 1e-300)
    return np.max(np.abs(a - b)) / scale


def _neigh_sets(i, j, img, r):
    key = np.lexsort((img[:, 2], img[:, 1], img[:, 0], j, i))
    return i[key], j[key], img[key], r[key]


def _oracle_neighbors(oracle, offs, posn, types, cell, rc):
    I, J, IMG, R = [], [], [], []
    for s in range(len(offs) - 1):
        a0, a1 = offs[s], offs[s + 1]
        if a1 == a0:
            continue
        Rm = cell[s].reshape(3, 3).T
        i, j, img, r, _ = oracle.neighbors(posn[a0:a1], Rm, rc)
        I.append(i + a0); J.append(j + a0); IMG.append(img); R.append(r)
    return (np.concatenate(I), np.concatenate(J), np.concatenate(IMG), np.concatenate(R))


def _check_fp64(ctx, pot, oracle, offs, posn, types, cell, check_nl=True):
    E, F, Wv = ctx.compute(offs, posn, types, cell, precision=FP64)
    Eo, Fo, Wo, Go, Do = pot.compute(offs, posn, types, cell, symm=True, dedg=True)
    G = ctx.symm()
    D = ctx.dedg()
    assert _rel_err(G, Go) < 1e-12, "symmetry functions"
    assert _rel_err(D, Do) < 1e-10, "dE/dG"
    assert _rel_err(E, Eo) < REL, ("energy", E, Eo)
    assert _rel_err(F, Fo) < REL, "forces"
    assert _rel_err(Wv, Wo) < REL, "virial"
    if check_nl:
        i, j, img, r = ctx.neighbors(with_vectors=True)
        io, jo, imgo, ro = _oracle_neighbors(oracle, offs, posn, types, cell, ctx.rc)
        a = _neigh_sets(i, j, img, r)
        b = _neigh_sets(io, jo, imgo, ro)
        assert len(a[0]) == len(b[0]), "neighbour count"
        for x, y in zip(a, b):
            assert np.array_equal(x, y), "neighbour list differs"
    return E, F, Wv


def _check_mixed(ctx, offs, posn, types, cell, E64, F64):
    E, F, _ = ctx.compute(offs, posn, types, cell, precision=MIXED)
    nat = np.diff(offs)
    e_err = np.max(np.abs(E - E64) / np.maximum(nat, 1)) * 1e3
    f_err = np.max(np.abs(F - F64)) * 1e3 if len(F) else 0.0
    assert e_err < E_MEV_ATOM, f"mixed energy error {e_err} meV/atom"
    assert f_err < F_MEV_A, f"mixed force error {f_err} meV/A"


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = Context(use_graphs=True)
    yield c
    c.close()


def test_config1_fcc_argon(ctx, oracle, tmp_path):
    offs, posn, types, cell = cases.batch(cases.W.config1())
    text = cases.config_potential(ctx, 1, tmp_path)
    pot = oracle.load_text(text)
    E, F, _ = _check_fp64(ctx, pot, oracle, offs, posn, types, cell)
    _check_mixed(ctx, offs, posn, types, cell, E, F)
    assert np.max(np.abs(F.sum(axis=0))) < 1e-9, "momentum conservation"


def test_binary_batch(ctx, oracle, tmp_path):
    structs = cases.small_binary()
    offs, posn, types, cell = cases.batch(structs)
    text = cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    pot = oracle.load_text(text)
    E, F, _ = _check_fp64(ctx, pot, oracle, offs, posn, types, cell)
    _check_mixed(ctx, offs, posn, types, cell, E, F)


def test_ternary_box(ctx, oracle, tmp_path):
    offs, posn, types, cell = cases.batch(cases.ternary_box())
    text = cases.config_potential(ctx, 4, tmp_path, precondition_batch=(offs, posn, types, cell))
    pot = oracle.load_text(text)
    E, F, _ = _check_fp64(ctx, pot, oracle, offs, posn, types, cell)
    _check_mixed(ctx, offs, posn, types, cell, E, F)


def test_small_cells_images_unwrapped(ctx, oracle, tmp_path):
    structs = cases.tiny_cells()
    offs, posn, types, cell = cases.batch(structs)
    text = cases.config_potential(ctx, 2, tmp_path)
    pot = oracle.load_text(text)
    E, F, _ = _check_fp64(ctx, pot, oracle, offs, posn, types, cell)
    _check_mixed(ctx, offs, posn, types, cell, E, F)


def test_generic_basis_variants(ctx, oracle, tmp_path):
    text = cases.generic_potential_text()
    ctx.load_text(text)
    pot = oracle.load_text(text)
    structs = cases.small_binary(n_struc=3, seed=21) + cases.tiny_cells()
    offs, posn, types, cell = cases.batch(structs)
    E, F, _ = _check_fp64(ctx, pot, oracle, offs, posn, types, cell)
    _check_mixed(ctx, offs, posn, types, cell, E, F)


def test_step_cutoff_logcosh2_and_cos_generic(ctx, oracle):
    """The variants the generic potential above leaves out: the STEP cutoff (cutoff.cpp:62-146),
    the LOGCOSH2 radial form (basis_radial.cpp:263-379), and the COS cutoff on generic angular forms."""
    text = cases.generic_potential_text()
    for blk in ("BasisR", "BasisA"):                   # every block of a type shares its cutoff
        text = text.replace(f"{blk} TANH 5.000000", f"{blk} STEP 5.000000").replace(f"{blk} POLY3 5.000000", f"{blk} COS 5.000000")
    text = text.replace("STEP 5.000000 SECH 3", "STEP 5.000000 LOGCOSH2 3").replace("COS 5.000000 LOGCOSH 2", "COS 5.000000 LOGCOSH2 2")
    assert text.count("LOGCOSH2") == 2 and text.count("STEP") == 5 and text.count(" COS ") == 5
    ctx.load_text(text)
    pot = oracle.load_text(text)
    structs = cases.small_binary(n_struc=3, seed=25) + cases.tiny_cells()
    offs, posn, types, cell = cases.batch(structs)
    E, F, _ = _check_fp64(ctx, pot, oracle, offs, posn, types, cell)
    _check_mixed(ctx, offs, posn, types, cell, E, F)


def test_large_structure_reductions(ctx, oracle, tmp_path):
    """A structure of 2,600 atoms (eleven reduction chunks of at most 256 atoms) between two
    small ones: energies and virials as the oracle's, also in the mixed form."""
    big = cases.W.random_binary(1, 2600, 2600, seed=77)
    structs = cases.small_binary(n_struc=1, seed=3) + big + cases.tiny_cells()[:1]
    offs, posn, types, cell = cases.batch(structs)
    text = cases.config_potential(ctx, 2, tmp_path)
    pot = oracle.load_text(text)
    E, F, Wv = ctx.compute(offs, posn, types, cell, precision=FP64)
    Eo, Fo, Wo, _, _ = pot.compute(offs, posn, types, cell)
    assert _rel_err(E, Eo) < REL and _rel_err(F, Fo) < REL and _rel_err(Wv, Wo) < REL
    _check_mixed(ctx, offs, posn, types, cell, E, F)


def test_empty_and_single_structures(ctx, oracle, tmp_path):
    text = cases.config_potential(ctx, 2, tmp_path)
    pot = oracle.load_text(text)
    s = cases.tiny_cells()
    structs = [s[0], (np.zeros((0, 3)), np.zeros(0, np.int32), np.eye(3) * 5.0), s[2]]
    offs, posn, types, cell = cases.batch(structs)
    E, F, Wv = ctx.compute(offs, posn, types, cell, precision=FP64)
    Eo, Fo, Wo, _, _ = pot.compute(offs, posn, types, cell)
    assert E[1] == 0.0
    assert _rel_err(E, Eo) < REL and _rel_err(F, Fo) < REL


def test_repeat_is_deterministic_fp64(ctx, tmp_path):
    offs, posn, types, cell = cases.batch(cases.small_binary(n_struc=3, seed=5))
    cases.config_potential(ctx, 2, tmp_path)
    a = ctx.compute(offs, posn, types, cell, precision=FP64)
    b = ctx.compute(offs, posn, types, cell, precision=FP64)
    assert np.allclose(a[0], b[0], rtol=1e-13, atol=0) and np.allclose(a[1], b[1], rtol=0, atol=1e-12)


def test_untranslated_newton_rule_matches_oracle(gpu_lib, oracle, tmp_path):
    """The reference's verlet::List rule (Newton-3rd only for n == 0, nnp.cpp:550) on request."""
    c = Context(newton=1)
    try:
        offs, posn, types, cell = cases.batch(cases.tiny_cells()[1:2] + cases.small_binary(n_struc=1))
        text = cases.config_potential(c, 2, tmp_path)
        pot = oracle.load_text(text)
        E, F, _ = c.compute(offs, posn, types, cell, precision=FP64)
        Eo, Fo, _, _, _ = pot.compute(offs, posn, types, cell, newton=0)
        assert _rel_err(F, Fo) < REL
    finally:
        c.close()


def test_capacity_growth(gpu_lib, oracle, tmp_path):
    """Start with a neighbour capacity far too small: the library grows it and recomputes."""
    c = Context(max_neighbors=8)
    try:
        offs, posn, types, cell = cases.batch(cases.small_binary(n_struc=2))
        text = cases.config_potential(c, 2, tmp_path)
        pot = oracle.load_text(text)
        E, F, _ = c.compute(offs, posn, types, cell, precision=FP64)
        Eo, Fo, _, _, _ = pot.compute(offs, posn, types, cell)
        assert _rel_err(E, Eo) < REL and _rel_err(F, Fo) < REL
    finally:
        c.close()


def test_learned_capacity_shrinks_and_regrows(gpu_lib, oracle, tmp_path):
    """The row capacity follows the longest rows seen (1.25 x): after a batch at the bench density it
    shrinks for the next call, and a batch twice as dense overflows it, regrows it and is computed
    again; every result matches the oracle."""
    c = Context()
    try:
        text = cases.config_potential(c, 2, tmp_path)
        pot = oracle.load_text(text)
        structs = cases.small_binary(n_struc=3, seed=21)
        dense = [(x * 0.8, t, np.asarray(R) * 0.8) for x, t, R in structs]
        for batch in (structs, structs, dense, structs, dense):
            offs, posn, types, cell = cases.batch(batch)
            E, F, W = c.compute(offs, posn, types, cell, precision=FP64)
            Eo, Fo, Wo, _, _ = pot.compute(offs, posn, types, cell)
            assert _rel_err(E, Eo) < REL and _rel_err(F, Fo) < REL and _rel_err(W, Wo) < REL
            Em, Fm, _ = c.compute(offs, posn, types, cell, precision=MIXED)
            assert np.abs(Fm - Fo).max() <= 1e-3 * np.abs(Fo).max()
    finally:
        c.close()


def test_errors_are_reported(ctx, tmp_path):
    from ann_gb300 import AnnError
    cases.config_potential(ctx, 2, tmp_path)
    offs, posn, types, cell = cases.batch(cases.small_binary(n_struc=1))
    bad = types.copy()
    bad[0] = 7
    with pytest.raises(AnnError):
        ctx.compute(offs, posn, bad, cell)
    nanx = posn.copy()
    nanx[0, 0] = np.nan
    with pytest.raises(AnnError):
        ctx.compute(offs, nanx, types, cell)
    with pytest.raises(AnnError):
        ctx.load_text("ann\nntypes 0\n")
    # the context stays usable
    ctx.compute(offs, posn, types, cell)


@pytest.mark.parametrize("neuron", cases.NEURONS)
def test_every_activation(ctx, oracle, neuron):
    """Hidden layers with each activation of nn.cpp:149-810: FP64 as the oracle, mixed (tensor-core
    networks where they apply) within the mixed bars."""
    text = cases.activation_potential_text(neuron)
    ctx.load_text(text)
    pot = oracle.load_text(text)
    offs, posn, types, cell = cases.batch(cases.small_binary(n_struc=2, seed=6))
    E, F, Wv = ctx.compute(offs, posn, types, cell, precision=FP64)
    Eo, Fo, Wo, _, _ = pot.compute(offs, posn, types, cell)
    assert _rel_err(E, Eo) < REL and _rel_err(F, Fo) < REL and _rel_err(Wv, Wo) < REL
    _check_mixed(ctx, offs, posn, types, cell, E, F)


def test_pinned_host_buffers(ctx, tmp_path):
    """ann_host_alloc buffers as inputs and outputs of ann_compute give the pageable-array results
    (FP64: bit-identical; the buffers outlive nothing and are freed with their arrays)."""
    structs = cases.small_binary(n_struc=4, seed=27)
    offs, posn, types, cell = cases.batch(structs)
    cases.config_potential(ctx, 2, tmp_path)
    E0, F0, W0 = ctx.compute(offs, posn, types, cell, precision=FP64)
    h = [ctx.pinned(offs.shape, np.int64), ctx.pinned(posn.shape), ctx.pinned(types.shape, np.int32), ctx.pinned(cell.shape)]
    for dst, src in zip(h, (offs, posn, types, cell)):
        dst[:] = src
    out = (ctx.pinned(E0.shape), ctx.pinned(F0.shape), ctx.pinned(W0.shape))
    E1, F1, W1 = ctx.compute(*h, precision=FP64, out=out)
    assert E1 is out[0] and np.array_equal(E1, E0) and np.allclose(F1, F0, rtol=0, atol=1e-12 * np.abs(F0).max())
    assert np.array_equal(W1, W0)
    assert ctx.pinned((0,)).size == 0
