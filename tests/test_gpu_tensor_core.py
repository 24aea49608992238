"""The tcgen05 network kernel (MIXED precision, mlp_backend auto / 2) against the SIMT kernels
and the FP64 pipeline, through the C ABI.

Bars: atom energies and dE/dG of the tensor-core pass within 1e-4 eV / 1e-4 relative of the FP64
pass (BF16 hi+lo operands, FP32 accumulation); structure energies and forces within the mixed
bars of 1 meV/atom and 10 meV/A.
"""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, AnnError, Context

pytestmark = pytest.mark.gpu

E_MEV_ATOM = 1.0
F_MEV_A = 10.0


@pytest.fixture(scope="module")
def contexts(gpu_lib):
    tc = Context(mlp_backend=2)
    simt = Context(mlp_backend=1)
    yield tc, simt
    tc.close()
    simt.close()


def _mixed_bars(E, F, E64, F64, offs):
    nat = np.maximum(np.diff(offs), 1)
    e_err = np.max(np.abs(E - E64) / nat) * 1e3
    f_err = np.max(np.abs(F - F64)) * 1e3 if len(F) else 0.0
    assert e_err < E_MEV_ATOM, f"energy error {e_err} meV/atom"
    assert f_err < F_MEV_A, f"force error {f_err} meV/A"


def _compare(tc, simt, text, structs):
    offs, posn, types, cell = cases.batch(structs)
    tc.load_text(text)
    simt.load_text(text)
    E64, F64, W64 = tc.compute(offs, posn, types, cell, precision=FP64)
    e64 = tc.atom_energies()
    d64 = tc.dedg()
    E, F, Wv = tc.compute(offs, posn, types, cell, precision=MIXED)
    e = tc.atom_energies()
    d = tc.dedg()
    assert np.max(np.abs(e - e64)) < 1e-4, "atom energies"
    assert np.max(np.abs(d - d64)) < 1e-4 * max(np.max(np.abs(d64)), 1.0), "dE/dG"
    _mixed_bars(E, F, E64, F64, offs)
    Es, Fs, _ = simt.compute(offs, posn, types, cell, precision=MIXED)
    _mixed_bars(E, F, Es, Fs, offs)
    return e, e64


def test_binary_batch_matches_fp64(contexts, tmp_path):
    tc, simt = contexts
    structs = cases.small_binary(n_struc=6, seed=13)
    offs, posn, types, cell = cases.batch(structs)
    text = cases.config_potential(tc, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    _compare(tc, simt, text, structs)


def test_many_tiles_per_block(contexts, tmp_path):
    """More 128-atom tiles of one type than blocks in the grid: the persistent loop is exercised."""
    tc, simt = contexts
    structs = cases.W.config2(nstruc=160)
    offs, posn, types, cell = cases.batch(structs)
    assert np.sum(types == 0) > 152 * 128
    text = cases.config_potential(tc, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    _compare(tc, simt, text, structs)


def test_ragged_and_missing_types(contexts, tmp_path):
    """Type counts that are not multiples of 128 and a type with no atoms at all."""
    tc, simt = contexts
    text = cases.config_potential(tc, 2, tmp_path)
    one_type = [(x, np.zeros_like(t), R) for (x, t, R) in cases.small_binary(n_struc=2, seed=3)]
    _compare(tc, simt, text, one_type)
    _compare(tc, simt, text, cases.tiny_cells())


def test_activation_variants(contexts, tmp_path):
    """Sigmoid / tanh / softplus networks with odd widths (padding to 16 columns)."""
    tc, simt = contexts
    text = cases.generic_potential_text()
    structs = cases.small_binary(n_struc=3, seed=21) + cases.tiny_cells()
    _compare(tc, simt, text, structs)


def test_config1_argon(contexts, tmp_path):
    tc, simt = contexts
    text = cases.config_potential(tc, 1, tmp_path)
    _compare(tc, simt, text, cases.W.config1())


def test_wide_networks_run_on_tensor_cores(contexts, tmp_path):
    """The 96-128-128-1 tanh networks of the ternary precision study run on the tensor cores with
    both operands split (one image of W per layer serves the forward GEMM as a K-major operand and
    the backward GEMM as the MN-major W^T): within 1e-4 of FP64 per atom and the mixed bars."""
    tc, simt = contexts
    structs = cases.ternary_box(dims=(8, 8, 6))
    offs, posn, types, cell = cases.batch(structs)
    text = cases.config_potential(tc, 4, tmp_path, precondition_batch=(offs, posn, types, cell))
    assert [tc.network_form(t) for t in range(3)] == [(2, 3)] * 3
    _compare(tc, simt, text, structs)


@pytest.mark.parametrize("split", [1, 2, 3])
def test_operand_split_forms(gpu_lib, tmp_path, split):
    """Each operand form (1: BF16 x BF16, 2: activations hi + lo, 3: both split) on the binary
    networks: structure energies and forces within the mixed bars of FP64, and atom energies /
    dE/dG within what the form's rounding allows (2^-8 relative per BF16 operand)."""
    tc = Context(mlp_backend=2, tc_split=split)
    try:
        structs = cases.small_binary(n_struc=6, seed=13)
        offs, posn, types, cell = cases.batch(structs)
        cases.config_potential(tc, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
        assert [tc.network_form(t) for t in range(2)] == [(2, split)] * 2
        E64, F64, _ = tc.compute(offs, posn, types, cell, precision=FP64)
        e64, d64 = tc.atom_energies(), tc.dedg()
        E, F, _ = tc.compute(offs, posn, types, cell, precision=MIXED)
        e, d = tc.atom_energies(), tc.dedg()
        _mixed_bars(E, F, E64, F64, offs)
        tol = {1: 2e-2, 2: 1e-2, 3: 1e-4}[split]
        assert np.max(np.abs(d - d64)) < tol * max(np.max(np.abs(d64)), 1.0), "dE/dG"
        assert np.max(np.abs(e - e64)) < tol, "atom energies"
    finally:
        tc.close()


def test_tc_split_validated(gpu_lib):
    with pytest.raises(AnnError):
        Context(tc_split=4)


@pytest.mark.parametrize("groups", [1, 2, 4])
def test_forced_warp_split(contexts, tmp_path, groups):
    """Each width of the kernel (1, 2 or 4 warps per TMEM lane quadrant, 4, 2 or 1 CTAs per SM)
    against FP64: a batch with many tiles per CTA, a ragged one-type batch and odd layer widths."""
    _, simt = contexts
    tc = Context(mlp_backend=2, tc_groups=groups)
    try:
        structs = cases.W.config2(nstruc=160)
        offs, posn, types, cell = cases.batch(structs)
        text = cases.config_potential(tc, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
        _compare(tc, simt, text, structs)
        one_type = [(x, np.zeros_like(t), R) for (x, t, R) in cases.small_binary(n_struc=2, seed=3)]
        _compare(tc, simt, text, one_type)
        _compare(tc, simt, cases.generic_potential_text(), cases.small_binary(n_struc=3, seed=21) + cases.tiny_cells())
    finally:
        tc.close()


def test_tc_groups_validated(gpu_lib):
    with pytest.raises(AnnError):
        Context(tc_groups=3)


@pytest.mark.parametrize("nstruc", [3, 24])
def test_training_gradient_on_tensor_cores(gpu_lib, tmp_path, nstruc):
    """The training pass (energy + force loss, forward-over-reverse through the networks, weight
    gradient over the atoms) on the tensor cores, tiles of 128 atoms, against the SIMT kernel on the
    same batch (both mixed precision: within 1e-4 of the gradient's scale) and against the FP64 form
    (1e-3 of the scale); a second backward call on the same forward state gives the same gradient bit
    for bit (per-tile sums added in tile order; the forward's force sums use FP32 atomics, so a new
    forward call may move the last bits)."""
    from ann_gb300 import workloads as W
    from ann_gb300.api import pack_batch
    structs = W.random_binary(nstruc, 32, 256, seed=77)
    offs, posn, types, cell = pack_batch(structs)
    Eref, Fref = W.lennard_jones(structs)
    Fref = np.concatenate(Fref)
    tc = Context(mlp_backend=2)
    simt = Context(mlp_backend=1)
    try:
        text = cases.config_potential(tc, 3, tmp_path, precondition_batch=(offs, posn, types, cell))
        simt.load_text(text)
        tc.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
        g64 = tc.train_backward()
        tc.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=MIXED)
        g_tc = tc.train_backward()
        assert np.array_equal(tc.train_backward(), g_tc)   # the same forward state: bit for bit
        simt.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=MIXED)
        g_simt = simt.train_backward()
        scale = np.abs(g64).max()
        assert np.abs(g_tc - g_simt).max() <= 1e-4 * scale, np.abs(g_tc - g_simt).max() / scale
        assert np.abs(g_tc - g64).max() <= 1e-3 * scale, np.abs(g_tc - g64).max() / scale
    finally:
        tc.close()
        simt.close()
