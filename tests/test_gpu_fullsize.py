"""Parity at the benchmark sizes, against the oracle, through the C ABI.

- The E+F workload in full (256 binary structures, N ~ U{32..512}, 74,710 atoms, 72 inputs,
  72-64-64-1 softplus): the FP64 GPU form matches the oracle with neighbour lists bit-exact
  (every (i, j, image) and every pair vector) and energies, forces and virials within 1e-10
  relative; the mixed form (FP32 basis and forces, BF16 tensor-core networks with FP32
  accumulation, FP64 energy sums) stays within 1 meV/atom and 10 meV/A of the oracle.
- The training batch in full (64 binary structures, N ~ U{32..256}, Lennard-Jones labels,
  L = mean (dE/N)^2/2 + 0.1 mean |dF|^2/6): the FP64 gradient of all 17,794 parameters equals the
  oracle's within 1e-9 of its scale and central finite differences of the GPU's own loss on 64
  random parameters; the mixed gradient stays within 1e-3 of the scale.
- Every parameter of the 16-20-20-1 argon network on the 108-atom FCC box (the small FP64
  configuration) against central finite differences of the GPU's loss.
The oracle runs on all host cores (structures block-distributed over threads).
"""
import os

import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, Context
from ann_gb300 import workloads as W
from ann_gb300.api import pack_batch

pytestmark = pytest.mark.gpu

NTH = os.cpu_count() or 1
REL = 1e-10


def _rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = Context(use_graphs=True)
    yield c
    c.close()


def _sorted_pairs(i, j, img, r):
    key = np.lexsort((img[:, 2], img[:, 1], img[:, 0], j, i))
    return i[key], j[key], img[key], r[key]


def test_energy_force_workload_in_full(ctx, oracle, tmp_path):
    structs = W.config2()
    offs, posn, types, cell = pack_batch(structs)
    assert len(structs) == 256 and int(offs[-1]) == 74710
    text = cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    pot = oracle.load_text(text)
    Eo, Fo, Wo, _, _ = pot.compute(offs, posn, types, cell, nthreads=NTH)

    E, F, Wv = ctx.compute(offs, posn, types, cell, precision=FP64)
    assert _rel_err(E, Eo) < REL, ("energy", _rel_err(E, Eo))
    assert _rel_err(F, Fo) < REL, ("forces", _rel_err(F, Fo))
    assert _rel_err(Wv, Wo) < REL, ("virial", _rel_err(Wv, Wo))

    # neighbour lists: the GPU's FP64 rows against the oracle's brute-force periodic search
    i, j, img, r = ctx.neighbors(with_vectors=True)
    parts = []
    for s in range(len(structs)):
        a0, a1 = offs[s], offs[s + 1]
        io, jo, imgo, ro, _ = oracle.neighbors(posn[a0:a1], cell[s].reshape(3, 3).T, ctx.rc)
        parts.append((io + a0, jo + a0, imgo, ro))
    ref = tuple(np.concatenate([p[k] for p in parts]) for k in range(4))
    a, b = _sorted_pairs(i, j, img, r), _sorted_pairs(*ref)
    assert len(a[0]) == len(b[0]) > 4_000_000, "neighbour count"
    for x, y in zip(a, b):
        assert np.array_equal(x, y), "neighbour list differs"

    Em, Fm, Wm = ctx.compute(offs, posn, types, cell, precision=MIXED)
    nat = np.diff(offs)
    e_mev = np.max(np.abs(Em - Eo) / nat) * 1e3
    f_mev = np.max(np.abs(Fm - Fo)) * 1e3
    assert e_mev < 1.0, f"mixed energy error {e_mev} meV/atom"
    assert f_mev < 10.0, f"mixed force error {f_mev} meV/A"
    print(f"full E+F workload: FP64 rel E {_rel_err(E, Eo):.1e} F {_rel_err(F, Fo):.1e} W {_rel_err(Wv, Wo):.1e}; "
          f"mixed {e_mev:.4f} meV/atom {f_mev:.4f} meV/A max")


def test_training_batch_in_full(ctx, oracle, tmp_path):
    structs = W.config3()
    offs, posn, types, cell = pack_batch(structs)
    assert len(structs) == 64
    Eref, Fref = W.lennard_jones(structs)
    Fref = np.concatenate(Fref)
    text = cases.config_potential(ctx, 3, tmp_path, precondition_batch=(offs, posn, types, cell))
    pot = oracle.load_text(text)
    lo, go = pot.train(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, nthreads=NTH)

    loss = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
    g = ctx.train_backward()
    assert len(g) == 17794
    assert np.allclose(loss, lo, rtol=1e-10, atol=1e-14)
    scale = np.abs(go).max()
    assert np.abs(g - go).max() <= 1e-9 * scale

    p0 = ctx.get_params()
    rng = np.random.default_rng(64)
    try:
        for k in rng.choice(len(p0), 64, replace=False):
            h = 1e-5 * max(1.0, abs(p0[k]))
            pp = p0.copy(); pp[k] += h
            ctx.set_params(pp)
            lp = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)[0]
            pp[k] -= 2 * h
            ctx.set_params(pp)
            lm = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)[0]
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[k]) <= 1e-6 * abs(g[k]) + 1e-7 * scale, (k, fd, g[k])
    finally:
        ctx.set_params(p0)

    ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=MIXED)
    gm = ctx.train_backward()
    err = np.abs(gm - go).max() / scale
    assert err <= 1e-3, err
    print(f"full training batch: FP64 gradient rel {np.abs(g - go).max() / scale:.1e}; mixed {err:.1e} of the scale")


def test_every_parameter_small_configuration(ctx, tmp_path):
    structs = W.config1()
    offs, posn, types, cell = pack_batch(structs)
    Eref, Fref = W.lennard_jones(structs)
    Fref = np.concatenate(Fref)
    cases.config_potential(ctx, 1, tmp_path)
    ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
    g = ctx.train_backward()
    p0 = ctx.get_params()
    assert len(p0) == 16 * 20 + 20 * 20 + 20 + 20 + 20 + 1
    scale = np.abs(g).max()
    try:
        for k in range(len(p0)):
            h = 1e-5 * max(1.0, abs(p0[k]))
            pp = p0.copy(); pp[k] += h
            ctx.set_params(pp)
            lp = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)[0]
            pp[k] -= 2 * h
            ctx.set_params(pp)
            lm = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)[0]
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[k]) <= 1e-6 * abs(g[k]) + 1e-7 * scale, (k, fd, g[k])
    finally:
        ctx.set_params(p0)


def test_precision_study_box_in_full(ctx, oracle, tmp_path):
    """The 32,000-atom ternary box (96 inputs, 96-128-128-1 tanh): FP64 GPU form within 1e-10 of the
    oracle with a bit-exact neighbour list; the mixed form, its networks on the tensor cores, within
    1 meV/atom and 10 meV/A of the oracle."""
    structs = W.config4()
    offs, posn, types, cell = pack_batch(structs)
    assert int(offs[-1]) == 32000
    text = cases.config_potential(ctx, 4, tmp_path, precondition_batch=(offs, posn, types, cell))
    pot = oracle.load_text(text)
    Eo, Fo, Wo, _, _ = pot.compute(offs, posn, types, cell, nthreads=NTH)
    E, F, Wv = ctx.compute(offs, posn, types, cell, precision=FP64)
    assert _rel_err(E, Eo) < REL and _rel_err(F, Fo) < REL and _rel_err(Wv, Wo) < REL
    i, j, img, r = ctx.neighbors(with_vectors=True)
    io, jo, imgo, ro, _ = oracle.neighbors(posn, cell[0].reshape(3, 3).T, ctx.rc)
    a, b = _sorted_pairs(i, j, img, r), _sorted_pairs(io, jo, imgo, ro)
    assert len(a[0]) == len(b[0]) > 1_500_000
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert [ctx.network_form(t) for t in range(3)] == [(2, 3)] * 3, "networks not on the tensor cores (split 3)"
    Em, Fm, _ = ctx.compute(offs, posn, types, cell, precision=MIXED)
    e_mev = abs(Em[0] - Eo[0]) / 32000 * 1e3
    f_mev = np.max(np.abs(Fm - Fo)) * 1e3
    assert e_mev < 1.0 and f_mev < 10.0, (e_mev, f_mev)
    print(f"32,000-atom box: FP64 rel E {_rel_err(E, Eo):.1e} F {_rel_err(F, Fo):.1e}; mixed {e_mev:.4f} meV/atom {f_mev:.4f} meV/A")
