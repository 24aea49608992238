"""The GPU path against the reference's own potential code directly, through the C ABI: the
structures of tests/golden/ref_nnp.npz (the outputs of the reference's nnp.cpp NNP::symm /
NNP::energy / NNP::force, compiled from its sources) in one batch per potential. The FP64 form
matches the reference's symmetry functions within 1e-12 and its energies and forces within 1e-10
(relative to the largest magnitude, at least 1); the mixed form stays within 1 meV/atom and
10 meV/A of them."""
from pathlib import Path

import numpy as np
import pytest

from ann_gb300 import FP64, MIXED, Context
from ann_gb300.api import pack_batch

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "ref_nnp.npz"


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = Context(use_graphs=True)
    yield c
    c.close()


def _batches():
    gold = np.load(GOLD)
    names = [str(n) for n in gold["pot_names"]]
    for pi, name in enumerate(names):
        ks = [k for k in range(int(gold["ncases"])) if int(gold[f"c{k}_pot"]) == pi]
        structs = [(gold[f"c{k}_posn"], gold[f"c{k}_types"], gold[f"c{k}_R"]) for k in ks]
        ref = [(gold[f"c{k}_symm"], float(gold[f"c{k}_energy"]), gold[f"c{k}_force"]) for k in ks]
        yield name, str(gold[f"pot_{name}"]), structs, ref


def test_fp64_and_mixed_against_reference_outputs(ctx):
    for name, text, structs, ref in _batches():
        ctx.load_text(text)
        offs, posn, types, cell = pack_batch(structs)
        E, F, _ = ctx.compute(offs, posn, types, cell, precision=FP64)
        G = ctx.symm()
        Em, Fm, _ = ctx.compute(offs, posn, types, cell, precision=MIXED)
        for s, (Gr, Er, Fr) in enumerate(ref):
            a0, a1 = int(offs[s]), int(offs[s + 1])
            label = f"{name} structure {s} ({a1 - a0} atoms)"
            gs = max(1.0, float(np.abs(Gr).max()))
            assert np.abs(G[a0:a1, :Gr.shape[1]] - Gr).max() <= 1e-12 * gs, f"{label}: symmetry functions"
            assert abs(E[s] - Er) <= 1e-10 * max(1.0, abs(Er)), f"{label}: energy {E[s]} vs {Er}"
            fs = max(1.0, float(np.abs(Fr).max()))
            assert np.abs(F[a0:a1] - Fr).max() <= 1e-10 * fs, f"{label}: forces"
            assert abs(Em[s] - Er) / (a1 - a0) * 1e3 < 1.0, f"{label}: mixed energy"
            assert np.abs(Fm[a0:a1] - Fr).max() * 1e3 < 10.0, f"{label}: mixed forces"
