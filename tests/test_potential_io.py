"""Potential files: the library's parser and writer (ann_gb300/csrc/potential.cpp, built for the
CPU from tests/potential_io.cpp) against the oracle's parser and, where the reference sources are
present, against the reference's own NNP::read / NNP::write (nnp.cpp:197-307): a file the library
writes is the file the reference writes for the same potential, byte for byte, and the reference
reads it back to the same symmetry functions, energies and forces."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle_lib import REF_SRC

ROOT = Path(__file__).resolve().parents[1]
GOLD = Path(__file__).resolve().parent / "golden" / "ref_nnp.npz"
needs_ref = pytest.mark.skipif(not REF_SRC.exists(), reason="reference sources not present on this machine")


@pytest.fixture(scope="module")
def pio(tmp_path_factory):
    so = tmp_path_factory.mktemp("pio") / "libpotential_io.so"
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I", str(ROOT / "ann_gb300" / "csrc"), "-o", str(so),
                    str(ROOT / "tests" / "potential_io.cpp"), str(ROOT / "ann_gb300" / "csrc" / "potential.cpp")], check=True)
    L = C.CDLL(str(so))
    L.pio_rewrite.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int]

    def rewrite(text: str) -> str:
        cap = 1 << 16
        while True:
            out, err = C.create_string_buffer(cap), C.create_string_buffer(1024)
            rc = L.pio_rewrite(text.encode(), out, cap, err, 1024)
            if rc == 0:
                return out.value.decode()
            if rc > 0:
                raise ValueError(err.value.decode())
            cap = -rc
    return rewrite


def _texts():
    import cases
    from ann_gb300 import workloads as W
    gold = np.load(GOLD)
    out = [(str(n), str(gold[f"pot_{n}"])) for n in gold["pot_names"]]
    out.append(("argon_example", cases.argon_example_potential()))
    out.append(("config1", W.config_potential_text(1)))
    out.append(("lj_argon", W.lj_argon_text()))
    return out


def test_library_writer_round_trip(oracle, pio):
    """The library's writer is stable (rewriting its own output changes nothing) and loses
    nothing: the oracle reads the same parameters, cutoff and inputs from it as from the original."""
    for name, text in _texts():
        once = pio(text)
        assert pio(once) == once, name
        a, b = oracle.load_text(text), oracle.load_text(once)
        assert a.ntypes == b.ntypes and a.nparams == b.nparams, name
        assert [a.ninput(t) for t in range(a.ntypes)] == [b.ninput(t) for t in range(b.ntypes)], name
        assert np.array_equal(a.get_params(), b.get_params()), name


@needs_ref
def test_library_writer_equals_reference_writer(pio, tmp_path):
    """NNP::read then NNP::write of each potential by the reference yields exactly the text the
    library writes for it."""
    from oracle_lib import RefNNP
    ref = RefNNP()
    for name, text in _texts():
        src, dst = tmp_path / f"{name}.ann", tmp_path / f"{name}.ref.ann"
        src.write_text(text)
        h = ref.read(src)
        try:
            ref.write(h, dst)
        finally:
            ref.L.ref_nnp_free(h)
        mine, theirs = pio(text), dst.read_text()
        if mine != theirs:
            for k, (x, y) in enumerate(zip(mine.splitlines(), theirs.splitlines())):
                assert x == y, f"{name}: line {k + 1}: library {x[:120]!r} vs reference {y[:120]!r}"
        assert mine == theirs, name


@needs_ref
def test_reference_computes_from_library_file(oracle, pio, tmp_path):
    """The reference (NNP::read, and the MD engine's PotNNPE::read) reads a file the library wrote
    and computes the golden structures' symmetry functions, energies and forces as the oracle does
    from the original text."""
    from oracle_lib import RefNNP
    from ann_gb300.api import pack_batch
    ref = RefNNP()
    gold = np.load(GOLD)
    names = [str(n) for n in gold["pot_names"]]
    for k in range(int(gold["ncases"])):
        name = names[int(gold[f"c{k}_pot"])]
        text = str(gold[f"pot_{name}"])
        p = tmp_path / f"{name}.lib.ann"
        p.write_text(pio(text))
        h = ref.read(p)
        hp = ref.potnnpe_read(p, ref.L.ref_nnp_rc(h))
        try:
            x, t, R = gold[f"c{k}_posn"], gold[f"c{k}_types"], gold[f"c{k}_R"]
            i, j, img, _, _ = oracle.neighbors(x, R, ref.L.ref_nnp_rc(h))
            G, E, F, _, _ = ref.structure(h, t, x, R, i, j, img)
            Ep, Fp = ref.potnnpe_compute(hp, t, x, R, i, j, img)
        finally:
            ref.L.ref_nnp_free(h)
            ref.L.ref_potnnpe_free(hp)
        offs, posn, types, cell = pack_batch([(x, t, R)])
        E0, F0, _, G0, _ = oracle.load_text(text).compute(offs, posn, types, cell, forces=True, symm=True)
        assert np.array_equal(G, G0[:, :G.shape[1]]), k
        assert abs(E - E0[0]) <= 1e-13 * max(1.0, abs(E0[0])), k
        assert np.abs(F - F0).max() <= 1e-13 * max(1.0, np.abs(F0).max()), k
        assert abs(Ep - E0[0]) <= 1e-13 * max(1.0, abs(E0[0])), k
        assert np.abs(Fp - F0).max() <= 1e-13 * max(1.0, np.abs(F0).max()), k
