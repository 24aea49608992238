"""Pin the CPU oracle to the reference's own code.

1. against the committed golden vectors (tests/golden/ref_basis.npz, produced by the
   reference's cutoff / basis / special-function sources compiled unmodified): bit-exact;
2. where the reference sources are present, against a fresh build of them at new random points
   and against the reference's own file readers (BasisR::read / BasisA::read).
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle_lib import REF_SRC, RefBasis, eval_basisA, eval_basisR

GOLD = Path(__file__).resolve().parent / "golden" / "ref_basis.npz"


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_special_functions_bit_exact(oracle, gold):
    L = oracle.L
    assert np.array_equal(np.array([L.orc_fmexp(float(v)) for v in gold["fmexp_x"]]), gold["fmexp_y"])
    assert np.array_equal(np.array([L.orc_coscut(float(v)) for v in gold["cut_x"]]), gold["coscut_y"])
    assert np.array_equal(np.array([L.orc_sincut(float(v)) for v in gold["cut_x"]]), gold["sincut_y"])


def test_cutoffs_bit_exact(oracle, gold):
    for name, rc, dr, f, g in gold["cutoff"]:
        fo, go = C.c_double(), C.c_double()
        assert oracle.L.orc_cutoff(int(name), rc, dr, C.byref(fo), C.byref(go)) == 0
        assert fo.value == f and go.value == g, (name, dr)


def test_radial_basis_bit_exact(oracle, gold):
    for inp, out in zip(gold["radial_in"], gold["radial_out"]):
        name, cut, rc, dr = int(inp[0]), int(inp[1]), inp[2], inp[3]
        rs, eta, dE = inp[4:8], inp[8:12], inp[12:16]
        s, amp, sd = eval_basisR(oracle.L, "orc_", cut, rc, name, rs, eta, dr, dE)
        assert np.array_equal(np.concatenate([s, [amp], sd]), out), (name, cut)


def test_angular_basis_bit_exact(oracle, gold):
    for inp, out in zip(gold["angular_in"], gold["angular_out"]):
        name, cut, rc, dij, dik, cs = int(inp[0]), int(inp[1]), inp[2], inp[3], inp[4], inp[5]
        eta, zeta, lam, dE = inp[6:10], inp[10:14], inp[14:18].astype(np.int32), inp[18:22]
        s, phi, e2, sd = eval_basisA(oracle.L, "orc_", cut, rc, name, eta, zeta, lam, dij, dik, cs, dE)
        assert np.array_equal(np.concatenate([s, [phi], e2, sd]), out), (name, cut)


needs_ref = pytest.mark.skipif(not REF_SRC.exists(), reason="reference sources not present on this machine")


@needs_ref
def test_fresh_points_against_reference_build(oracle):
    ref = RefBasis()
    rng = np.random.default_rng(99)
    for _ in range(300):
        name, cut = int(rng.integers(1, 7)), int(rng.integers(1, 5))
        n = 6
        rs, eta = rng.uniform(0, 2, n), rng.uniform(0.2, 2, n)
        dr = float(rng.uniform(0.3, 6.5)); dE = rng.normal(size=n)
        a = eval_basisR(oracle.L, "orc_", cut, 6.5, name, rs, eta, dr, dE)
        b = eval_basisR(ref.L, "ref_", cut, 6.5, name, rs, eta, dr, dE)
        assert all(np.array_equal(np.atleast_1d(x), np.atleast_1d(y)) for x, y in zip(a, b))
        etaA = np.repeat(rng.uniform(1, 15, 3), 2)
        zeta = rng.choice([1.0, 2.0, 4.0, 8.0, 2.7], n)
        lam = rng.choice([-1, 1], n).astype(np.int32)
        dij, dik = (float(v) for v in rng.uniform(0.3, 6.5, 2))
        cs = float(rng.uniform(-1, 1))
        a = eval_basisA(oracle.L, "orc_", cut, 6.5, name, etaA, zeta, lam, dij, dik, cs, dE)
        b = eval_basisA(ref.L, "ref_", cut, 6.5, name, etaA, zeta, lam, dij, dik, cs, dE)
        assert all(np.array_equal(np.atleast_1d(x), np.atleast_1d(y)) for x, y in zip(a, b))


@needs_ref
def test_basis_file_readers_agree(oracle, tmp_path):
    """The reference's BasisR::read / BasisA::read and the oracle's reader see the same numbers."""
    ref = RefBasis()
    pR = tmp_path / "r.txt"
    pR.write_text("BasisR COS 6.500000 GAUSSIAN 3\n\t0.000000 0.100000\n\t0.500000 0.316228\n\t1.000000 1.000000\n")
    cut, name, n = C.c_int(), C.c_int(), C.c_int()
    rc = C.c_double()
    rs = np.zeros(8); eta = np.zeros(8)
    assert ref.L.ref_read_basisR(str(pR).encode(), C.byref(cut), C.byref(rc), C.byref(name), C.byref(n),
                                 rs.ctypes.data_as(C.POINTER(C.c_double)), eta.ctypes.data_as(C.POINTER(C.c_double)), 8) == 0
    assert (cut.value, rc.value, name.value, n.value) == (2, 6.5, 1, 3)
    assert np.array_equal(rs[:3], [0.0, 0.5, 1.0]) and np.array_equal(eta[:3], [0.1, 0.316228, 1.0])
    pA = tmp_path / "a.txt"
    pA.write_text("BasisA COS 6.000000 GAUSS 4\n\t10.000000 1.000000 1 0\n\t10.000000 2.000000 -1 0\n"
                  "\t5.000000 4.000000 1 0\n\t5.0000005 8.000000 -1 0\n")
    zeta = np.zeros(8); lam = np.zeros(8, np.int32); rfl = np.zeros(8, np.int32)
    assert ref.L.ref_read_basisA(str(pA).encode(), C.byref(cut), C.byref(rc), C.byref(name), C.byref(n),
                                 eta.ctypes.data_as(C.POINTER(C.c_double)), zeta.ctypes.data_as(C.POINTER(C.c_double)),
                                 lam.ctypes.data_as(C.POINTER(C.c_int)), rfl.ctypes.data_as(C.POINTER(C.c_int)), 8) == 0
    # eta groups: |5.0000005 - 5| < 1e-6 joins the previous group (basis_angular.cpp:190)
    assert list(rfl[:4]) == [0, 0, 1, 1]
    assert list(lam[:4]) == [1, -1, 1, -1]
