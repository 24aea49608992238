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


# ---------------------------------------------------------------- the networks (ml/nn.cpp)
NN_GOLD = Path(__file__).resolve().parent / "golden" / "ref_nn.npz"
# activations whose second derivative in the reference's AFFPBP2 forms is the exact one; for the
# others (ARCTAN, TANHRE, SQRE, GELU, MISH, SERF, LOGISH, ATISH, TEST) the reference's d2 is zero or
# inexact, so its D2ODZDI is not pinned there (the oracle's d2 is checked against finite differences)
EXACT_D2 = {"LINEAR", "SIGMOID", "TANH", "ISRU", "RELU", "ELU", "SWISH", "PFLU", "SOFTPLUS", "SQPLUS"}


@pytest.fixture(scope="module")
def nn_gold():
    return np.load(NN_GOLD)


def _close(a, b, tol=1e-13):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) <= tol * max(np.max(np.abs(b)), 1e-300)


def _oracle_network(oracle, neuron, c, params, scal, nin, nodes):
    import cases
    inpw, inpb, outw, outb = scal[:nin], scal[nin:2 * nin], scal[2 * nin], scal[2 * nin + 1]
    pot = oracle.load_text(cases.single_network_text(nin, nodes, cases.NEURONS[neuron - 1], c, inpw, inpb, outw, outb))
    pot.set_params(params)
    return pot


def _d2_expected(ref_d2u, g, inpw, u, nin, nodes):
    """The reference's d2O/(dp dI) . u with its layer-0 weight term made exact. D2ODZDI
    (nn.cpp:2053-2059) adds dO/dz0_n to d2O/(dW0(n,m) dI_m) without the input scaling inpw_m that
    dz0/dI carries (DZDI, nn.cpp:1946); the exact term is dO/dz0_n * inpw_m, and dO/dz0_n =
    dO/db0_n = g[n] (biases first in the packing)."""
    nbias = int(sum(nodes))
    exp = np.array(ref_d2u, copy=True)
    for m in range(nin):
        for n in range(nodes[0]):
            exp[nbias + m * nodes[0] + n] += g[n] * (inpw[m] - 1.0) * u[m]
    return exp


def test_network_initialisation_bit_exact(nn_gold):
    """ANN::resize (nn.cpp:1019-1190, XAVIER, NORMAL) as the reference's own code draws it."""
    import hashlib
    from ann_gb300 import workloads as W
    for k in range(3):
        nin, seed, *nodes = (int(v) for v in nn_gold[f"init{k}_shape"])
        p = W.xavier_network(seed, nin, nodes)
        assert np.array_equal(p[:64], nn_gold[f"init{k}_head"]), k
        digest = np.frombuffer(hashlib.sha256(p.astype("<f8").tobytes()).digest(), np.uint8)
        assert np.array_equal(digest, nn_gold[f"init{k}_sha256"]), k


def test_network_pass_and_gradients_against_reference(oracle, nn_gold):
    """ANN::fpbp2 output, DODZ's dO/dI and Cost::grad's dO/dp for every activation, with unit and
    with general input / output scaling: equal to the reference's own code up to the order of the
    sums (1e-13 of each quantity's scale); D2ODZDI's d2O/(dp dI) likewise where its second
    derivative is exact, with the reference's missing input scaling in the layer-0 weight term."""
    import cases
    nin, *nodes = (int(v) for v in nn_gold["nn_shape"])
    checked_d2 = 0
    for k, (neuron, c, scaled) in enumerate(nn_gold["nn_cases"]):
        neuron, scaled = int(neuron), int(scaled)
        pot = _oracle_network(oracle, neuron, c, nn_gold["nn_params"][k], nn_gold["nn_scaling"][k], nin, nodes)
        o, dodi, g, d2 = pot.nn_eval(0, nn_gold["nn_x"][k])
        name = cases.NEURONS[neuron - 1]
        assert _close([o], [nn_gold["nn_out"][k]]), (name, scaled, "output")
        assert _close(dodi, nn_gold["nn_dodi"][k]), (name, scaled, "dO/dI")
        assert _close(g, nn_gold["nn_grad"][k]), (name, scaled, "dO/dp")
        if name in EXACT_D2:
            u = nn_gold["nn_u"][k]
            inpw = nn_gold["nn_scaling"][k][:nin]
            assert _close(d2 @ u, _d2_expected(nn_gold["nn_d2u"][k], g, inpw, u, nin, nodes), 1e-12), (name, scaled, "d2O/dpdI")
            checked_d2 += 1
    assert checked_d2 == 2 * len(EXACT_D2)


def test_full_second_derivative_matrices(oracle, nn_gold):
    import cases
    nin, *nodes = (int(v) for v in nn_gold["nn_shape"])
    for name, scaled in (("TANH", 0), ("SOFTPLUS", 1)):
        k = next(i for i, (n, _, s) in enumerate(nn_gold["nn_cases"]) if cases.NEURONS[int(n) - 1] == name and int(s) == scaled)
        neuron, c, _ = nn_gold["nn_cases"][k]
        pot = _oracle_network(oracle, int(neuron), c, nn_gold["nn_params"][k], nn_gold["nn_scaling"][k], nin, nodes)
        o, dodi, g, d2 = pot.nn_eval(0, nn_gold["nn_x"][k])
        ref = np.array(nn_gold[f"d2full_{name}_{scaled}"])
        inpw = nn_gold["nn_scaling"][k][:nin]
        nbias = int(sum(nodes))
        for m in range(nin):
            for n in range(nodes[0]):
                ref[nbias + m * nodes[0] + n, m] += g[n] * (inpw[m] - 1.0)
        assert _close(d2, ref, 1e-12), name


@needs_ref
def test_networks_against_fresh_reference_build(oracle):
    """New random networks (first-layer width different from the input count, general scaling)
    through the reference's own code, full d2O/(dp dI) matrices."""
    import ctypes as C
    import cases
    from oracle_lib import RefNN, nn_eval
    ref = RefNN()
    rng = np.random.default_rng(2026)
    _D = C.POINTER(C.c_double)
    for name in sorted(EXACT_D2):
        neuron = cases.NEURONS.index(name) + 1
        nin, nodes = 11, [int(rng.integers(5, 14)), int(rng.integers(3, 9)), 1]
        c = float(rng.uniform(0.7, 1.6))
        h = ref.create(nin, nodes, neuron, c=c, init=4, seed=int(rng.integers(1, 10 ** 6)), dist=3)
        try:
            p = ref.params(h)
            inpw, inpb = rng.uniform(0.3, 1.5, nin), rng.uniform(-0.5, 0.5, nin)
            outw, outb = float(rng.uniform(0.5, 1.5)), float(rng.normal())
            ref.L.ref_nn_set_scaling(h, inpw.ctypes.data_as(_D), inpb.ctypes.data_as(_D), outw, outb)
            pot = _oracle_network(oracle, neuron, c, p, np.concatenate([inpw, inpb, [outw, outb]]), nin, nodes)
            for _ in range(3):
                x = rng.normal(0.0, 1.0, nin)
                a = nn_eval(ref.L, "ref_nn_eval", h, nin, len(p), x)
                b = pot.nn_eval(0, x)
                assert _close([b[0]], [a[0]]) and _close(b[1], a[1]) and _close(b[2], a[2]), name
                d2ref = np.array(a[3])
                nbias = int(sum(nodes))
                for m in range(nin):
                    for n in range(nodes[0]):
                        d2ref[nbias + m * nodes[0] + n, m] += b[2][n] * (inpw[m] - 1.0)
                assert _close(b[3], d2ref, 1e-12), name
        finally:
            ref.L.ref_nn_free(h)
