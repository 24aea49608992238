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


# ---- the assembly: the reference's own nnp.cpp / nnh.cpp (NNP::symm, energy, force, compute)

NNP_GOLD = Path(__file__).resolve().parent / "golden" / "ref_nnp.npz"


@pytest.fixture(scope="module")
def nnp_gold():
    return np.load(NNP_GOLD)


def _vacuum_energies(text):
    """Per-type vacuum energies of a potential text ('name X mass m energy e' lines, type order)."""
    return np.array([float(ln.split()[5]) for ln in text.splitlines() if ln.startswith("name ")])


def _nnp_cases(gold):
    names = [str(n) for n in gold["pot_names"]]
    for k in range(int(gold["ncases"])):
        name = names[int(gold[f"c{k}_pot"])]
        yield (k, name, str(gold[f"pot_{name}"]), gold[f"c{k}_posn"], gold[f"c{k}_types"], gold[f"c{k}_R"])


def _assembly_matches(pot, evac, x, t, R, G_ref, E_ref, F_ref, Fu_ref, Ec_ref, label):
    from ann_gb300.api import pack_batch
    offs, posn, types, cell = pack_batch([(x, t, R)])
    E, F, _, G, _ = pot.compute(offs, posn, types, cell, forces=True, symm=True, newton=1)
    assert np.array_equal(G[:, :G_ref.shape[1]], G_ref), f"{label}: symmetry functions differ"
    assert abs(E[0] - E_ref) <= 1e-13 * max(1.0, abs(E_ref)), f"{label}: energy {E[0]} vs {E_ref}"
    fs = max(1.0, float(np.abs(F_ref).max()))
    assert np.abs(F - F_ref).max() <= 1e-13 * fs, f"{label}: forces"
    _, Fu, _, _, _ = pot.compute(offs, posn, types, cell, forces=True, newton=0)
    assert np.abs(Fu - Fu_ref).max() <= 1e-13 * fs, f"{label}: forces with untranslated reactions"
    # NNP::compute's energy is the networks' sum alone; NNP::energy adds each atom's vacuum energy
    assert abs((E_ref - Ec_ref) - evac[t].sum()) <= 1e-12 * max(1.0, abs(E_ref)), label


def test_potential_assembly_against_reference(oracle, nnp_gold):
    """The oracle against the reference's own NNP::symm / energy / force / compute on 13
    structures of three potentials (tests/golden/ref_nnp.npz): the symmetry functions bit for bit
    (same neighbour entries in the same order, so the same sums), energies and forces within
    1e-13 (the force sums run in another order); forces with the Newton's-third-law reaction on
    every neighbour entry, and with the reaction on untranslated entries only (the verlet::List
    rule of nnp.cpp:550); NNP::compute's energy without the vacuum energies (nnp.cpp:617). The
    MD engine's PotNNPE::compute (torch/pot_nnpe.cpp:169-288), the call the library's ann_compute
    stands in for, gave NNP::energy's energy and NNP::force's forces bit for bit."""
    pots = {}
    for k, name, text, x, t, R in _nnp_cases(nnp_gold):
        if name not in pots:
            pots[name] = (oracle.load_text(text), _vacuum_energies(text))
        pot, evac = pots[name]
        E_ref = float(nnp_gold[f"c{k}_energy"])
        _assembly_matches(pot, evac, x, t, R, nnp_gold[f"c{k}_symm"], E_ref, nnp_gold[f"c{k}_force"],
                          nnp_gold[f"c{k}_force_untranslated"], float(nnp_gold[f"c{k}_energy_compute"]), f"case {k} ({name})")
        assert float(nnp_gold[f"c{k}_energy_potnnpe"]) == E_ref and float(nnp_gold[f"c{k}_force_potnnpe_vs_force"]) == 0.0


@needs_ref
def test_potential_assembly_against_fresh_reference_build(oracle, tmp_path):
    """New random structures of each golden potential through a fresh build of the reference's
    nnp.cpp (NNP::read of the same file) and of the MD engine's PotNNPE, with the oracle's
    neighbour entries."""
    import cases
    from oracle_lib import RefNNP
    ref = RefNNP()
    gold = np.load(NNP_GOLD)
    rng = np.random.default_rng(77)
    for name in [str(n) for n in gold["pot_names"]]:
        text = str(gold[f"pot_{name}"])
        p = tmp_path / f"{name}.ann"
        p.write_text(text)
        h = ref.read(p)
        hp = ref.potnnpe_read(p, ref.L.ref_nnp_rc(h))
        try:
            pot, evac = oracle.load_text(text), _vacuum_energies(text)
            nt = len(evac)
            assert ref.L.ref_nnp_nparams(h) == pot.nparams and ref.L.ref_nnp_ntypes(h) == nt
            rc = ref.L.ref_nnp_rc(h)
            structs = [(x, (t % nt).astype(np.int32), R) for x, t, R in cases.small_binary(n_struc=1, seed=int(rng.integers(1, 999)))]
            A = np.array([[5.0, 0.8, -0.6], [0.0, 4.6, 1.1], [0.0, 0.0, 5.3]])
            structs.append((rng.uniform(-0.5, 1.5, (9, 3)) @ A.T, rng.integers(0, nt, 9).astype(np.int32), A))
            for x, t, R in structs:
                i, j, img, _, _ = oracle.neighbors(x, R, rc)
                G, E, F, Ec, Fc = ref.structure(h, t, x, R, i, j, img, newton=1, form=0)
                _, _, Fu, _, _ = ref.structure(h, t, x, R, i, j, img, newton=0, form=1)
                assert np.array_equal(F, Fc)
                _assembly_matches(pot, evac, x, t, R, G, E, F, Fu, Ec, name)
                Ep, Fp = ref.potnnpe_compute(hp, t, x, R, i, j, img)
                assert abs(Ep - E) <= 1e-13 * max(1.0, abs(E)) and np.abs(Fp - F).max() <= 1e-13 * max(1.0, np.abs(F).max()), name
        finally:
            ref.L.ref_nnp_free(h)
            ref.L.ref_potnnpe_free(hp)
