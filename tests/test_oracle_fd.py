"""Identities the reference's own test programs check (print-only there, asserting here), applied
to the oracle: forces vs central finite differences of the energy (nnp/test_nnp_force.cpp:47-75),
basis / cutoff derivatives vs finite differences (test_basis_radial.cpp, test_basis_angular.cpp,
test_nnp_cutoff.cpp), the cutoff integral (test_nnp_cutoff.cpp:55), supercell invariance of the
symmetry functions (test_nnp_symm.cpp:292-500), the virial vs a strain derivative, and the
training gradient (energy and force terms) vs finite differences of the loss."""
import numpy as np
import pytest

import cases
from ann_gb300 import workloads as W
from ann_gb300.api import pack_batch
from oracle_lib import eval_basisA, eval_basisR


@pytest.fixture(scope="module")
def pot1(oracle):
    return oracle.load_text(W.config_potential_text(1))


@pytest.fixture(scope="module")
def pot2(oracle):
    return oracle.load_text(W.config_potential_text(2))


def test_cutoff_derivative_and_integral(oracle):
    import ctypes as C
    for name in (2, 3, 4):
        h = 1e-6
        for dr in np.linspace(0.3, 5.7, 25):
            f, g, fp, gp, fm, gm = (C.c_double() for _ in range(6))
            oracle.L.orc_cutoff(name, 6.0, dr, C.byref(f), C.byref(g))
            oracle.L.orc_cutoff(name, 6.0, dr + h, C.byref(fp), C.byref(gp))
            oracle.L.orc_cutoff(name, 6.0, dr - h, C.byref(fm), C.byref(gm))
            assert abs((fp.value - fm.value) / (2 * h) - g.value) < 1e-8
    # COS: integral_0^rc fc = rc/2
    xs = np.linspace(0, 6.0, 20001)
    vals = []
    for x in xs:
        f, g = C.c_double(), C.c_double()
        oracle.L.orc_cutoff(2, 6.0, x, C.byref(f), C.byref(g))
        vals.append(f.value)
    assert abs(np.trapezoid(vals, xs) - 3.0) < 1e-6


def test_basis_derivatives_fd(oracle):
    rng = np.random.default_rng(1)
    h = 1e-6
    for name in range(1, 7):
        rs, eta = rng.uniform(0, 2, 4), rng.uniform(0.2, 1.5, 4)
        for dr in rng.uniform(0.6, 5.5, 6):
            s, amp, sd = eval_basisR(oracle.L, "orc_", 2, 6.0, name, rs, eta, dr, np.ones(4))
            sp = eval_basisR(oracle.L, "orc_", 2, 6.0, name, rs, eta, dr + h, np.ones(4))[0]
            sm = eval_basisR(oracle.L, "orc_", 2, 6.0, name, rs, eta, dr - h, np.ones(4))[0]
            assert np.allclose((sp - sm) / (2 * h), sd, rtol=1e-5, atol=1e-8)
            assert abs(amp + sd.sum()) < 1e-10 * max(1.0, np.abs(sd).sum())
        eta = np.repeat(rng.uniform(2, 10, 2), 2)
        zeta = np.array([1.0, 2.0, 4.0, 3.5])
        lam = np.array([1, -1, 1, -1], np.int32)
        for _ in range(6):
            dij, dik = rng.uniform(0.6, 5.5, 2)
            cs = rng.uniform(-0.9, 0.9)
            s, phi, e2, sd = eval_basisA(oracle.L, "orc_", 2, 6.0, name, eta, zeta, lam, dij, dik, cs, np.ones(4))
            sd = sd.reshape(4, 3)
            num_c = (eval_basisA(oracle.L, "orc_", 2, 6.0, name, eta, zeta, lam, dij, dik, cs + h, np.ones(4))[0]
                     - eval_basisA(oracle.L, "orc_", 2, 6.0, name, eta, zeta, lam, dij, dik, cs - h, np.ones(4))[0]) / (2 * h)
            num_j = (eval_basisA(oracle.L, "orc_", 2, 6.0, name, eta, zeta, lam, dij + h, dik, cs, np.ones(4))[0]
                     - eval_basisA(oracle.L, "orc_", 2, 6.0, name, eta, zeta, lam, dij - h, dik, cs, np.ones(4))[0]) / (2 * h)
            num_k = (eval_basisA(oracle.L, "orc_", 2, 6.0, name, eta, zeta, lam, dij, dik + h, cs, np.ones(4))[0]
                     - eval_basisA(oracle.L, "orc_", 2, 6.0, name, eta, zeta, lam, dij, dik - h, cs, np.ones(4))[0]) / (2 * h)
            assert np.allclose(num_c, sd[:, 0], rtol=1e-5, atol=1e-9)
            assert np.allclose(num_j, sd[:, 1], rtol=1e-5, atol=1e-9)
            assert np.allclose(num_k, sd[:, 2], rtol=1e-5, atol=1e-9)
            # force() returns minus the dEdG-weighted sums of the same partials
            assert abs(phi + sd[:, 0].sum()) < 1e-9 and np.allclose(e2, -sd[:, 1:].sum(axis=0), atol=1e-9)


def _fd_forces(pot, offs, posn, types, cell, atoms, h=1e-5):
    out = []
    for a in atoms:
        row = []
        for c in range(3):
            xp = posn.copy(); xp[a, c] += h
            xm = posn.copy(); xm[a, c] -= h
            Ep = pot.compute(offs, xp, types, cell, forces=False)[0].sum()
            Em = pot.compute(offs, xm, types, cell, forces=False)[0].sum()
            row.append(-(Ep - Em) / (2 * h))
        out.append(row)
    return np.array(out)


def test_forces_fd_fcc(pot1):
    offs, posn, types, cell = pack_batch(W.config1())
    E, F, _, _, _ = pot1.compute(offs, posn, types, cell)
    atoms = [0, 17, 55, 107]
    assert np.allclose(_fd_forces(pot1, offs, posn, types, cell, atoms), F[atoms], rtol=1e-6, atol=1e-8)
    assert np.abs(F.sum(axis=0)).max() < 1e-10


def test_forces_fd_images_and_types(pot2):
    """cells smaller than the cutoff: every periodic image carries its Newton-3rd force"""
    offs, posn, types, cell = pack_batch(cases.tiny_cells())
    E, F, _, _, _ = pot2.compute(offs, posn, types, cell)
    atoms = list(range(len(types)))
    assert np.allclose(_fd_forces(pot2, offs, posn, types, cell, atoms), F, rtol=1e-6, atol=1e-7)


def test_generic_basis_forces_fd(oracle):
    pot = oracle.load_text(cases.generic_potential_text())
    offs, posn, types, cell = pack_batch(cases.tiny_cells()[1:2] + cases.small_binary(n_struc=1, seed=4))
    E, F, _, _, _ = pot.compute(offs, posn, types, cell)
    atoms = [0, 2, 4, 7, 20]
    assert np.allclose(_fd_forces(pot, offs, posn, types, cell, atoms), F[atoms], rtol=1e-6, atol=1e-7)


def test_virial_is_strain_derivative(pot2):
    offs, posn, types, cell = pack_batch(cases.tiny_cells()[1:2])
    E, F, Wv, _, _ = pot2.compute(offs, posn, types, cell)
    R = cell[0].reshape(3, 3).T
    eps = 1e-6
    for a in range(3):
        for b in range(3):
            def energy(e):
                M = np.eye(3); M[a, b] += e
                return pot2.compute(offs, posn @ M.T, types, (M @ R).T.reshape(1, 9), forces=False)[0][0]
            dE = (energy(eps) - energy(-eps)) / (2 * eps)
            assert abs(dE + Wv[0][b, a]) < 1e-6 * max(1.0, abs(Wv[0]).max())


def test_supercell_invariance(pot1):
    """every atom of a 2x1x1 replica has the symmetry functions of its original"""
    x, t, R = W.config1()[0]
    R2 = R.copy(); R2[:, 0] *= 2
    x2 = np.concatenate([x, x + R[:, 0]])
    t2 = np.concatenate([t, t])
    o1, p1, ty1, c1 = pack_batch([(x, t, R)])
    o2, p2, ty2, c2 = pack_batch([(x2, t2, R2)])
    _, _, _, G1, _ = pot1.compute(o1, p1, ty1, c1, forces=False, symm=True)
    _, _, _, G2, _ = pot1.compute(o2, p2, ty2, c2, forces=False, symm=True)
    assert np.allclose(G2[:len(x)], G1, rtol=1e-12, atol=1e-14)
    assert np.allclose(G2[len(x):], G1, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("wE,wF", [(1.0, 0.0), (1.0, 0.1), (0.0, 1.0)])
def test_training_gradient_fd(oracle, wE, wF):
    pot = oracle.load_text(W.config_potential_text(3))
    structs = cases.small_binary(n_struc=2, seed=8)
    offs, posn, types, cell = pack_batch(structs)
    Eref, Fref = W.lennard_jones(structs)
    Fref = np.concatenate(Fref)
    Eref = Eref * 0.01
    Fref = Fref * 0.01
    loss, g = pot.train(offs, posn, types, cell, Eref, Fref, wE, wF)
    p0 = pot.get_params()
    rng = np.random.default_rng(3)
    gscale = np.abs(g).max()
    for k in rng.choice(len(p0), 12, replace=False):
        h = 1e-5 * max(1.0, abs(p0[k]))
        pp = p0.copy(); pp[k] += h
        pot.set_params(pp)
        lp = pot.train(offs, posn, types, cell, Eref, Fref, wE, wF)[0][0]
        pp[k] -= 2 * h
        pot.set_params(pp)
        lm = pot.train(offs, posn, types, cell, Eref, Fref, wE, wF)[0][0]
        pot.set_params(p0)
        fd = (lp - lm) / (2 * h)
        # central differences: O(h^2) truncation plus cancellation against the loss value
        assert abs(fd - g[k]) <= 1e-6 * max(abs(fd), abs(g[k])) + 1e-7 * gscale, (k, fd, g[k])


def test_training_gradient_threads(oracle):
    """structures split over threads (block rule, thread sums added in order) give the one-thread
    loss and gradient up to the order of the additions"""
    pot = oracle.load_text(W.config_potential_text(3))
    structs = cases.small_binary(n_struc=5, seed=12)
    offs, posn, types, cell = pack_batch(structs)
    Eref, Fref = W.lennard_jones(structs)
    Fref = np.concatenate(Fref)
    l1, g1 = pot.train(offs, posn, types, cell, Eref, Fref, 1.0, 0.1)
    l3, g3 = pot.train(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, nthreads=3)
    assert np.allclose(l3, l1, rtol=1e-13, atol=0)
    assert np.abs(g3 - g1).max() <= 1e-13 * np.abs(g1).max()


def test_energy_gradient_matches_error_cost_o1(oracle):
    """the energy term equals the reference trainer's energy gradient (nnptefr2.cpp:1321-1374,
    984-995): MSE loss, LINEAR normalisation, averaged over the batch"""
    pot = oracle.load_text(W.config_potential_text(3))
    structs = cases.small_binary(n_struc=3, seed=9)
    offs, posn, types, cell = pack_batch(structs)
    Eref = np.array([-0.2 * len(t) for _, t, _ in structs])
    Fref = np.zeros_like(posn)
    loss, g = pot.train(offs, posn, types, cell, Eref, Fref, 1.0, 0.0)
    l2, g2 = pot.error_cost_o1(offs, posn, types, cell, Eref)
    assert abs(loss[1] - l2) < 1e-12 * max(1, abs(l2))
    assert np.allclose(g, g2, rtol=1e-10, atol=1e-14)


@pytest.mark.parametrize("loss", [1, 2, 3, 4])
def test_energy_loss_variants_fd(oracle, loss):
    """Every loss (MSE, MAE, HUBER, ASINH; nnptefr2.cpp:1339-1368) under every normalisation
    (IDENTITY, LINEAR, SQRT, CBRT, LOG; 606-612): the gradient of the energy term against central
    differences, and the same numbers from the error_cost_o1 restatement."""
    pot = oracle.load_text(W.config_potential_text(3))
    structs = cases.small_binary(n_struc=2, seed=14)
    offs, posn, types, cell = pack_batch(structs)
    Eref = np.array([-0.05 * len(t) for _, t, _ in structs])
    Fref = np.zeros_like(posn)
    p0 = pot.get_params()
    rng = np.random.default_rng(loss)
    for norm in range(5):
        (L, LE, _), g = pot.train(offs, posn, types, cell, Eref, Fref, 1.0, 0.0, loss=loss, norm=norm, delta=0.5)
        l2, g2 = pot.error_cost_o1(offs, posn, types, cell, Eref, loss=loss, norm=norm, delta=0.5)
        assert abs(LE - l2) <= 1e-12 * max(1.0, abs(l2)) and np.allclose(g, g2, rtol=1e-10, atol=1e-14), (loss, norm)
        gscale = np.abs(g).max()
        for k in rng.choice(len(p0), 4, replace=False):
            h = 1e-5 * max(1.0, abs(p0[k]))
            pp = p0.copy(); pp[k] += h
            pot.set_params(pp)
            lp = pot.error_cost_o1(offs, posn, types, cell, Eref, loss=loss, norm=norm, delta=0.5)[0]
            pp[k] -= 2 * h
            pot.set_params(pp)
            lm = pot.error_cost_o1(offs, posn, types, cell, Eref, loss=loss, norm=norm, delta=0.5)[0]
            pot.set_params(p0)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[k]) <= 1e-6 * max(abs(fd), abs(g[k])) + 1e-7 * gscale, (loss, norm, k, fd, g[k])
    with pytest.raises(RuntimeError):
        pot.error_cost_o1(offs, posn, types, cell, Eref, loss=loss, norm=5)


@pytest.mark.parametrize("neuron", range(1, 20))
def test_activation_derivatives_fd(oracle, neuron):
    """d = da/dz and d2 = dd/dz for every activation of nn.cpp:149-810, away from the kinks at 0"""
    h = 1e-5
    for c in (0.7, 1.3):
        for z in np.concatenate([np.linspace(-3.0, -0.05, 9), np.linspace(0.05, 3.0, 9)]):
            a, d, d2 = oracle.activate(neuron, c, z)
            ap, dp, _ = oracle.activate(neuron, c, z + h)
            am, dm, _ = oracle.activate(neuron, c, z - h)
            assert abs((ap - am) / (2 * h) - d) <= 1e-7 * max(1.0, abs(d)), (neuron, c, z, d)
            assert abs((dp - dm) / (2 * h) - d2) <= 1e-6 * max(1.0, abs(d2)), (neuron, c, z, d2)


@pytest.mark.parametrize("neuron", ["ISRU", "ARCTAN", "TANHRE", "SWISH", "GELU", "MISH", "PFLU", "SERF", "LOGISH",
                                    "SQPLUS", "ATISH", "TEST"])
def test_training_gradient_fd_activations(oracle, neuron):
    """the force term of the training loss uses f'' of the hidden activations"""
    pot = oracle.load_text(cases.activation_potential_text(neuron))
    structs = cases.small_binary(n_struc=1, seed=4)
    offs, posn, types, cell = pack_batch(structs)
    Eref, Fref = W.lennard_jones(structs)
    Fref = np.concatenate(Fref) * 0.01
    Eref = Eref * 0.01
    loss, g = pot.train(offs, posn, types, cell, Eref, Fref, 0.3, 1.0)
    p0 = pot.get_params()
    rng = np.random.default_rng(11)
    gscale = np.abs(g).max()
    for k in rng.choice(len(p0), 8, replace=False):
        hh = 1e-5 * max(1.0, abs(p0[k]))
        pp = p0.copy(); pp[k] += hh
        pot.set_params(pp)
        lp = pot.train(offs, posn, types, cell, Eref, Fref, 0.3, 1.0)[0][0]
        pp[k] -= 2 * hh
        pot.set_params(pp)
        lm = pot.train(offs, posn, types, cell, Eref, Fref, 0.3, 1.0)[0][0]
        pot.set_params(p0)
        fd = (lp - lm) / (2 * hh)
        assert abs(fd - g[k]) <= 1e-6 * max(abs(fd), abs(g[k])) + 1e-7 * gscale, (neuron, k, fd, g[k])


def test_angular_sums_equal_moment_contractions(pot2):
    """The oracle's triplet sums of the GAUSS angular functions (|1/2 + lambda/2 cos|^zeta with
    integer zeta, basis_angular.cpp:376-381, each unordered neighbour pair once) against an
    independent form: with a_j = fc(r_j) exp(-r_j^2/eta^2) and moments M_a = sum_j a_j u_j^a over
    multi-indices a, sum_pairs a_j a_k cos^m = sum_{|a|=m} (m!/a!) M^J_a M^K_a (same species: half
    of it minus sum_j a_j^2); the binomial expansion in cos then gives every function."""
    import itertools
    import math
    structs = W.config2(nstruc=1)
    offs, posn, types, cell = pack_batch(structs)
    G = pot2.compute(offs, posn, types, cell, symm=True)[3]
    x, t, R = structs[0]
    rc = 6.5
    fc = lambda r: 0.5 * (np.cos(np.pi * r / rc) + 1.0)
    etas = [float(f"{1 / np.sqrt(eb):f}") for eb in (0.003, 0.01)]
    rows = [(e, z, lam) for e in etas for z in (1, 2, 4, 8) for lam in (1, -1)]
    alphas = sorted({a for m in range(9) for a in itertools.product(range(m + 1), repeat=3) if sum(a) == m},
                    key=lambda a: (sum(a), a))
    mdeg = np.array([sum(a) for a in alphas])
    mcoef = np.array([math.factorial(sum(a)) / math.prod(math.factorial(k) for k in a) for a in alphas])
    shifts = np.array(list(itertools.product(range(-2, 3), repeat=3)), float) @ R
    for i in (0, 7, len(x) - 1):
        M = np.zeros((2, 2, len(alphas)))
        S = np.zeros((2, 2))
        for sh in shifts:
            d = x[i] - x - sh
            dd = np.linalg.norm(d, axis=1)
            for j in np.nonzero((dd < rc) & (dd > 1e-9))[0]:
                u = d[j] / dd[j]
                mono = np.array([u[0] ** a[0] * u[1] ** a[1] * u[2] ** a[2] for a in alphas])
                for g, e in enumerate(etas):
                    a = fc(dd[j]) * np.exp(-dd[j] ** 2 / e ** 2)
                    M[t[j], g] += a * mono
                    S[t[j], g] += a * a
        want = []
        for J in range(2):
            for K in range(J, 2):
                for e, z, lam in rows:
                    g = etas.index(e)
                    v = 0.0
                    for m in range(z + 1):
                        sel = mdeg == m
                        D = np.sum(mcoef[sel] * M[J, g, sel] * M[K, g, sel])
                        v += math.comb(z, m) * 0.5 ** (z - m) * (0.5 * lam) ** m * (0.5 * (D - S[J, g]) if J == K else D)
                    want.append(v)
        got = G[i, 24:24 + len(want)]
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12)
