"""GPU training adjoint and molecular dynamics vs the oracle, through the C ABI.

Training: L = wE/S sum 1/2 ((E_s-Eref_s)/N_s)^2 + wF/(3N) sum 1/2 |F-Fref|^2. The FP64 gradient
matches the oracle (relative to the gradient's scale, 1e-9) and central finite differences of the
GPU's own loss; with wF = 0 it equals the reference trainer's energy gradient
(NNPTEFR::error_cost_o1, nnptefr2.cpp:1321-1374 + 984-995, restated in the oracle).
MD: velocity Verlet (integrator.cpp:177-200) step by step against the oracle, and energy
conservation over a longer run.
"""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, AnnError, Context
from ann_gb300 import workloads as W
from ann_gb300.api import pack_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = Context(use_graphs=True)
    yield c
    c.close()


def _train_case():
    structs = cases.small_binary(n_struc=3, seed=8)
    offs, posn, types, cell = pack_batch(structs)
    Eref, Fref = W.lennard_jones(structs)
    return offs, posn, types, cell, Eref * 0.01, np.concatenate(Fref) * 0.01


def test_init_network_matches_reference_rng(ctx):
    ctx.load_text(W.config_potential_text(2, with_weights=False))
    ctx.init_network(0, 1234, dist=0, init=4, sigma_b=0.001, sigma_w=1.0)
    ctx.init_network(1, 99, dist=0, init=4, sigma_b=0.001, sigma_w=1.0)
    p = ctx.get_params()
    want = np.concatenate([W.xavier_network(1234, 72, [64, 64, 1]), W.xavier_network(99, 72, [64, 64, 1])])
    assert np.array_equal(p, want)


@pytest.mark.parametrize("wE,wF", [(1.0, 0.1), (1.0, 0.0), (0.0, 1.0)])
def test_gradient_matches_oracle(ctx, oracle, tmp_path, wE, wF):
    text = cases.config_potential(ctx, 3, tmp_path)
    pot = oracle.load_text(text)
    offs, posn, types, cell, Eref, Fref = _train_case()
    loss = ctx.train_forward(offs, posn, types, cell, Eref, Fref, wE, wF, precision=FP64)
    g = ctx.train_backward()
    lo, go = pot.train(offs, posn, types, cell, Eref, Fref, wE, wF)
    assert np.allclose(loss, lo, rtol=1e-10, atol=1e-14)
    scale = np.abs(go).max()
    assert np.abs(g - go).max() <= 1e-9 * scale
    if wF == 0.0:
        l2, g2 = pot.error_cost_o1(offs, posn, types, cell, Eref)
        assert np.abs(g - g2).max() <= 1e-9 * np.abs(g2).max()
    # mixed precision gradient stays close to FP64
    ctx.train_forward(offs, posn, types, cell, Eref, Fref, wE, wF, precision=MIXED)
    gm = ctx.train_backward()
    assert np.abs(gm - g).max() <= 1e-3 * scale


@pytest.mark.parametrize("loss", ["MSE", "MAE", "HUBER", "ASINH"])
def test_loss_variants_match_oracle(ctx, oracle, tmp_path, loss):
    """The trainer's energy losses (MSE, MAE, HUBER, ASINH) under every normalisation (IDENTITY,
    LINEAR, SQRT, CBRT, LOG) with the force term on: loss and gradient vs the oracle in FP64, the
    mixed gradient near FP64, and the setting left as found for the other tests."""
    text = cases.config_potential(ctx, 3, tmp_path)
    pot = oracle.load_text(text)
    offs, posn, types, cell, Eref, Fref = _train_case()
    try:
        for norm in range(5):
            ctx.train_set_loss(loss, norm, delta=0.5)
            lo, go = pot.train(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, loss=ctx.LOSS[loss], norm=norm, delta=0.5)
            l3 = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
            g = ctx.train_backward()
            assert np.allclose(l3, lo, rtol=1e-10, atol=1e-14), (loss, norm)
            assert np.abs(g - go).max() <= 1e-9 * np.abs(go).max(), (loss, norm)
            if norm == 1:
                ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=MIXED)
                gm = ctx.train_backward()
                assert np.abs(gm - go).max() <= 2e-3 * np.abs(go).max(), loss
        with pytest.raises(AnnError, match="loss"):
            ctx.train_set_loss(5, 1)
        with pytest.raises(AnnError, match="normalization"):
            ctx.train_set_loss(loss, 5)
        with pytest.raises(AnnError, match="delta"):
            ctx.train_set_loss(loss, 1, delta=0.0)
    finally:
        ctx.train_set_loss("MSE", "LINEAR", 1.0)


def test_gradient_finite_differences_on_gpu(ctx, tmp_path):
    cases.config_potential(ctx, 3, tmp_path)
    offs, posn, types, cell, Eref, Fref = _train_case()
    ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
    g = ctx.train_backward()
    p0 = ctx.get_params()
    rng = np.random.default_rng(5)
    scale = np.abs(g).max()
    for k in rng.choice(len(p0), 10, replace=False):
        h = 1e-5 * max(1.0, abs(p0[k]))
        pp = p0.copy(); pp[k] += h
        ctx.set_params(pp)
        lp = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)[0]
        pp[k] -= 2 * h
        ctx.set_params(pp)
        lm = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)[0]
        ctx.set_params(p0)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * abs(g[k]) + 1e-7 * scale, (k, fd, g[k])


def _md_case():
    x, v, t, R = W.config5(cells=(3, 3, 3))
    return x, v, t, R


def test_md_steps_match_oracle(ctx, oracle, tmp_path):
    text = cases.config_potential(ctx, 5, tmp_path)
    pot = oracle.load_text(text)
    x, v, t, R = _md_case()
    masses = np.array([39.948])
    ctx.md_init(x, v, t, R, masses, dt_fs=2.0, skin=0.5, precision=FP64)
    xo, vo = x.copy(), v.copy()
    offs, _, _, cell = pack_batch([(x, t, R)])
    Fo = pot.compute(offs, xo, t, cell)[1]
    for step in range(5):
        pe, ke, _ = ctx.md_run(1)
        peo, keo = pot.md_step(xo, vo, t, R, masses, 2.0, Fo)
        xg, vg, fg = ctx.md_state()
        d = xg - xo
        Ri = np.linalg.inv(R)
        d -= (np.round(d @ Ri.T)) @ R.T      # the GPU wraps only when it rebuilds its list
        assert np.abs(d).max() < 1e-9
        assert np.abs(vg - vo).max() < 1e-10
        assert abs(pe - peo) < 1e-9 * max(1.0, abs(peo)) and abs(ke - keo) < 1e-9 * max(1.0, keo)


def test_md_multitype_steps_match_oracle(ctx, oracle, tmp_path):
    """three species, so every MD step compacts type-sorted list rows segment by segment: FP64
    steps against the oracle, and the MIXED forces of the first step within 10 meV/A"""
    text = cases.config_potential(ctx, 4, tmp_path)
    pot = oracle.load_text(text)
    [(x, t, R)] = cases.ternary_box(dims=(8, 8, 6))
    masses = np.array([39.948, 20.180, 83.798])
    v = np.random.default_rng(4).normal(0.0, 0.002, x.shape)
    offs, _, _, cell = pack_batch([(x, t, R)])
    ctx.md_init(x, v, t, R, masses, dt_fs=1.0, skin=0.5, precision=MIXED)
    Fm = ctx.md_state()[2]
    ctx.md_init(x, v, t, R, masses, dt_fs=1.0, skin=0.5, precision=FP64)
    xo, vo = x.copy(), v.copy()
    Fo = pot.compute(offs, xo, t, cell)[1]
    assert np.abs(Fm - Fo).max() < 10e-3
    Ri = np.linalg.inv(R)
    for step in range(5):
        pe, ke, _ = ctx.md_run(1)
        peo, keo = pot.md_step(xo, vo, t, R, masses, 1.0, Fo)
        xg, vg, fg = ctx.md_state()
        d = xg - xo
        d -= (np.round(d @ Ri.T)) @ R.T
        assert np.abs(d).max() < 1e-9
        assert np.abs(vg - vo).max() < 1e-10
        assert np.abs(fg - Fo).max() < 1e-8 * max(1.0, np.abs(Fo).max())
        assert abs(pe - peo) < 1e-9 * max(1.0, abs(peo)) and abs(ke - keo) < 1e-9 * max(1.0, keo)


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_md_energy_conservation(ctx, tmp_path, prec):
    cases.config_potential(ctx, 5, tmp_path)
    x, v, t, R = _md_case()
    ctx.md_init(x, v, t, R, np.array([39.948]), dt_fs=2.0, skin=0.5, precision=prec)
    pe0, ke0, _ = ctx.md_run(1)
    e0 = pe0 + ke0
    pe, ke, rebuilds = ctx.md_run(400)
    drift = abs(pe + ke - e0) / len(t)          # eV/atom over 0.8 ps
    assert drift < 2e-4, drift
    assert rebuilds >= 0


def test_md_lj_argon_crystal_mixed(ctx):
    """mixed-precision MD of an FCC argon box (256 atoms) under the networks that hold a
    Lennard-Jones pair potential: over 2 ps the crystal holds (minimum distance > 3 A, temperature
    near equipartition of the 80 K start) and the total energy drifts < 0.05 meV/atom"""
    ctx.load_text(W.lj_argon_text(5))
    x, v, t, R = W.config5(cells=(4, 4, 4))
    ctx.md_init(x, v, t, R, np.array([W.MASS["Ar"]]), dt_fs=2.0, skin=0.5, precision=MIXED)
    pe0, ke0, _ = ctx.md_run(1)
    pe, ke, rebuilds = ctx.md_run(1000)
    n = len(t)
    T = 2 * ke / (3 * n * 8.617333262e-5)
    assert 15.0 < T < 70.0, T
    assert abs(pe + ke - pe0 - ke0) / n < 5e-5, (pe + ke - pe0 - ke0) / n
    xs = ctx.md_state()[0]
    d = xs[:, None] - xs[None]
    Ls = np.diag(R)
    d -= Ls * np.round(d / Ls)
    dd = np.linalg.norm(d, axis=2)
    np.fill_diagonal(dd, np.inf)
    assert dd.min() > 3.0
    assert rebuilds < 1000


@pytest.mark.parametrize("neuron", ["GELU", "MISH", "SERF", "ARCTAN", "TEST"])
def test_gradient_other_activations(ctx, oracle, neuron):
    """the force-term adjoint through f'' of the other activations, FP64 vs the oracle"""
    text = cases.activation_potential_text(neuron)
    ctx.load_text(text)
    pot = oracle.load_text(text)
    offs, posn, types, cell, Eref, Fref = _train_case()
    loss = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 0.3, 1.0, precision=FP64)
    g = ctx.train_backward()
    lo, go = pot.train(offs, posn, types, cell, Eref, Fref, 0.3, 1.0)
    assert np.allclose(loss, lo, rtol=1e-10, atol=1e-14)
    assert np.abs(g - go).max() <= 1e-9 * np.abs(go).max()


def test_adam_steps_on_device(ctx, tmp_path):
    """Adam (NN::ADAM::step, opt/algo.cpp:280-296) applied on the device to the resident parameters:
    the parameters after three steps equal the same update done in numpy, and the refreshed device
    copies (FP64, FP32 and the tensor-core images) give the energies of a context loaded with them."""
    text = cases.config_potential(ctx, 3, tmp_path)
    offs, posn, types, cell, Eref, Fref = _train_case()
    p = ctx.get_params()
    lr, b1, b2, eps = 1e-3, 0.9, 0.999, 1e-16
    ctx.adam_init(lr, b1, b2, eps)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for t in range(1, 4):
        ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
        g = ctx.train_backward()
        ctx.adam_step()
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        p = p - lr / (1 - b1 ** t) * m / (np.sqrt(v / (1 - b2 ** t)) + eps)
    pd = ctx.get_params()
    assert np.allclose(pd, p, rtol=1e-12, atol=1e-15)
    # the same three steps with the gradient left on the device (train_backward without download)
    ctx.load_text(text)
    ctx.adam_init(lr, b1, b2, eps)
    for t in range(1, 4):
        ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
        assert ctx.train_backward(download=False) is None
        ctx.adam_step()
    assert np.allclose(ctx.get_params(), pd, rtol=1e-12, atol=1e-15)   # gradient sums are atomic: last bits vary
    other = Context()
    try:
        other.load_text(text)
        other.set_params(pd)
        for prec in (FP64, MIXED):
            E1, F1, _ = ctx.compute(offs, posn, types, cell, precision=prec)
            E2, F2, _ = other.compute(offs, posn, types, cell, precision=prec)
            # forces: Newton-3rd shares are added atomically, so their order (and the last FP32 bit) varies
            assert np.allclose(E1, E2, rtol=1e-12, atol=1e-12)
            assert np.abs(F1 - F2).max() <= (1e-12 if prec == FP64 else 1e-5)
    finally:
        other.close()


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_staged_training_steps_equal_full_steps(ctx, tmp_path, prec):
    """ann_train_forward_staged (the neighbour rows and symmetry functions of the preceding
    ann_train_forward kept on the device, as the reference trainer keeps each structure's symm)
    gives the losses, gradients and Adam trajectory of full ann_train_forward calls on the same
    batch: to 1e-12 in FP64, to 1e-5 in the mixed form (FP32 force atomics add in varying order)."""
    text = cases.config_potential(ctx, 3, tmp_path)
    offs, posn, types, cell, Eref, Fref = _train_case()
    p0 = ctx.get_params()
    tol = 1e-12 if prec == FP64 else 1e-5

    def run(staged):
        ctx.set_params(p0)
        ctx.adam_init(1e-3, 0.9, 0.999, 1e-16)
        losses, grads = [], []
        for k in range(4):
            if staged and k > 0:
                losses.append(ctx.train_forward_staged(1.0, 0.1, precision=prec))
            else:
                losses.append(ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=prec))
            grads.append(ctx.train_backward())
            ctx.adam_step()
        return np.array(losses), np.array(grads), ctx.get_params()

    La, Ga, Pa = run(False)
    Lb, Gb, Pb = run(True)
    assert np.allclose(Lb, La, rtol=tol, atol=1e-15)
    assert np.abs(Gb - Ga).max() <= tol * np.abs(Ga).max()
    if prec == FP64:   # (mixed: Adam's first steps are sign steps, so last-bit noise in tiny gradients moves them by lr)
        assert np.allclose(Pb, Pa, rtol=tol, atol=1e-15)
    # new parameters set from the host between staged steps are used
    ctx.set_params(p0)
    l1 = ctx.train_forward_staged(1.0, 0.1, precision=prec)
    assert np.allclose(l1, La[0], rtol=tol, atol=1e-15)
    ctx.load_text(text)


def test_staged_training_refused_without_its_batch(ctx, tmp_path):
    ANN_ERR_STATE = 6
    cases.config_potential(ctx, 3, tmp_path)
    offs, posn, types, cell, Eref, Fref = _train_case()
    with pytest.raises(AnnError) as e:          # a freshly loaded potential: nothing staged
        ctx.train_forward_staged(1.0, 0.1, precision=FP64)
    assert e.value.code == ANN_ERR_STATE
    ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
    with pytest.raises(AnnError) as e:          # the other precision
        ctx.train_forward_staged(1.0, 0.1, precision=MIXED)
    assert e.value.code == ANN_ERR_STATE
    ctx.train_forward_staged(1.0, 0.1, precision=FP64)
    ctx.compute(offs, posn, types, cell, precision=FP64)
    with pytest.raises(AnnError) as e:          # an E+F call in between replaced the staged state
        ctx.train_forward_staged(1.0, 0.1, precision=FP64)
    assert e.value.code == ANN_ERR_STATE


def _decay(name, gamma, t, alpha, period):
    """opt::Decay::step (opt/decay.cpp:42-62)."""
    return {"CONST": gamma, "EXP": gamma * (1.0 - alpha), "GAUSS": gamma * (1.0 - 2.0 * alpha * t),
            "SQRT": gamma * (1.0 - 0.5 * alpha / (1.0 + alpha * t)), "INV": gamma * (1.0 - alpha / (1.0 + alpha * t)),
            "STEP": gamma * alpha if (t > 0 and t % period == 0) else gamma}[name]


@pytest.mark.parametrize("decay", ["CONST", "EXP", "GAUSS", "SQRT", "INV", "STEP"])
def test_adam_schedule_and_weight_decay(ctx, tmp_path, decay):
    """The trainer's order (nnptefr2.cpp:1025-1049): gamma from the decay schedule, the Adam step,
    then weight decay of the weights (not the biases) from the pre-step values, for every
    regularisation; four steps against a numpy replay of the same gradients."""
    text = cases.config_potential(ctx, 3, tmp_path)
    offs, posn, types, cell, Eref, Fref = _train_case()
    wm = np.tile(np.r_[np.zeros(64 + 64 + 1), np.ones(72 * 64 + 64 * 64 + 64)], 2)   # biases, then weights, per type
    f = {"LASSO": np.sign, "RIDGE": lambda x: x, "HUBER": lambda x: x / np.sqrt(1.0 + x * x), "ASINH": np.arcsinh}
    lr, b1, b2, eps, alpha, period, eta = 1e-3, 0.9, 0.999, 1e-16, 0.05, 2, 0.01
    try:
        for reg in ("NONE", "LASSO", "RIDGE", "HUBER", "ASINH"):
            ctx.load_text(text)
            p = ctx.get_params()
            assert len(p) == len(wm)
            ctx.adam_init(lr, b1, b2, eps)
            ctx.opt_schedule(decay, alpha=alpha, period=period, reg=reg, eta=eta)
            m = np.zeros_like(p); v = np.zeros_like(p)
            gamma, b1i, b2i = lr, b1, b2
            for t in range(4):
                ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
                g = ctx.train_backward()
                ctx.adam_step()
                gamma = _decay(decay, gamma, t, alpha, period)
                m = b1 * m + (1 - b1) * g
                v = b2 * v + (1 - b2) * g * g
                pn = p - gamma * (1.0 / (1.0 - b1i)) * m / (np.sqrt((1.0 / (1.0 - b2i)) * v) + eps)
                if reg != "NONE":
                    pn = pn - gamma * eta * wm * f[reg](p)
                p = pn
                b1i *= b1; b2i *= b2
            assert np.allclose(ctx.get_params(), p, rtol=1e-10, atol=1e-13), (decay, reg)
        with pytest.raises(AnnError, match="decay"):
            ctx.opt_schedule(7)
        with pytest.raises(AnnError, match="regularization"):
            ctx.opt_schedule("CONST", reg=5)
    finally:
        ctx.opt_schedule()


class _RefOpt:
    """The reference's optimiser steps (src/opt/algo.cpp:97-660) in numpy, for the replay."""

    def __init__(self, algo, n, gamma, eta, eps, w):
        self.a, self.gamma, self.eta, self.eps, self.w = algo, gamma, eta, eps, w
        self.s0 = np.full(n, 0.1) if algo == "RPROP" else np.zeros(n)
        self.s1, self.s2, self.gold, self.cg = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n)
        self.b1i, self.b2i, self.b1, self.b2 = 0.9, 0.999, 0.9, 0.999
        self.val_old = 0.0

    def step(self, p, g, val):
        a, gm, eta, eps = self.a, self.gamma, self.eta, self.eps
        b1, b2 = self.b1, self.b2
        b1ii, b2ii = 1.0 / (1.0 - self.b1i), 1.0 / (1.0 - self.b2i)
        p = p.copy(); g = g.copy()
        if a == "SGD":
            p -= gm * g
        elif a in ("SDM", "NAG"):
            self.s0 = eta * self.s0 + gm * ((eta + 1.0) if a == "NAG" else 1.0) * g
            p -= self.s0
        elif a == "ADAGRAD":
            self.s0 += g * g; p -= gm * g / (np.sqrt(self.s0) + eps)
        elif a == "ADADELTA":
            self.s0 = eta * self.s0 + (1 - eta) * g * g
            dx = g * np.sqrt(self.s1) / (np.sqrt(self.s0) + eps)
            p -= dx
            self.s1 = eta * self.s1 + (1 - eta) * dx * dx
        elif a == "RMSPROP":
            self.s0 = 0.9 * self.s0 + 0.1 * g * g; p -= gm * g / (np.sqrt(self.s0) + eps)
        elif a in ("ADAM", "ADAMW", "ADAB", "YOGI", "NOGI", "NADAM", "AMSGRAD"):
            self.s0 = self.s0 * b1 + (1 - b1) * g
            if a == "ADAB":
                self.s1 = self.s1 * b2 + (1 - b2) * (g - self.s0) * (g - self.s0) + eps
            elif a in ("YOGI", "NOGI"):
                self.s1 = self.s1 - (1 - b2) * np.sign(self.s1 - g * g) * (g * g)
            else:
                self.s1 = self.s1 * b2 + (1 - b2) * g * g
            vv = self.s1
            if a == "AMSGRAD":
                self.s2 = np.maximum(self.s2, self.s1); vv = self.s2
            mm = b1 * self.s0 + (1 - b1) * g if a in ("NOGI", "NADAM") else self.s0
            if a == "ADAMW":
                p -= gm * (b1ii * mm / (np.sqrt(b2ii * vv) + eps) + self.w * p)
            else:
                p -= gm * b1ii * mm / (np.sqrt(b2ii * vv) + eps)
        elif a == "RPROP":
            inc = val > self.val_old
            sg = g * self.gold
            up, dn, ze = sg > 0, sg < 0, sg == 0
            self.s0[up] = np.minimum(self.s0[up] * 1.2, 50.0)
            self.s1[up] = -1.0 * np.sign(g[up]) * self.s0[up]
            p[up] += self.s1[up]
            self.s0[dn] = np.maximum(self.s0[dn] * 0.5, 1e-14)
            if inc:
                p[dn] -= self.s1[dn]
            g[dn] = 0.0
            self.s1[ze] = -1.0 * np.sign(g[ze]) * self.s0[ze]
            p[ze] += self.s1[ze]
        elif a == "CG":
            beta = np.dot(g, g - self.gold) / (np.dot(self.gold, self.gold) + eps)
            self.cg = beta * self.cg - g
            p += gm * self.cg
        self.gold = g
        self.val_old = val
        self.b1i *= b1; self.b2i *= b2
        return p


@pytest.mark.parametrize("algo", ["SGD", "SDM", "NAG", "ADAGRAD", "ADADELTA", "RMSPROP", "ADAM", "ADAMW", "ADAB", "YOGI", "NOGI",
                                  "NADAM", "AMSGRAD", "RPROP", "CG"])
def test_every_optimiser_matches_reference_steps(ctx, tmp_path, algo):
    """Every optimiser of the reference trainer on the device: three steps with the gradients and
    losses of the same batch against a numpy replay of opt::algo's step (CG's dot products on the
    device in a fixed order: 1e-9)."""
    text = cases.config_potential(ctx, 3, tmp_path)
    offs, posn, types, cell, Eref, Fref = _train_case()
    ctx.load_text(text)
    p = ctx.get_params()
    gamma, eta, eps, w = 1e-3, 0.5, 1e-8, 0.01
    ctx.opt_init(algo, gamma=gamma, eta=eta, eps=eps, w=w)
    ref = _RefOpt(algo, len(p), gamma, eta, eps, w)
    for _ in range(3):
        loss = ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=FP64)
        g = ctx.train_backward()
        ctx.opt_step()
        p = ref.step(p, g, loss[0])
    assert np.allclose(ctx.get_params(), p, rtol=1e-9, atol=1e-12), algo


def test_optimiser_errors(ctx, tmp_path):
    cases.config_potential(ctx, 3, tmp_path)
    with pytest.raises(AnnError, match="BFGS"):
        ctx.opt_init("BFGS")
    with pytest.raises(AnnError, match="algorithm"):
        ctx.opt_init(17)


def test_compute_after_md_leaves_md(ctx, tmp_path):
    """A batch computed after an MD run replaces the MD system: same results as a fresh context."""
    text = cases.config_potential(ctx, 5, tmp_path)
    x, v, t, R = _md_case()
    ctx.md_init(x, v, t, R, np.array([39.948]), dt_fs=2.0, skin=0.5, precision=MIXED)
    ctx.md_run(3)
    offs, posn, types, cell = pack_batch([(x, t, R)])
    other = Context()
    try:
        other.load_text(text)
        for prec in (FP64, MIXED):
            a = ctx.compute(offs, posn, types, cell, precision=prec)
            b = other.compute(offs, posn, types, cell, precision=prec)
            assert np.array_equal(a[0], b[0])
            assert np.abs(a[1] - b[1]).max() <= (1e-12 if prec == FP64 else 1e-5)
        with pytest.raises(Exception):
            ctx.md_run(1)
    finally:
        other.close()
