"""The oracle's restatement of the trainer's input statistics and pre-conditioning
(nnptefr2.cpp:686-858), pinned on the CPU against the reference's formulas written out directly."""
import numpy as np
import pytest


def _direct(G, types, nin, T):
    out = []
    for t in range(T):
        g = G[types == t, :nin[t]]
        N = len(g)
        mx, mn = g.max(axis=0), g.min(axis=0)
        har = N / np.sum(1.0 / g, axis=0)
        avg = g.sum(axis=0) / N
        dev = np.sqrt(np.sum((avg - g) ** 2, axis=0) / (N - 1.0))
        rms = np.sqrt(np.sum(g * g, axis=0) / N)
        out.append((N, np.stack([mx, mn, har, avg, dev, rms])))
    return out


def test_input_stats_match_the_reference_formulas(oracle):
    rng = np.random.default_rng(4)
    T, imax, nin = 3, 9, [9, 6, 4]
    types = rng.integers(0, T, 500).astype(np.int32)
    G = rng.lognormal(0.0, 1.0, (500, imax))
    st, cnt = oracle.input_stats(nin, types, G)
    for t, (N, ref) in enumerate(_direct(G, types, nin, T)):
        assert cnt[t] == N
        assert np.allclose(st[t, :, :nin[t]], ref, rtol=1e-13, atol=0)


@pytest.mark.parametrize("prebias", range(6))
@pytest.mark.parametrize("prescale", range(4))
def test_precondition_enums(oracle, prebias, prescale):
    rng = np.random.default_rng(prebias * 7 + prescale)
    n = 5
    mx = rng.uniform(0.5, 2.0, n)
    mx[0] = 0.0                                   # MAX: not positive -> 1
    mn = mx - rng.uniform(0.0, 1.0, n)
    mn[1] = mx[1]                                 # MINMAX: zero range -> 1
    st = np.stack([mx, mn, rng.uniform(0.1, 1, n), rng.uniform(0.1, 1, n), rng.uniform(0.1, 1, n), rng.uniform(0.1, 1, n)])
    st[4, 2] = 0.0                                # DEV: zero deviation -> 1
    b, w = oracle.precondition(st, n, prebias, prescale, inbias=0.25, inscale=2.0)
    bias = [np.zeros(n), -st[3], -st[2], -st[5], -0.5 * (st[0] + st[1]), -st[1]][prebias]
    with np.errstate(divide="ignore"):
        scale = [np.ones(n), np.where(st[4] == 0, 1.0, 1.0 / st[4]),
                 np.where(st[0] - st[1] > 0, 1.0 / (st[0] - st[1]), 1.0), np.where(st[0] > 0, 1.0 / st[0], 1.0)][prescale]
    assert np.array_equal(b, bias + 0.25)
    assert np.array_equal(w, scale * 2.0)


def test_precondition_rejects_unknown_enums(oracle):
    st = np.ones((6, 3))
    with pytest.raises(ValueError, match="bias"):
        oracle.precondition(st, 3, 6, 0)
    with pytest.raises(ValueError, match="scaling"):
        oracle.precondition(st, 3, 0, 4)
