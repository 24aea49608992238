"""Input statistics and pre-conditioning of a training set on the device (nnptefr2.cpp:686-858)
vs the oracle's restatement over the same symmetry functions.

Bars: FP64 batches give the oracle's statistics within 1e-12 relative (the device merges chunk
partials with a pairwise update where the reference makes one pass per statistic); mixed batches
(FP32 symmetry functions) within 1e-5; the input scaling set by every PreBias x PreScale pair is
the oracle's from those statistics."""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, AnnError, Context

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


@pytest.fixture(scope="module")
def setup(gpu_lib, oracle, tmp_path_factory):
    ctx = Context()
    tmp = tmp_path_factory.mktemp("stats")
    batches = [cases.batch(cases.W.random_binary(n, 32, 200, seed=40 + k)) for k, n in enumerate((5, 3, 7))]
    text = cases.config_potential(ctx, 2, tmp)
    pot = oracle.load_text(text)
    nin = [pot.ninput(t) for t in range(pot.ntypes)]
    Gs, Ts = [], []
    for offs, posn, types, cell in batches:
        _, _, _, G, _ = pot.compute(offs, posn, types, cell, symm=True)
        Gs.append(G); Ts.append(types)
    ref = oracle.input_stats(nin, np.concatenate(Ts), np.concatenate(Gs))
    yield ctx, text, batches, nin, ref
    ctx.close()


def _accumulate(ctx, batches, prec):
    ctx.stats_reset()
    for offs, posn, types, cell in batches:
        ctx.compute(offs, posn, types, cell, forces=False, virial=False, precision=prec)
        ctx.stats_accumulate()


@pytest.mark.parametrize("prec,tol", [(FP64, 1e-12), (MIXED, 1e-5)])
def test_statistics_match_oracle(setup, prec, tol):
    ctx, text, batches, nin, (st, cnt) = setup
    ctx.load_text(text)
    _accumulate(ctx, batches, prec)
    for t in range(len(nin)):
        n, s = ctx.stats(t)
        ref = st[t, :, :nin[t]]
        assert n == cnt[t]
        # relative to each statistic, or to the mean magnitude of its input (the deviation of an input
        # with a small spread inherits the FP32 rounding of the input itself)
        scale = np.maximum(np.abs(ref), np.abs(ref[3])[None, :])
        assert np.max(np.abs(s - ref) / scale) < tol, t


def test_every_prebias_prescale_pair(setup, oracle):
    ctx, text, batches, nin, (st, cnt) = setup
    for pb in range(6):
        for ps in range(4):
            ctx.load_text(text)
            _accumulate(ctx, batches, FP64)
            ctx.precondition(pb, ps, inbias=0.1, inscale=0.5)
            for t in range(len(nin)):
                b_ref, w_ref = oracle.precondition(st[t, :, :nin[t]], nin[t], pb, ps, 0.1, 0.5)
                w, b = ctx.input_scaling(t)
                assert np.allclose(b, b_ref, rtol=1e-11, atol=1e-13), (pb, ps, t)
                assert np.allclose(w, w_ref, rtol=1e-11, atol=0), (pb, ps, t)


def test_preconditioned_potential_round_trip(setup, oracle, tmp_path):
    """The preconditioned networks (inpb, inpw, outb = 0, outw = 1) are what the file says, and the
    oracle reading that file computes what the device computes."""
    ctx, text, batches, nin, _ = setup
    ctx.load_text(text)
    _accumulate(ctx, batches, FP64)
    ctx.precondition("MEAN", "DEV")
    p = tmp_path / "pre.ann"
    ctx.write(p)
    body = p.read_text()
    assert all(float(ln.split()[1]) == 1.0 for ln in body.splitlines() if ln.startswith("outw"))
    assert all(float(ln.split()[1]) == 0.0 for ln in body.splitlines() if ln.startswith("outb"))
    pot = oracle.load_text(body)
    offs, posn, types, cell = batches[0]
    E, F, _ = ctx.compute(offs, posn, types, cell, precision=FP64)
    Eo, Fo, _, _, _ = pot.compute(offs, posn, types, cell)
    assert _rel(E, Eo) < 1e-10


def test_accumulation_order_and_state(setup):
    ctx, text, batches, nin, (st, cnt) = setup
    ctx.load_text(text)
    with pytest.raises(AnnError):
        ctx.stats(0)                                   # nothing accumulated since the load
    offs, posn, types, cell = batches[1]
    ctx.stats_reset()
    ctx.compute(offs, posn, types, cell, forces=False, virial=False, precision=FP64)
    ctx.stats_accumulate()
    n1, s1 = ctx.stats(0)
    ctx.stats_accumulate()                             # the same batch again: counts double, moments stay
    n2, s2 = ctx.stats(0)
    assert n2 == 2 * n1
    assert _rel(s2[[0, 1, 2, 3, 5]], s1[[0, 1, 2, 3, 5]]) < 1e-13
    # a batch of type-0 atoms only: type 1 has no atoms and keeps its scaling
    x, t, R = cases.W.random_binary(1, 40, 40, seed=2)[0]
    t[:] = 0
    o2, p2, t2, c2 = cases.batch([(x, t, R)])
    ctx.load_text(text)
    w1, b1 = ctx.input_scaling(1)
    ctx.stats_reset()
    ctx.compute(o2, p2, t2, c2, forces=False, virial=False, precision=FP64)
    ctx.stats_accumulate()
    assert ctx.stats(1)[0] == 0
    ctx.precondition("MID", "MINMAX")
    w1b, b1b = ctx.input_scaling(1)
    assert np.array_equal(w1, w1b) and np.array_equal(b1, b1b)
    with pytest.raises(AnnError, match="bias"):
        ctx.precondition(6, 0)
