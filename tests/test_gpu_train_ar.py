"""The reference's argon example run as a real-data fixture (examples/Ar: trainer input
nn_pot_train_init.txt, basis_Ar, the QE outputs it lists; converted by
tests/golden/make_ar_qe_fixture.py): input statistics and MEAN/DEV pre-conditioning on the device,
then Adam (gamma 1e-3) on the energy loss, all on the device, in FP64.

Parity: the first steps follow the oracle's gradient with the reference's Adam update applied on
the host (parameters within 1e-7 relative). Learning: after 500 steps the energy RMSE of the
training set (one-atom cells, 19-254 A^3 per atom) and of the validation set (32-atom NVE frames,
not trained on) are a few meV/atom."""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, Context

pytestmark = pytest.mark.gpu


def _rmse(ctx, b, e_ref):
    offs, posn, types, cell = b[:4]
    E, _, _ = ctx.compute(offs, posn, types, cell, forces=False, virial=False, precision=FP64)
    return np.sqrt(np.mean(((E - e_ref) / np.diff(offs)) ** 2)) * 1e3


def _oracle_adam(oracle, text, tb, steps, lr=1e-3, b1=0.9, b2=0.999, eps=1e-16):
    """The oracle's energy-loss gradient with NN::ADAM::step (opt/algo.cpp:280-296) on the host."""
    pot = oracle.load_text(text)
    p = pot.get_params()
    m, v = np.zeros_like(p), np.zeros_like(p)
    for it in range(1, steps + 1):
        _, g = pot.train(*tb[:4], tb[4], np.zeros((int(tb[0][-1]), 3)), 1.0, 0.0)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        p = p - lr * (m / (1 - b1 ** it)) / (np.sqrt(v / (1 - b2 ** it)) + eps)
        pot.set_params(p)
    return p


def test_argon_example_trains_on_device(gpu_lib, oracle, tmp_path):
    tb, vb = cases.argon_example_data()
    ctx = Context()
    try:
        ctx.load_text(cases.argon_example_potential())
        ctx.stats_reset()
        ctx.compute(*tb[:4], forces=False, virial=False, precision=FP64)
        ctx.stats_accumulate()
        ctx.precondition("MEAN", "DEV")
        p = tmp_path / "pre.ann"
        ctx.write(p)
        text = p.read_text()                       # the pre-conditioned potential, as the oracle reads it
        r0 = (_rmse(ctx, tb, tb[4]), _rmse(ctx, vb, vb[4]))
        ctx.adam_init(lr=1e-3)
        zero_f = np.zeros((int(tb[0][-1]), 3))

        def step():
            ctx.train_forward(*tb[:4], tb[4], zero_f, w_energy=1.0, w_force=0.0, precision=FP64)
            ctx.train_backward()
            ctx.adam_step()

        for _ in range(5):
            step()
        p_dev = ctx.get_params()
        p_orc = _oracle_adam(oracle, text, tb, 5)
        assert np.max(np.abs(p_dev - p_orc) / np.maximum(np.abs(p_orc), 1e-3)) < 1e-7
        for _ in range(495):
            step()
        r1 = (_rmse(ctx, tb, tb[4]), _rmse(ctx, vb, vb[4]))
        print(f"argon example: energy RMSE train {r0[0]:.2f} -> {r1[0]:.2f} meV/atom, validation {r0[1]:.2f} -> {r1[1]:.2f}")
        assert r1[0] < 10.0 and r1[1] < 5.0
        assert r1[0] < r0[0] / 5 and r1[1] < r0[1] / 5
    finally:
        ctx.close()
