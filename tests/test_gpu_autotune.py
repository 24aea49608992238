"""The launch-shape autotuner (ann_autotune / ann_set_tuning) through the C ABI: the choice is
valid and never slower than the built-in rules, results are unchanged under every shape (mixed
bars against FP64), and invalid shapes or states are refused with the context left usable."""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, AnnError, Context

pytestmark = pytest.mark.gpu


def _bars(E, F, E64, F64, offs):
    nat = np.maximum(np.diff(offs), 1)
    assert np.max(np.abs(E - E64) / nat) * 1e3 < 1.0
    assert np.max(np.abs(F - F64)) * 1e3 < 10.0


def test_autotune_choice_and_results(gpu_lib, tmp_path):
    ctx = Context()
    try:
        structs = cases.W.config2(nstruc=32)
        offs, posn, types, cell = cases.batch(structs)
        cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
        E64, F64, _ = ctx.compute(offs, posn, types, cell, precision=FP64)
        E0, F0, _ = ctx.compute(offs, posn, types, cell, precision=MIXED)
        t = ctx.autotune(precision=MIXED, reps=3)
        assert all(g in (0, 1, 2, 4) for g in t["tc_groups"])
        assert 0 <= t["bp_blocks_per_sm"] <= 16 and 0 <= t["nbr_blocks_per_sm"] <= 64
        assert 0.0 < t["ms"] <= t["ms_default"]
        E1, F1, _ = ctx.compute(offs, posn, types, cell, precision=MIXED)
        _bars(E1, F1, E64, F64, offs)
        assert np.max(np.abs(E1 - E0)) < 1e-6 * max(1.0, np.max(np.abs(E0)))
        for g in (1, 2, 4):
            for bp, nb in ((1, 1), (3, 8)):
                ctx.set_tuning(tc_groups=(g, g, 0, 0), bp_blocks_per_sm=bp, nbr_blocks_per_sm=nb)
                E, F, _ = ctx.compute(offs, posn, types, cell, precision=MIXED)
                _bars(E, F, E64, F64, offs)
        ctx.set_tuning(bp_blocks_per_sm=1, nbr_blocks_per_sm=1)
        E, F, _ = ctx.compute(offs, posn, types, cell, precision=FP64)
        assert np.max(np.abs(E - E64)) <= 1e-10 * max(1.0, np.max(np.abs(E64)))
        t64 = ctx.autotune(precision=FP64, reps=1)
        assert t64["tc_groups"] == [0, 0, 0, 0]
        ctx.set_tuning()
        for bad in (dict(tc_groups=(3, 0, 0, 0)), dict(bp_blocks_per_sm=17), dict(nbr_blocks_per_sm=-1)):
            with pytest.raises(AnnError):
                ctx.set_tuning(**bad)
        E, F, _ = ctx.compute(offs, posn, types, cell, precision=MIXED)
        _bars(E, F, E64, F64, offs)
    finally:
        ctx.close()


def test_autotune_needs_a_staged_batch(gpu_lib, tmp_path):
    ctx = Context()
    try:
        cases.config_potential(ctx, 5, tmp_path)
        with pytest.raises(AnnError):
            ctx.autotune()
        x, v, t, R = cases.W.config5(cells=(3, 3, 3))
        ctx.md_init(x, v, t, R, np.array([39.948]), dt_fs=2.0, skin=0.5, precision=MIXED)
        with pytest.raises(AnnError):
            ctx.autotune()
        ctx.md_run(2)
    finally:
        ctx.close()
