"""Batch transfers through the library's page-locked buffers (one copy kernel each way) against
the copy-engine path of ordinary arrays, also for buffers viewed at offsets that are not 16-byte
aligned: the inputs arrive unchanged (the FP64 neighbour lists and pair vectors, which depend on
positions, types and cells only, are identical), and the results equal a copy-engine download of
the same device state bit for bit. Forces of two runs agree to 1e-12 (Newton's-third-law shares
are added by atomics, so their last bits vary between runs)."""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, Context
from ann_gb300.api import pack_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = Context(use_graphs=True)
    yield c
    c.close()


def _pinned_view(ctx, arr, offset):
    """arr copied into a library page-locked buffer, viewed `offset` elements in."""
    buf = ctx.pinned((arr.size + offset,), arr.dtype)
    v = buf[offset:].reshape(arr.shape)
    v[...] = arr
    return v


@pytest.mark.parametrize("offset", [0, 1])
def test_pinned_batches_equal_ordinary_arrays(ctx, tmp_path, offset):
    cases.config_potential(ctx, 2, tmp_path)
    offs, posn, types, cell = pack_batch(cases.small_binary(n_struc=5, seed=4))
    E0, F0, W0 = ctx.compute(offs, posn, types, cell, precision=FP64)
    h_posn, h_types, h_cell = _pinned_view(ctx, posn, offset), _pinned_view(ctx, types, offset), _pinned_view(ctx, cell, offset)
    S, N = len(offs) - 1, int(offs[-1])
    out = (_pinned_view(ctx, np.zeros(S), offset), _pinned_view(ctx, np.zeros((N, 3)), offset),
           _pinned_view(ctx, np.zeros((S, 3, 3)), offset))
    nb0 = ctx.neighbors(with_vectors=True)

    def check():
        E1, F1, W1 = ctx.compute(offs, h_posn, h_types, h_cell, precision=FP64, out=out)
        for x, y in zip(ctx.neighbors(with_vectors=True), nb0):
            assert np.array_equal(x, y), "inputs changed in transfer"
        Ed, Fd, Wd = ctx.download()
        assert np.array_equal(E1, Ed) and np.array_equal(F1, Fd) and np.array_equal(W1, Wd), "results changed in transfer"
        assert np.array_equal(E1, E0)
        assert np.abs(F1 - F0).max() <= 1e-12 * np.abs(F0).max() and np.abs(W1 - W0).max() <= 1e-12 * np.abs(W0).max()

    check()
    check()   # the second call repeats the staged offsets (tables kept on the device)
    # the same buffers again after a different batch
    offs2, posn2, types2, cell2 = pack_batch(cases.small_binary(n_struc=5, seed=9))
    ctx.compute(offs2, posn2, types2, cell2, precision=MIXED)
    check()
