"""The timeout path of the bounded device waits, driven without a fault or a hang.

ann_set_wait_limit(0) makes every device wait (the staged neighbour rows of the symmetry-function,
force and tangent passes, the network weight image and the MMA completions of the tensor-core
kernel) give up without polling. The kernel then records the timeout, lets its copies finish
(with the full bound) and returns. The call must report ANN_ERR_TIMEOUT; after
ann_set_wait_limit(-1) the same context must give the oracle's results again.
"""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, AnnError, Context

pytestmark = pytest.mark.gpu

ANN_ERR_TIMEOUT = 7


def _rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("precision,backend", [(FP64, 0), (MIXED, 2), (MIXED, 1)], ids=["fp64", "mixed_tensor_cores", "mixed_simt"])
def test_wait_limit_times_out_then_recovers(gpu_lib, oracle, tmp_path, precision, backend):
    ctx = Context(mlp_backend=backend)
    try:
        structs = cases.small_binary(n_struc=4, seed=31)
        offs, posn, types, cell = cases.batch(structs)
        text = cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
        Eo, Fo, Wo, _, _ = oracle.load_text(text).compute(offs, posn, types, cell)
        ctx.compute(offs, posn, types, cell, precision=precision)       # graphs captured with the built-in bounds
        for _ in range(2):
            ctx.set_wait_limit(0)
            with pytest.raises(AnnError) as err:
                ctx.compute(offs, posn, types, cell, precision=precision)
            assert err.value.code == ANN_ERR_TIMEOUT
            ctx.set_wait_limit(-1)
            E, F, W = ctx.compute(offs, posn, types, cell, precision=precision)
            if precision == FP64:
                assert _rel_err(E, Eo) < 1e-10 and _rel_err(F, Fo) < 1e-10 and _rel_err(W, Wo) < 1e-10
            else:
                assert np.max(np.abs(E - Eo) / np.diff(offs)) * 1e3 < 1.0
                assert np.max(np.abs(F - Fo)) * 1e3 < 10.0
    finally:
        ctx.close()


def test_network_image_wait_times_out_alone(gpu_lib, tmp_path):
    """The tensor-core kernel on its own (the no-allocation network pass): its weight-image wait
    gives up, TMEM is freed, and the next call with the built-in bound matches ann_compute."""
    torch = pytest.importorskip("torch")
    ctx = Context(mlp_backend=2)
    try:
        structs = cases.small_binary(n_struc=4, seed=32)
        offs, posn, types, cell = cases.batch(structs)
        cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
        ctx.compute(offs, posn, types, cell, precision=MIXED)
        G, e_ref = ctx.symm(), ctx.atom_energies()
        n, width = G.shape
        dev = torch.device("cuda:0")
        t_d = torch.from_numpy(types.astype(np.int32)).to(dev)
        G_d = torch.from_numpy(G).to(dev, torch.float32).contiguous()
        E_d = torch.zeros(n, dtype=torch.float64, device=dev)
        D_d = torch.zeros((n, width), dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        ctx.set_wait_limit(0)
        with pytest.raises(AnnError) as err:
            ctx.network_noalloc(n, t_d.data_ptr(), G_d.data_ptr(), E_d.data_ptr(), D_d.data_ptr(), MIXED)
        assert err.value.code == ANN_ERR_TIMEOUT
        ctx.set_wait_limit(-1)
        ctx.network_noalloc(n, t_d.data_ptr(), G_d.data_ptr(), E_d.data_ptr(), D_d.data_ptr(), MIXED)
        assert np.max(np.abs(E_d.cpu().numpy() - e_ref)) < 1e-5
    finally:
        ctx.close()


def test_wait_limit_validated(gpu_lib):
    ctx = Context()
    try:
        with pytest.raises(AnnError):
            ctx.set_wait_limit(-2)
    finally:
        ctx.close()
