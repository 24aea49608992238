"""ann_network_noalloc (the network stage on device-resident symmetry functions, with its scratch
in a static device array) against the existing entry point, ann_compute, through the C ABI.

The entry point exists for callers that cannot allocate device memory during a step (an MD engine
or plugin host that reserves its memory up front). So besides the results, the test checks that a
call allocates nothing: the device's free memory (cudaMemGetInfo) and torch's allocator counters
are the same before and after the second call. Each precision and network backend (tensor cores
and the SIMT kernel for MIXED, the FP64 kernel) is checked on two calls in a row (the second
reuses the shared scratch): atom energies and dE/dG equal ann_compute's to 1e-12 relative for
FP64 and 1e-5 eV / 1e-5 relative for MIXED (the same network kernels on the same inputs). A call
with no atoms does nothing and succeeds.
"""
import numpy as np
import pytest

import cases
from ann_gb300 import FP64, MIXED, AnnError, Context

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", params=[0, 1], ids=["default_backend", "simt_backend"])
def ctx(request, gpu_lib):
    c = Context(mlp_backend=request.param)
    yield c
    c.close()


def _reference(ctx, tmp_path, precision):
    structs = cases.small_binary(n_struc=5, seed=29)
    offs, posn, types, cell = cases.batch(structs)
    cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    ctx.compute(offs, posn, types, cell, precision=precision)
    return types, ctx.symm(), ctx.atom_energies(), ctx.dedg()


def _allocator_counts():
    s = torch.cuda.memory_stats()
    return s.get("allocation.all.allocated", 0), s.get("segment.all.allocated", 0)


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_matches_ann_compute_twice(ctx, tmp_path, precision):
    types, G, e_ref, d_ref = _reference(ctx, tmp_path, precision)
    n, width = G.shape
    dt = torch.float64 if precision == FP64 else torch.float32
    dev = torch.device("cuda:0")
    t_d = torch.from_numpy(types.astype(np.int32)).to(dev)
    G_d = torch.from_numpy(G).to(dev, dt).contiguous()
    torch.cuda.synchronize()
    for call in range(2):
        E_d = torch.full((n,), np.nan, dtype=torch.float64, device=dev)
        D_d = torch.full((n, width), np.nan, dtype=dt, device=dev)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info(dev)
        counts0 = _allocator_counts()
        ctx.network_noalloc(n, t_d.data_ptr(), G_d.data_ptr(), E_d.data_ptr(), D_d.data_ptr(), precision)
        free1, _ = torch.cuda.mem_get_info(dev)
        counts1 = _allocator_counts()
        if call == 1:   # the first call may load the library's device code (lazy module loading)
            assert free1 == free0, f"device free memory changed by {free0 - free1} B across the call"
            assert counts1 == counts0
        e = E_d.cpu().numpy()
        d = D_d.to(torch.float64).cpu().numpy()
        if precision == FP64:
            assert np.max(np.abs(e - e_ref)) <= 1e-12 * np.max(np.abs(e_ref))
            assert np.max(np.abs(d - d_ref)) <= 1e-12 * np.max(np.abs(d_ref))
        else:
            assert np.max(np.abs(e - e_ref)) < 1e-5
            assert np.max(np.abs(d - d_ref)) <= 1e-5 * np.max(np.abs(d_ref))


def test_no_atoms_is_a_no_op(ctx, tmp_path):
    cases.config_potential(ctx, 2, tmp_path)
    for precision in (FP64, MIXED):
        ctx.network_noalloc(0, None, None, None, None, precision)


def test_rejects_more_atoms_than_the_scratch_holds(ctx, tmp_path):
    cases.config_potential(ctx, 2, tmp_path)
    too_many = 262144 + 1
    with pytest.raises(AnnError, match="at most 262144 atoms"):
        ctx.network_noalloc(too_many, None, None, None, None, MIXED)
    with pytest.raises(AnnError):
        ctx.network_noalloc(4, None, None, None, None, MIXED)
