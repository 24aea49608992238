"""CPU tests of the host side: the C ABI library loads and exports every symbol include/ann_gpu.h
declares (no compute call without a GPU), fails cleanly with no device, the synthetic
workloads have their stated shapes, the pure-Python network initialisation reproduces
std::mt19937 + std::normal_distribution, and the multi-rank sharding covers every structure
once (two gloo ranks)."""
import os
import re
import subprocess
import textwrap
from pathlib import Path

import numpy as np
import pytest

from ann_gb300 import workloads as W
from ann_gb300.api import ABI_SYMBOLS, AnnError, load_library, pack_batch
from ann_gb300.parallel import dist_block, shard_by_atoms, subset

ROOT = Path(__file__).resolve().parents[1]


def _header_functions():
    text = (ROOT / "include" / "ann_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ann_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from ann_gb300 import build_library, library_path
    if not library_path().exists():
        build_library()
    return load_library()


def test_library_exports_every_declared_symbol(lib):
    declared = _header_functions()
    assert len(declared) > 30
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(ABI_SYMBOLS), set(declared) ^ set(ABI_SYMBOLS)
    assert lib.ann_abi_version() == 4


def test_no_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ann_gb300 import Context
    with pytest.raises(AnnError) as e:
        Context()
    assert e.value.code == 4   # ANN_ERR_CUDA, no exception crossed the C boundary


def test_workload_shapes():
    s1 = W.config1()
    assert len(s1) == 1 and len(s1[0][1]) == 108
    s2 = W.config2(nstruc=8)
    for x, t, R in s2:
        n = len(t)
        assert 32 <= n <= 512 and (t == 0).sum() == n // 2
        L = R[0, 0]
        assert abs(n / L ** 3 - 0.05) < 1e-9
        d = x[:, None] - x[None]
        d -= L * np.round(d / L)
        dd = np.sqrt((d ** 2).sum(-1)) + np.eye(n) * 99
        assert dd.min() >= 1.8
    x4, t4, R4 = W.config4(dims=(4, 4, 2))[0]
    assert len(t4) == 32 and (t4 == 2).sum() == 16
    x5, v5, t5, R5 = W.config5(cells=(2, 2, 2))
    assert len(t5) == 32 and np.abs(v5.mean(0)).max() < 1e-12


def test_potential_texts_parse(oracle):
    for cfg, nin in ((1, 16), (2, 72), (4, 96), (5, 16)):
        pot = oracle.load_text(W.config_potential_text(cfg))
        assert pot.ninput(0) == nin


def test_python_init_matches_libstdcxx(tmp_path):
    src = tmp_path / "n.cpp"
    src.write_text(textwrap.dedent("""
        #include <random>
        #include <cstdio>
        int main(){ std::mt19937 g(20261205);
          for (int l = 0; l < 3; ++l) { std::normal_distribution<double> d(0.0, 0.1 * (l + 1));
            for (int i = 0; i < 7; ++i) std::printf("%.17g\\n", d(g)); } }"""))
    exe = tmp_path / "n"
    subprocess.run(["g++", "-O2", "-o", str(exe), str(src)], check=True)
    want = np.array([float(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()])
    g = W._StdMT19937Normal(20261205)
    got = []
    for l in range(3):
        g.reset()
        got += [g.normal(0.1 * (l + 1)) for _ in range(7)]
    assert np.array_equal(np.array(got), want)


def test_dist_and_atom_shards():
    for n, world in ((10, 3), (256, 8), (5, 8)):
        covered = []
        for r in range(world):
            lo, hi = dist_block(n, r, world)
            covered += list(range(lo, hi))
        assert covered == list(range(n))
    offs, posn, types, cell = pack_batch(W.config2(nstruc=32))
    for world in (2, 3, 4):
        parts = [shard_by_atoms(offs, r, world) for r in range(world)]
        assert parts[0][0] == 0 and parts[-1][1] == 32
        assert all(parts[k][1] == parts[k + 1][0] for k in range(world - 1))
        atoms = [offs[hi] - offs[lo] for lo, hi in parts]
        assert max(atoms) - min(atoms) <= 2 * 512
        o, x, t, c = subset(offs, posn, types, cell, *parts[-1])
        assert o[0] == 0 and o[-1] == len(t) == len(x) and len(c) == len(o) - 1


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    offs, posn, types, cell = pack_batch(W.config2(nstruc=24))
    lo, hi = shard_by_atoms(offs, rank, world)
    mine = torch.zeros(24, dtype=torch.int64)
    mine[lo:hi] = 1
    dist.all_reduce(mine)
    t = torch.tensor([float(offs[hi] - offs[lo])])
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    q.put((rank, mine.tolist(), float(t), float(tmax)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_sharding():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mine, t, tmax in out:
        assert mine == [1] * 24          # every structure owned by exactly one rank
        assert tmax >= t


def test_xyz_round_trip_and_wrapping(tmp_path):
    """Extended XYZ as XYZ::read / XYZ::write (format/xyz_struc.cpp): properties, energy, lattice
    columns, forces, wrapping into the cell, and the batch packing by type names."""
    from ann_gb300.io import XYZStructure, batch_from_xyz, read_xyz, write_xyz
    rng = np.random.default_rng(2)
    R = np.array([[5.0, 1.0, 0.5], [0.0, 6.0, 0.7], [0.0, 0.0, 7.0]])     # columns = lattice vectors
    x = rng.uniform(-3.0, 12.0, (5, 3))
    f = rng.normal(size=(5, 3))
    s = XYZStructure(["Ar", "Ne", "Ar", "Ar", "Ne"], x, R, -12.345678, f)
    write_xyz(tmp_path / "a.xyz", s)
    r = read_xyz(tmp_path / "a.xyz")
    assert r.names == s.names and abs(r.energy - s.energy) < 1e-6
    assert np.allclose(r.cell, R, atol=1e-6) and np.allclose(r.forces, f, atol=1e-9)
    frac = np.linalg.solve(R, r.posn.T).T
    assert np.all(frac >= 0) and np.all(frac < 1)
    d = np.linalg.solve(R, (r.posn - x).T).T                            # wrapped by whole cell vectors
    assert np.allclose(d, np.round(d), atol=1e-6)
    # header tags in any case, extra columns, no forces
    (tmp_path / "b.xyz").write_text('2\nlattice="4 0 0 0 4 0 0 0 4" properties=species:S:1:pos:R:3:Z:I:1 Potential_Energy=-1.5\n'
                                    "Ar 0.5 0.5 0.5 18\nAr 4.5 1.0 1.0 18\n")
    b = read_xyz(tmp_path / "b.xyz")
    assert b.forces is None and b.energy == -1.5 and np.allclose(b.posn[1], [0.5, 1.0, 1.0])

    class Names:
        def type_index(self, n):
            return {"Ar": 0, "Ne": 1}[n]
    offs, posn, types, cell = batch_from_xyz(Names(), [r, b])
    assert list(offs) == [0, 5, 7] and list(types) == [0, 1, 0, 0, 1, 0, 0]
    assert np.allclose(cell[0].reshape(3, 3).T, R, atol=1e-6)


def test_split_position_pair_vectors():
    """The mixed caller-list rows' pair vectors (csrc/extlist.cu): positions split into FP32 hi and
    lo parts, r = (hi_i - hi_j) + (lo_i - lo_j) in FP32 arithmetic. For entries within 8 A every
    component lies within 5e-7 A of the exact difference at coordinates up to 2e7 A (the FP64
    difference rounded to FP32 is within 2.4e-7 A), and within one FP32 ulp of |r| at coordinates
    up to 1000 A; FP32 positions alone are off by up to half an ulp of the coordinate."""
    rng = np.random.default_rng(8)

    def split(x):
        h = x.astype(np.float32)
        return h, (x - h.astype(np.float64)).astype(np.float32)

    for L in (10.0, 400.0, 1000.0, 2.0e4, 2.0e7):
        xi = rng.uniform(-0.2, 1.2, 200_000) * L
        xj = xi - rng.uniform(-8.0, 8.0, len(xi))
        exact = xi - xj
        hi, li = split(xi)
        hj, lj = split(xj)
        r = (hi - hj) + (li - lj)                  # FP32 operations, each rounded
        assert r.dtype == np.float32
        err = np.abs(r.astype(np.float64) - exact)
        assert err.max() <= 5e-7, L
        if L <= 1000.0:
            assert np.all(err <= np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)), L
        naive = (xi.astype(np.float32) - xj.astype(np.float32)).astype(np.float64)
        if L >= 400.0:
            assert np.abs(naive - exact).max() > 10 * err.max(), L
