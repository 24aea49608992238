"""include/ann_nnp.hpp (the C++ adapter with the reference's call shapes) and include/ann_pair_nn.hpp
(the LAMMPS pair style shape): they compile against the C ABI, report a missing device as an
exception, and compute what the Python binding computes."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import cases

ROOT = Path(__file__).resolve().parents[1]


def _build(tmp_path, program="adapter_main"):
    from ann_gb300.api import library_path
    lib = library_path()
    if not lib.exists():
        pytest.skip("libann_gpu.so not built")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / program
    cmd = [cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(ROOT / "tests" / "adapter" / f"{program}.cpp"),
           "-o", str(exe), str(lib), f"-Wl,-rpath,{lib.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("program", ["adapter_main", "pair_main"])
def test_adapter_reports_missing_device(tmp_path, program):
    exe = _build(tmp_path, program)
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([str(exe), "x", "x", "nodevice"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("error: libann_gpu:"), r.stdout + r.stderr


@pytest.mark.gpu
def test_adapter_matches_python_binding(tmp_path, gpu_lib):
    from ann_gb300 import FP64, Context
    exe = _build(tmp_path)
    ctx = Context()
    text = cases.config_potential(ctx, 1, tmp_path)
    (tmp_path / "pot.ann").write_text(text)
    x, t, R = cases.W.config1()[0]
    lines = [str(len(t)), " ".join(f"{v:.17g}" for v in R.T.reshape(9))]
    lines += [f"{int(ti)} {xi[0]:.17g} {xi[1]:.17g} {xi[2]:.17g}" for ti, xi in zip(t, x)]
    (tmp_path / "s.txt").write_text("\n".join(lines) + "\n")
    r = subprocess.run([str(exe), str(tmp_path / "pot.ann"), str(tmp_path / "s.txt"), "compute"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    out = r.stdout.split("\n")
    e = float(out[0])
    F = np.array([[float(v) for v in ln.split()] for ln in out[1:1 + len(t)]])
    e2, pe = (float(v) for v in out[1 + len(t)].split())
    offs, posn, types, cell = cases.batch([(x, t, R)])
    E, Fp, _ = ctx.compute(offs, posn, types, cell, precision=FP64)
    assert abs(e - E[0]) <= 1e-10 * abs(E[0]) and abs(e2 - E[0]) <= 1e-10 * abs(E[0]) and pe == e2
    assert np.abs(F - Fp).max() <= 1e-10 * np.abs(Fp).max()
    ctx.close()


@pytest.mark.gpu
def test_pair_style_adapter_matches_list_call(tmp_path, gpu_lib):
    """PairNN on LAMMPS-shaped arrays: 1-based types mapped through pair_coeff's element names (the
    potential's order reversed, plus a NULL type), special-bond bits in the neighbour indices, an
    atom of the NULL type inside a row, forces added to f. The result is the list call's on the
    same domain without the NULL atom."""
    from ann_gb300 import FP64, Context
    from lmp_domain import build_domain
    exe = _build(tmp_path, "pair_main")
    ctx = Context()
    structs = cases.small_binary(n_struc=1, seed=17)
    offs, posn, types, cell = cases.batch(structs)
    text = cases.config_potential(ctx, 2, tmp_path, precondition_batch=(offs, posn, types, cell))
    (tmp_path / "pot.ann").write_text(text)
    x, t, R = structs[0]
    dom = build_domain(x, t, R, ctx.rc + 1.0, seed=6)
    E, F, Wv, ea = ctx.compute_list(dom.x, dom.type, dom.numneigh, dom.neigh, eatom=True, precision=FP64)
    names = [ctx.type_name(k) for k in range(2)]
    elements = [names[1], names[0], "NULL"]                 # LAMMPS type 1 -> potential type 1, ...
    lmp_type = np.where(dom.type == 1, 1, 2)
    nall = dom.nall + 1                                     # one NULL-type atom next to atom 0
    xn = np.vstack([dom.x, dom.x[0] + [0.6, 0.0, 0.0]])
    tn = np.concatenate([lmp_type, [3]])
    off = np.concatenate([[0], np.cumsum(dom.numneigh)])
    lines = [f"{nall} {dom.nlocal + 1} 3", " ".join(elements)]
    lines += [f"{int(ti)} {xi[0]:.17g} {xi[1]:.17g} {xi[2]:.17g}" for ti, xi in zip(tn, xn)]
    rng = np.random.default_rng(2)
    for i in range(dom.nlocal):
        row = [int(j) | ((1 << 30) if rng.random() < 0.3 else 0) for j in dom.neigh[off[i]:off[i + 1]]]
        if i == 0:
            row.append(nall - 1)
        lines.append(f"{i} {len(row)} " + " ".join(map(str, row)))
    lines.append(f"{nall - 1} {int(dom.numneigh[0])} " + " ".join(map(str, dom.neigh[off[0]:off[1]])))
    (tmp_path / "dom.txt").write_text("\n".join(lines) + "\n")
    r = subprocess.run([str(exe), str(tmp_path / "pot.ann"), str(tmp_path / "dom.txt"), "compute"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    out = r.stdout.split("\n")
    e, eng, rc = (float(v) for v in out[0].split())
    Fp = np.array([[float(v) for v in ln.split()] for ln in out[1:1 + nall]])
    vir = np.array([float(v) for v in out[1 + nall].split()])
    eat = np.array([float(v) for v in out[2 + nall:2 + 2 * nall]])
    assert abs(e - E) <= 1e-10 * abs(E) and eng == e and abs(rc - ctx.rc) < 1e-12
    assert np.max(np.abs(Fp[:-1] - F)) <= 1e-10 * np.max(np.abs(F)) and np.all(Fp[-1] == 0.0)
    Wref = np.array([Wv[0, 0], Wv[1, 1], Wv[2, 2], Wv[0, 1], Wv[0, 2], Wv[1, 2]])
    assert np.max(np.abs(vir - Wref)) <= 1e-10 * np.max(np.abs(Wref))
    # LAMMPS's fdotr virial (sum over local and ghost atoms of x_a f_b) is the same tensor
    fd = dom.x.T @ F
    assert np.max(np.abs(np.array([fd[0, 0], fd[1, 1], fd[2, 2], fd[0, 1], fd[0, 2], fd[1, 2]]) - Wref)) <= 1e-9 * np.max(np.abs(Wref))
    assert np.max(np.abs(eat[:dom.nlocal] - ea)) <= 1e-12 * np.max(np.abs(ea)) and np.all(eat[dom.nlocal:] == 0.0)
    e2 = float(out[2 + 2 * nall])                           # the second step, list kept on the device
    assert abs(e2 - e) <= 1e-13 * abs(e)
    ctx.close()
