"""include/ann_nnp.hpp (the C++ adapter with the reference's call shapes): it compiles against the
C ABI, reports a missing device as an exception, and computes what the Python binding computes."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import cases

ROOT = Path(__file__).resolve().parents[1]


def _build(tmp_path):
    from ann_gb300.api import library_path
    lib = library_path()
    if not lib.exists():
        pytest.skip("libann_gpu.so not built")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "adapter_main"
    cmd = [cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(ROOT / "tests" / "adapter" / "adapter_main.cpp"),
           "-o", str(exe), str(lib), f"-Wl,-rpath,{lib.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_adapter_reports_missing_device(tmp_path):
    exe = _build(tmp_path)
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
