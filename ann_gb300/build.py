"""Build recipe of libann_gpu.so (the GB300 library) for sm_103a.

Compiles every translation unit under ann_gb300/csrc in parallel with nvcc and links them into
ann_gb300/libann_gpu.so (in-tree, git-ignored). Re-runs only what changed (mtime of the unit
and of the headers). Usable as `python -m ann_gb300.build`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
OBJ = HERE / "_build"
LIB = HERE / "libann_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code is compiled without floating-point contraction so that x86-64 and aarch64 hosts give
# the same bits (the std::mt19937 / normal_distribution network initialisation and the plans)
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
         "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unused-function", "-diag-suppress", "177,550"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libann_gpu.so")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _compile(nvcc: str, src: Path, verbose_ptxas: bool) -> Path:
    obj = OBJ / (src.name + ".o")
    newest_dep = max([src.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if obj.exists() and obj.stat().st_mtime >= newest_dep and not verbose_ptxas:
        return obj
    cmd = [nvcc, *ARCH, *FLAGS, "-I", str(CSRC), "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    if verbose_ptxas and src.suffix == ".cu":
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas:
        sys.stderr.write(res.stderr)
    return obj


def build(verbose_ptxas: bool = False, jobs: int | None = None) -> Path:
    """Compile and link libann_gpu.so; returns its path."""
    nvcc = _nvcc()
    OBJ.mkdir(exist_ok=True)
    stamp = OBJ / "flags.txt"   # a change of compiler or flags invalidates every object
    key = " ".join([nvcc, *ARCH, *FLAGS])
    if not stamp.exists() or stamp.read_text() != key:
        for o in OBJ.glob("*.o"):
            o.unlink()
        stamp.write_text(key)
    srcs = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, verbose_ptxas), srcs))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
