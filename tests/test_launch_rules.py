"""Host-side launch rules, compiled from the library's own header with the host compiler (no GPU):
the tensor-core network kernel's warp split per launch (tc_groups, mlp_tc.hpp)."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "ann_gb300" / "csrc"
CUDA_INC = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"

PROGRAM = r'''
#include "mlp_tc.hpp"
#include <cstdio>
#include <cstdlib>
int main(int argc, char** argv) {
    ann::TcType t{};
    t.tmem_cols = std::atoi(argv[1]);
    std::printf("%d\n", ann::tc_groups(t, std::atoll(argv[2]), std::atoi(argv[3])));
    return 0;
}
'''


@pytest.fixture(scope="module")
def rule(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None or not (CUDA_INC / "cuda_runtime.h").exists():
        pytest.skip("host compiler or CUDA headers not available")
    d = tmp_path_factory.mktemp("rule")
    src, exe = d / "rule.cpp", d / "rule"
    src.write_text(PROGRAM)
    subprocess.run([cxx, "-std=c++17", "-I", str(CSRC), "-I", str(CUDA_INC), str(src), "-o", str(exe)], check=True)
    return lambda cols, atoms, nsm=152: int(subprocess.run([str(exe), str(cols), str(atoms), str(nsm)], check=True,
                                                           capture_output=True, text=True).stdout)


@pytest.mark.parametrize("cols,atoms,want", [
    (128, 262144, 1),     # MD box, 16-32-32-1: 2,048 tiles, tensor memory for four CTAs per SM
    (32, 262144, 1),      # narrower still: four CTAs per SM is the register limit
    (256, 37355, 4),      # one type of the 74,710-atom binary batch: ~292 tiles, one CTA per SM
    (256, 100000, 2),     # tensor memory for two CTAs and tiles enough for two each
    (128, 100000, 2),     # room for four CTAs, tiles enough only for two
    (512, 10 ** 6, 4),    # a CTA takes all of tensor memory
    (128, 1, 4),          # a single tile
])
def test_network_warp_split(rule, cols, atoms, want):
    assert rule(cols, atoms) == want


def test_split_never_exceeds_tensor_memory(rule):
    for cols in (32, 64, 128, 256, 512):
        for atoms in (1, 1000, 50000, 300000, 5 * 10 ** 6):
            g = rule(cols, atoms)
            assert g in (1, 2, 4)
            assert (4 // g) * cols <= 512 or g == 4    # CTAs per SM x columns within 512


LAYOUT = r'''
#include <cstddef>
#include <cstdio>
#include "ann_gpu.h"
#define F(T, m) std::printf(#T " " #m " %zu\n", offsetof(T, m))
int main() {
    std::printf("ann_options size %zu\n", sizeof(ann_options));
    F(ann_options, device); F(ann_options, precision); F(ann_options, newton); F(ann_options, max_neighbors);
    F(ann_options, use_graphs); F(ann_options, mlp_backend); F(ann_options, tc_groups); F(ann_options, tc_split);
    std::printf("ann_tuning size %zu\n", sizeof(ann_tuning));
    F(ann_tuning, tc_groups); F(ann_tuning, bp_blocks_per_sm); F(ann_tuning, nbr_blocks_per_sm);
    F(ann_tuning, ms); F(ann_tuning, ms_default);
    return 0;
}
'''


def test_ctypes_structs_match_the_header(tmp_path):
    """ann_options and ann_tuning as the ctypes binding declares them have the C header's layout."""
    import ctypes as C
    from ann_gb300.api import Options, Tuning
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host compiler")
    src, exe = tmp_path / "layout.cpp", tmp_path / "layout"
    src.write_text(LAYOUT)
    subprocess.run([cxx, "-std=c++17", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        a, b, v = ln.split()
        got[(a, b)] = int(v)
    for cls, name in ((Options, "ann_options"), (Tuning, "ann_tuning")):
        assert got[(name, "size")] == C.sizeof(cls), name
        for field, _ in cls._fields_:
            assert got[(name, field)] == getattr(cls, field).offset, (name, field)
