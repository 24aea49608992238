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
