import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    from oracle_lib import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library (builds it if missing); GPU tests fail loudly without it."""
    from ann_gb300 import build_library, load_library, library_path
    if not library_path().exists():
        build_library()
    return load_library()
