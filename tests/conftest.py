import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the kernels through the C-ABI)")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    """Builds libqsi_ed.so (and the oracle) in-tree once per session."""
    from qsi_subspace_ed_gb300._build import build
    from oracle import oracle as O

    build()
    O.build_port()
    return True
