import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "hpc-multigpu-matrixmult_gb300"
for p in (PKG, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 (GB300) GPU; runs through the CUDA C ABI")


@pytest.fixture(scope="session")
def built():
    """Builds the library, host programs and oracle once per session (no GPU needed)."""
    import build as pkg_build  # hpc-multigpu-matrixmult_gb300/build.py

    pkg_build.build_all()
    return True


@pytest.fixture(scope="session")
def phpc(built):
    import phpc as mod  # hpc-multigpu-matrixmult_gb300/phpc.py

    return mod


@pytest.fixture(scope="session")
def oracle(built):
    import oracle_py

    return oracle_py


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch
