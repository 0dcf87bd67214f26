import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402

entry.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_100 family) and the built library")


@pytest.fixture(scope="session")
def st():
    return entry.load_package()


@pytest.fixture(scope="session")
def abi():
    import stencils_gb300._abi as A
    return A


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def goldens():
    d = json.loads((ROOT / "tests" / "golden" / "reference_goldens.json").read_text())
    return d["entries"]


@pytest.fixture(scope="session")
def lib():
    """The built library (compiled here if missing; nvcc cross-compiles without a GPU)."""
    from stencils_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from stencils_gb300 import _lib, build
    build.build()
    _lib.load()
    return torch
