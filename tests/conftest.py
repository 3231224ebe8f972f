"""pytest setup: the `gpu` marker, import paths, and native builds.

The CPU suite (-m "not gpu") needs the oracle and the product library built
(it loads the library to check its exports but launches nothing); both
builds are incremental and take seconds.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT), str(ROOT / "tests" / "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _native_builds():
    from opencuda_gb300 import build
    build.build_library()
    build.build_oracle()
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
