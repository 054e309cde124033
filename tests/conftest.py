import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "tnl-mhfem_gb300"
for p in (str(PKG), str(REPO)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Builds the CUDA library and the oracle once per session (incremental)."""
    sys.path.insert(0, str(PKG))
    import build as _build

    _build.build_oracle()
    if os.environ.get("MHFEM_SKIP_LIB_BUILD") != "1":
        _build.build_library()
    yield
