"""pytest set-up: markers, import paths and shared fixtures."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session")
def dc():
    """The product package (distributed-cube-average_gb300/ as dc_gb300),
    built in-tree if needed."""
    import __graft_entry__ as ge
    pkg = ge.package()
    pkg.build()
    return pkg


@pytest.fixture(scope="session")
def port():
    from oracle.oracle import Port
    return Port()


@pytest.fixture(scope="session")
def reference():
    """The reference's own sources built here; skipped where the reference
    checkout is absent (e.g. on the GPU host)."""
    from oracle.oracle import Reference
    try:
        return Reference()
    except FileNotFoundError:
        pytest.skip("reference checkout not present")
