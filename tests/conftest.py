import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

ORACLE_SO = ROOT / "oracle" / "_build" / "libgomoracle.so"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_so():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    return ORACLE_SO


@pytest.fixture(scope="session")
def core_so():
    from gom_release_gb300.build import build_core
    return build_core()


@pytest.fixture(scope="session")
def gpu_lib(core_so):
    from gom_release_gb300.core import load_core
    return load_core()
