import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle (and the CUDA library, which cross-compiles without
    a GPU) once per session."""
    from tpls_gb300 import build
    build.build_oracle()
    build.build_cuda()
    from oracle.oracle import set_threads
    set_threads(int(os.environ.get("TPLS_ORACLE_THREADS", "1")))
    yield
