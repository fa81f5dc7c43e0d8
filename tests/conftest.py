"""pytest setup: repo root on sys.path, the `gpu` marker, shared builders."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libubr.so")


@pytest.fixture(scope="session")
def oracle_lib():
    from umbreon_gb300 import build
    build.build_oracle()
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx():
    """One ubr_context on GPU 0; fails loudly when the CUDA library is absent."""
    from umbreon_gb300 import build
    from umbreon_gb300.abi import lib_path
    if not lib_path().exists():
        build.build_ubr()
    from umbreon_gb300.api import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
