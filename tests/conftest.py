import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
for p in (str(REPO), str(REPO / "gate-level-simulator_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libgls kernels)")


@pytest.fixture(scope="session")
def oracle_bin():
    from oracle import build
    return build.build_oracle()


@pytest.fixture(scope="session")
def ref_bin():
    from oracle import build
    exe = build.build_reference()
    if exe is None:
        pytest.skip("reference sources not available on this machine")
    return exe


@pytest.fixture(scope="session")
def libgls():
    from gls import build as gbuild
    from gls.capi import load_library
    if not gbuild.LIB.exists() and os.environ.get("GLS_NO_BUILD") != "1":
        gbuild.build_lib()
    return load_library()


@pytest.fixture(scope="session")
def gpu(libgls):
    from gls.capi import Simulator
    try:
        s = Simulator()
        s.close()
    except Exception as e:  # a GPU test must not pass without the CUDA path
        pytest.fail(f"CUDA device not usable by libgls: {e}")
    return True
