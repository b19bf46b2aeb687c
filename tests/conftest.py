import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "helm-project_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    from oracle import build as obuild
    obuild.build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def reflib():
    from oracle import RefLib
    from oracle import build as obuild
    path = obuild.build_ref()
    if path is None:
        pytest.skip("reference checkout not present: reference-header library not built")
    return RefLib(path)


@pytest.fixture(scope="session")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import axgb
    axgb.init(0)
    return axgb
