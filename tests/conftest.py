import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "paper-rsf-vesselseg_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    from oracle import rsf_oracle

    rsf_oracle.build()
    return rsf_oracle


@pytest.fixture(scope="session")
def rsflib():
    import __graft_entry__  # noqa: F401
    from rsf_gb300 import _lib, build

    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def ws_big(cuda, rsflib):
    from rsf_gb300 import Workspace

    ws = Workspace(20_000_000, 64)
    yield ws
    ws.close()
