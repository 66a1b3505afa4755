import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs librtcore.so on the device)")
    config.addinivalue_line("markers", "slow: large CPU case")


def cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle

    return oracle.load()


@pytest.fixture(scope="session")
def rtlib():
    from rtgallery import abi, build

    build.build()
    return abi.load_library()


@pytest.fixture(scope="session")
def device(rtlib):
    if not cuda_available():
        pytest.skip("no CUDA device")
    from rtgallery import host

    d = host.Device()
    yield d
    d.close()
