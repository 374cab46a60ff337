import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the libflygpu C ABI)")


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure), built on first use."""
    from oracle import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def table_path():
    from openfly_gb300 import workloads

    return workloads.TABLE


@pytest.fixture(scope="session")
def odata(oracle, table_path):
    return oracle.EAMData(table_path)


@pytest.fixture(scope="session")
def fly():
    """libflygpu through its C ABI; built in-tree if missing. Fails loudly without it."""
    from openfly_gb300 import build

    build.build()
    import openfly_gb300

    openfly_gb300.lib()
    return openfly_gb300


@pytest.fixture(scope="session")
def gpu(fly):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("a -m gpu test ran without a visible CUDA device")
    return fly


@pytest.fixture(scope="session")
def geam(gpu, table_path):
    return gpu.EAM(table_path)
