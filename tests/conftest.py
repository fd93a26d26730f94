import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle_nn():
    import oracle
    from owl_gb300.dense import NN

    return NN(oracle.OracleBackend())


@pytest.fixture(scope="session")
def ref_nn():
    import oracle
    from owl_gb300.dense import NN

    if not oracle.ref_available():
        pytest.skip("compiled reference stubs not available on this machine")
    return NN(oracle.RefBackend())


@pytest.fixture(scope="session")
def gpu_lib():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from owl_gb300 import _lib

    return _lib.lib()
