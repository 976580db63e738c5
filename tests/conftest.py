"""pytest configuration: markers, build fixtures and shared helpers.

`-m "not gpu"` runs the oracle checks, host logic and C-ABI export checks on
CPU; `-m gpu` runs the parity tests of the CUDA path against the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: large inputs (minutes on CPU)")


@pytest.fixture(scope="session")
def oracle_built():
    from oracle.build import build_oracle
    return build_oracle()


@pytest.fixture(scope="session")
def lib_built():
    from morpheus_gb300.build import build_library
    return build_library()


@pytest.fixture(scope="session")
def cuda(lib_built):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    torch.cuda.init()
    return torch.device("cuda:0")
