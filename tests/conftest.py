"""Shared test set-up: the `gpu` marker, repository paths, and helpers.

GPU tests (`-m gpu`) call the CUDA path through the C ABI of libplbm.so and compare with the
CPU oracle in oracle/; CPU tests (`-m "not gpu"`) check the oracle against golden vectors, the
host logic, and that the library loads and exports the declared symbols.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def plbm():
    from portlbm_gb300 import build as b
    b.build()
    import portlbm_gb300
    portlbm_gb300.load_library()
    return portlbm_gb300


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import plbm_oracle
    plbm_oracle.build()
    return plbm_oracle
