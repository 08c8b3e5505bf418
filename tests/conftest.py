"""Shared test setup: import paths, the ``gpu`` marker, library builds."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "regularized-drot_gb300")
for path in (REPO, PKG):
    if path not in sys.path:
        sys.path.insert(0, path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def solver_lib():
    """Build (if stale) and load libdrot_gb300.so."""
    import build as solver_build  # regularized-drot_gb300/build.py
    solver_build.build()
    from reg_drot import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
