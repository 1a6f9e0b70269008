"""pytest configuration: the ``gpu`` marker and import paths.

``-m "not gpu"`` runs the oracle checks, the golden-vector checks, the host
logic and the C-ABI export checks; ``-m gpu`` runs the parity tests, which
call libfrgpu.so through its C ABI on a GB300 and compare with the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "fluxreconstruction.jl_gb300", "oracle"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libfrgpu.so")


def _has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def has_gpu():
    return _has_gpu()


@pytest.fixture(scope="session")
def frgpu():
    import frgpu as F

    F.lib()
    return F


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.lib()
    return O
