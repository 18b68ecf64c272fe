import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("labinius-fast-challenge_gb300", "oracle"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: full-size (2^31-bit) cases")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The prover library built for sm_103a; fails loudly when it cannot be built or loaded."""
    import build as lfbuild
    import lfgpu

    lfbuild.build()
    return lfgpu


@pytest.fixture(scope="session")
def prover(gpu_lib):
    p = gpu_lib.Prover(0)
    yield p
    p.close()
