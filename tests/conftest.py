import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

REFERENCE = os.environ.get("PRGPU_REFERENCE", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libprgpu.so)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def lib_built():
    from poissonrecon_gpu_gb300 import builder
    builder.build()
    return builder.LIB


def reference_file(name):
    p = os.path.join(REFERENCE, name)
    return p if os.path.exists(p) else None


def sphere(n, seed=0, radius=0.35):
    from poissonrecon_gpu_gb300 import shapes
    return shapes.sphere(n, radius=radius, seed=seed)
