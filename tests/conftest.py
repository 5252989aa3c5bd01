import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_NAME = "simferrofluid-cuda_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built CUDA library")


def pkg():
    return importlib.import_module(PKG_NAME)


def scenes():
    return importlib.import_module(PKG_NAME + ".scenes")


@pytest.fixture(scope="session")
def sfpkg():
    return pkg()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_ctx(sfpkg):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    sfpkg.load_library()
    ctx = sfpkg.Context(0)
    yield ctx
    ctx.close()


def oracle_grid(O, g):
    return O.Grid(*g.shape, g.spacing, tuple(g.origin))


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
