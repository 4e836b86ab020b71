import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle.bind import REF_ROOT  # noqa: E402  (the reference checkout, NURAY_REF_ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libnuray_gpu.so")


@pytest.fixture(scope="session")
def port_lib():
    from oracle import bind
    return bind.build_port()


@pytest.fixture(scope="session")
def ref_lib():
    """The reference compiled from source; skipped where the checkout is absent."""
    from oracle import bind
    if os.path.exists(bind.REF_LIB):
        return bind.REF_LIB
    path = bind.build_ref()
    if path is None:
        pytest.skip("reference sources not present on this machine")
    return path


@pytest.fixture(scope="session")
def gpu_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nuray_gb300 import build
    build.build()
    from nuray_gb300 import lib
    return lib()


def golden(name):
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", name), allow_pickle=False))
