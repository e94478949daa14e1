import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and runs the library's kernels")
    config.addinivalue_line("markers", "slow: larger CPU oracle cases")


@pytest.fixture(scope="session")
def pkg():
    import importlib
    return importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300")


@pytest.fixture(scope="session")
def dev(pkg):
    import importlib
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from importlib import import_module
    build = import_module("arap-deformation-of-gaussian-radiance-fields_gb300.build")
    build.build()
    return import_module("arap-deformation-of-gaussian-radiance-fields_gb300.deform")
