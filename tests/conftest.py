import importlib
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (the GB300 parity tests)")


def _ensure_native():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "lsg_build_native", os.path.join(REPO, "lattice-symmetries_gb300", "build_native.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


_ensure_native()


@pytest.fixture(scope="session")
def ls():
    return importlib.import_module("lattice-symmetries_gb300")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def goldens():
    import json
    with open(os.path.join(REPO, "tests", "golden", "reference_goldens.json"), encoding="utf-8") as f:
        return json.load(f)


@pytest.fixture(scope="session")
def ref_kernels():
    import numpy as np
    return dict(np.load(os.path.join(REPO, "tests", "golden", "reference_kernels.npz")))


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
