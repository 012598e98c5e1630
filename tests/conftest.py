import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle"), GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle_py

    oracle_py.build()
    return oracle_py


def load_golden(name: str):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def sha(a) -> str:
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden_index(g):
    return dict(compact=g["compact"], residual=g["residual"], msb=g["msb"], factors=g["factors"],
                degrees=g["degrees"], edges=g["edges"], total_points=int(g["n"]), base_points=int(g["n"]))


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from quantization_graph_gb300 import _native

    _native.load()
    return torch
