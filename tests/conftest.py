import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden", "known_answers.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle():
    from oracle import kmref

    kmref.build()
    return kmref


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("CUDA device not available")
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def kdp(cuda):
    import kmeans_dpcpp_gb300 as kdp

    return kdp


def has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
