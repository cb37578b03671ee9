import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle as po
    po.build()
    return po


@pytest.fixture(scope="session")
def golden_q():
    return np.load(os.path.join(GOLDEN, "golden_q.npz"))


@pytest.fixture(scope="session")
def golden_w():
    return np.load(os.path.join(GOLDEN, "golden_w_n8.npz"))


@pytest.fixture(scope="session")
def lib_built():
    from spectralbte_gb300 import builder as b
    b.build()
    import spectralbte_gb300 as sb
    return sb


@pytest.fixture(scope="session")
def gpu(lib_built):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    torch.cuda.set_device(0)
    return lib_built


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def golden_case(G, name):
    N, L_v, kind, lam = G[name + "_meta"]
    return int(N), float(L_v), ("0d" if int(kind) == 0 else "1d"), float(lam)
