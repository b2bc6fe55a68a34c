import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
# Checkout of the reference (read for its known-answer tables): the
# BNSN_REFERENCE_DIR environment variable, else a sibling of this repository.
REF_DIR = os.environ.get("BNSN_REFERENCE_DIR") or os.path.join(os.path.dirname(REPO),
                                                               "reference")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (run with -m gpu)")


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def port():
    import oracle
    return oracle.port()


@pytest.fixture(scope="session")
def ref():
    import oracle
    r = oracle.ref()
    if r is None:
        pytest.skip("reference build (oracle/_ref) not present on this host")
    return r


@pytest.fixture(scope="session")
def lib():
    from bns_nurates_gb300 import build
    build.build()
    import bns_nurates_gb300 as bn
    return bn.lib()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import build
    build.build()
    import oracle
    bn.set_gp19_table(oracle._synthetic_gp19())
    return torch


def rel_err(a, b, floor=0.0):
    """|a - b| / max(|b|, floor), elementwise, with 0/0 = 0."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor)
    num = np.abs(a - b)
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.where(num == 0, 0.0, num / den)
    return r
