import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C-ABI")
    config.addinivalue_line("markers", "slow: long-running full-size check")


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


@pytest.fixture(scope="session")
def lm():
    import lagrangian_microbes_gb300 as pkg
    return pkg


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def small_field(lm):
    # configuration S: 0.25 deg grid over 195-206E x 20-31N, 6-hourly frames covering 48 h + margin
    return lm.synthetic_psi_field(195.0, 206.0, 20.0, 31.0, 0.25, n_frames=10, frame_seconds=6 * 3600.0, seed=1)
