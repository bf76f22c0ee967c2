"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the sm_103a library)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle, build_oracle
    build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def golden_rotations():
    return dict(np.load(os.path.join(GOLDEN, "rotations.npz"), allow_pickle=False))


@pytest.fixture(scope="session")
def golden_trajectories():
    return dict(np.load(os.path.join(GOLDEN, "trajectories.npz"), allow_pickle=False))


@pytest.fixture(scope="session")
def engine():
    from ddevol_gb300.engine import Engine
    eng = Engine(0)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def branch_ctx():
    from ddevol_gb300.engine import CudaBranchContext
    ctx = CudaBranchContext(0)
    yield ctx
    ctx.close()
