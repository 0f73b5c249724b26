import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name)) as f:
        return {k: f[k] for k in f.files}


@pytest.fixture(scope="session")
def golden():
    return load_golden


def clamp_face_dofs(grid):
    """Dirichlet dofs of the i = 0 face (all components), the cantilever support used in the fixtures."""
    nodes = grid.nodes_where(i=0)
    return (nodes[:, None] * grid.dim + np.arange(grid.dim)).ravel()
