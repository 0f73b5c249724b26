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


# The hot path's kernel and pipeline parity files (and MMA, VTI) run first, the other next rows and the
# auxiliary subsystems after them, then the parity at the benchmark sizes (the slowest file: its oracle solves
# a 1.6M-dof system on the host), so that with -x a failure in a later file does not hide the earlier results;
# test_zz_no_alloc stays last.
_LATER = ("test_filter_variants", "test_mass", "test_poisson", "test_scalar_operator", "test_overhang",
          "test_math_expression",
          "test_scalars", "test_einsum", "test_routines", "test_design_runs", "test_checkpoint", "test_faults",
          "test_config_parity", "test_zz_no_alloc")


def pytest_collection_modifyitems(session, config, items):
    def rank(item):
        mod = item.module.__name__.rsplit(".", 1)[-1] if item.module is not None else ""
        return _LATER.index(mod) + 1 if mod in _LATER else 0
    items[:] = sorted(items, key=rank)     # stable: the order within a file is kept
