"""Host-side fault injection (GPU): a zero load, an exhausted iteration limit, NaN in the load and a wrongly
sized design end in a defined result, a warning or an exception -- never a hang or a device fault (every
device loop is bounded)."""
import warnings

import numpy as np
import pytest
import torch

import oracle as O
from conftest import clamp_face_dofs

pytestmark = pytest.mark.gpu

SHAPE = (16, 8, 8)


def _problem():
    g = O.Grid(*SHAPE)
    f = np.zeros(g.ndof)
    f[3 * g.node_number(16, 4, 4) + 1] = -1.0
    return g, clamp_face_dofs(g), f


def _operator(pg, bc, x=None):
    d = pg.VoxelDomain(*SHAPE)
    x = np.random.default_rng(3).uniform(0.1, 1.0, d.nel) if x is None else x
    return d, pg.AssembleStiffness(d, bc=bc)(torch.from_numpy(x).cuda())


def test_zero_load_gives_zero_displacement_without_warning():
    import pymoto_gb300 as pg
    g, bc, f = _problem()
    d, K = _operator(pg, bc)
    mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smoother_w=0.6, smooth_steps=2)
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        u = pg.LinSolve(hermitian=True, symmetric=True, solver=pg.CG(preconditioner=mgs[0], tol=1e-10))(
            K, torch.zeros(g.ndof, dtype=torch.float64, device="cuda"))
    assert not [w for w in rec if "Maximum iterations" in str(w.message)]
    assert torch.count_nonzero(u).item() == 0       # the stored (zero) pair is harmless: no NaN


def test_exhausted_iteration_limit_warns_and_returns_the_iterate():
    import pymoto_gb300 as pg
    g, bc, f = _problem()
    d, K = _operator(pg, bc)
    mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smoother_w=0.6, smooth_steps=2)
    cg = pg.CG(preconditioner=mgs[0], tol=1e-14, maxit=2)
    cg.update(K)
    with pytest.warns(UserWarning, match="Maximum iterations"):
        u = cg.solve(torch.from_numpy(f).cuda())
    assert torch.isfinite(u).all() and cg.iterations == 2


@pytest.mark.parametrize("mixed", [False, True], ids=["cg", "mixed"])
def test_nan_in_the_load_ends_the_solve_with_a_warning(mixed):
    import pymoto_gb300 as pg
    g, bc, f = _problem()
    d, K = _operator(pg, bc)
    f = f.copy()
    f[3 * g.node_number(8, 4, 4)] = np.nan
    mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smoother_w=0.6, smooth_steps=2,
                                          precision="fp32" if mixed else None)
    solver = (pg.MixedPrecisionCG(preconditioner=mgs[0], tol=1e-8, maxit=50) if mixed
              else pg.CG(preconditioner=mgs[0], tol=1e-8, maxit=50))
    solver.update(K)
    with pytest.warns(UserWarning):
        solver.solve(torch.from_numpy(f).cuda())
    assert solver.iterations <= 50 + 1     # a non-finite residual ends the solve at once


def test_wrongly_sized_design_is_rejected():
    import pymoto_gb300 as pg
    g, bc, f = _problem()
    d = pg.VoxelDomain(*SHAPE)
    with pytest.raises(ValueError):
        pg.AssembleStiffness(d, bc=bc)(torch.ones(d.nel + 1, dtype=torch.float64, device="cuda"))
