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


def test_a_bounded_device_wait_that_runs_out_reports_a_timeout():
    """The OC update's grid-wide barrier waits a bounded number of polls.  With the test control, the last CTA
    withholds its arrival (a flag nothing else sets) and the waits give up after 1,000 polls: the update ends
    with PMG_TIMEOUT in its status word, the context stays usable, and with the control reset the same update
    succeeds and matches the oracle's bisection."""
    import pymoto_gb300 as pg
    from pymoto_gb300 import _lib
    lib = _lib.load()
    n = 200_000
    rng = np.random.default_rng(5)
    x = rng.uniform(0.2, 0.8, n)
    dg = -rng.uniform(0.1, 1.0, n)
    xd, dgd = torch.from_numpy(x).cuda(), torch.from_numpy(dg).cuda()
    xnew = torch.empty_like(xd)
    scratch = torch.zeros(lib.pmg_oc_scratch_bytes() // 8 + 1, dtype=torch.float64, device="cuda")
    st = _lib.stream()
    try:
        _lib.call("pmg_set_wait_test", 1000, 1)
        _lib.call("pmg_oc_update", n, xd, dgd, xnew, 0.5, 0.2, 0.0, 1.0, 0.0, 1e5, 1e-4, scratch, st)
        torch.cuda.synchronize()
        assert lib.pmg_oc_status(scratch.data_ptr()) == 3           # PMG_TIMEOUT
    finally:
        _lib.call("pmg_set_wait_test", 0, 0)
    _lib.call("pmg_oc_update", n, xd, dgd, xnew, 0.5, 0.2, 0.0, 1.0, 0.0, 1e5, 1e-4, scratch, st)
    torch.cuda.synchronize()
    assert lib.pmg_oc_status(scratch.data_ptr()) == 0
    ref = O.oc_step(x, dg, 0.5, move=0.2)
    np.testing.assert_allclose(xnew.cpu().numpy(), ref, rtol=0, atol=1e-12)
