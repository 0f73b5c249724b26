"""Parity at the benchmark configurations' sizes (GPU), against the oracle:

* the 2D cantilever of 400 x 200 Q4 elements (161,202 dofs; smoothed-noise density, FilterConv r=3, multigrid
  of 4 levels with damped Jacobi w=0.6, 2 sweeps), against the FP64 direct solve (SuperLU, as pyMOTO's
  SolverSparseLU, pymoto/solvers/sparse.py:515-555);
* the 3D cantilevers of 64 x 32 x 32 and 128 x 64 x 64 hex8 elements (212,355 and 1,635,075 dofs; seeded
  U(1e-3, 1) density -- the benchmark's first design --, FilterConv r=2.5), against pyMOTO's FP64 CG + geometric
  multigrid (pymoto/solvers/iterative.py:124-403) driven to a relative residual of 1e-11 (an FP64 direct solve
  does not fit at these sizes);
* central finite differences on 64 elements drawn by rng.choice(nel, 64) of both 3D cases (the adjoint
  sensitivities).

Both GPU arms are checked: the FP64 path (CG + FP64 multigrid) to 1e-8, the mixed path (FP64 flexible CG around
FP32 multigrid-preconditioned PCG) at the relative residuals it is run at.  The errors are printed (pytest -s).
"""
import numpy as np
import pytest
import torch
from scipy.ndimage import gaussian_filter

import oracle as O

pytestmark = pytest.mark.gpu


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


@pytest.fixture(scope="module")
def pg():
    import pymoto_gb300 as pg
    pg._lib.load()
    return pg


def cantilever(g):
    """Left face (i = 0) clamped, unit -y load at the middle node of the right face."""
    nodes = g.nodes_where(i=0)
    bc = (nodes[:, None] * g.dim + np.arange(g.dim)).ravel()
    f = np.zeros(g.ndof)
    tip = g.node_number(g.nelx, g.nely // 2, g.nelz // 2) if g.dim == 3 else g.node_number(g.nelx, g.nely // 2)
    f[g.dim * tip + 1] = -1.0
    return bc, f


def smoothed_noise(shape, seed, sigma=4.0):
    """Gaussian-smoothed U(0, 1) noise (sigma in elements), min-max mapped to [1e-3, 1], element order."""
    nx, ny, nz = shape
    a = np.random.default_rng(seed).uniform(0.0, 1.0, (nz, ny, nx) if nz else (ny, nx))
    a = gaussian_filter(a, sigma=sigma)
    a = (a - a.min()) / (a.max() - a.min())
    return (1e-3 + (1.0 - 1e-3) * a).ravel()


def gpu_run(pg, shape, bc, f, x, radius, plane, levels, arm, tol):
    """c, u, dc/dx of the GPU network for design x; arm 'fp64' (CG + FP64 GMG, damped Jacobi 0.6, 2 sweeps) or
    'mixed' (FP64 FCG + FP32 GMG with the Chebyshev smoother, mixed sensitivity contraction)."""
    d = pg.VoxelDomain(*shape)
    sx = pg.Signal("x", dev(x))
    fd = dev(f)
    mixed = arm == "mixed"
    with pg.Network() as fn:
        xf = pg.FilterConv(d, radius=radius)(sx)
        xs = pg.SIMP(xmin=1e-9, penal=3.0)(xf)
        K = pg.AssembleStiffness(d, bc=bc, plane=plane, sensitivity_precision="mixed" if mixed else "fp64")(xs)
        if mixed:
            mgs = pg.GeometricMultigrid.hierarchy(d, levels=levels, smooth_steps=1, precision="fp32",
                                                  coarse_smooth_steps=[2, 3, 6], smoother="chebyshev", cheb_ratio=15.0)
            solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=tol, inner_iters=4, inner_tol=0.1)
        else:
            mgs = pg.GeometricMultigrid.hierarchy(d, levels=levels, smoother_w=0.6, smooth_steps=2)
            solver = pg.CG(preconditioner=mgs[0], tol=tol, maxit=5000)
        lin = pg.LinSolve(hermitian=True, symmetric=True, solver=solver)
        u = lin(K, fd)
        c = pg.EinSum("i,i->")(u, fd)
    fn.reset()
    c.sensitivity = 1.0
    fn.sensitivity()
    res = pg.LinearSolver.residual(lin.A, lin._u_dev, fd)
    return (float(c.state), u.state.cpu().numpy(), sx.sensitivity.cpu().numpy(), res,
            (fn, sx, c))


def errors(c, u, dc, c_ref, u_ref, dc_ref):
    return {"c": abs(c - c_ref) / abs(c_ref),
            "u": float(np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref)),
            "dc": float(np.abs(dc - dc_ref).max() / np.abs(dc_ref).max())}


# ------------------------------------------------------------------------------------------ 2D, 400 x 200
@pytest.fixture(scope="module")
def q4_400x200():
    shape = (400, 200, 0)
    g = O.Grid(*shape)
    bc, f = cantilever(g)
    x = smoothed_noise(shape, seed=11)
    P = O.CompliancePipeline(g, bc, f, filter_kind="conv", radius=3.0, plane="stress", levels=0)
    c = P.response(x)
    dc = P.sensitivity()
    return shape, bc, f, x, c, P.u.copy(), dc


# The mixed path's sensitivities come from the FP32 contraction of FP64-shifted element vectors: their error
# stays near 1e-7 of max |dc| whatever the residual, within the 1e-6 bar of the mixed path.
LIMITS = [("fp64", 1e-10, {"c": 1e-8, "u": 1e-8, "dc": 1e-8}),
          ("mixed", 1e-6, {"c": 1e-6, "u": 1e-5, "dc": 1e-6}),
          ("mixed", 1e-8, {"c": 1e-8, "u": 1e-7, "dc": 1e-6})]


@pytest.mark.parametrize("arm,tol,lim", LIMITS, ids=["fp64", "mixed-1e-6", "mixed-1e-8"])
def test_q4_400x200_against_direct_solve(pg, q4_400x200, arm, tol, lim):
    shape, bc, f, x, c_ref, u_ref, dc_ref = q4_400x200
    c, u, dc, res, _ = gpu_run(pg, shape, bc, f, x, 3.0, "stress", 4, arm, tol)
    err = errors(c, u, dc, c_ref, u_ref, dc_ref)
    print(f"\n400x200 Q4 {arm} tol {tol:g}: true residual {res:.2e}, errors {err}")
    assert res <= tol * 1.0001
    for k, v in lim.items():
        assert err[k] <= v, (k, err[k], v)


# ------------------------------------------------------------------------------------------ 3D
@pytest.fixture(scope="module", params=[(64, 32, 32), (128, 64, 64)], ids=["64x32x32", "128x64x64"])
def h8_case(request):
    shape = request.param
    x = np.random.default_rng(1234).uniform(1e-3, 1.0, int(np.prod(shape)))
    ref = O.fp64_cg_reference(shape, x, radius=2.5, levels=4, tol=1e-12)
    print(f"\noracle {shape}: FP64 CG + GMG, {ref['iterations']} iterations, true relative residual "
          f"{ref['residual']:.2e}")
    assert ref["residual"] <= 1e-11
    return shape, ref["bc"], ref["f"], x, ref["c"], ref["u"], ref["dc"]


@pytest.mark.parametrize("arm,tol,lim", LIMITS, ids=["fp64", "mixed-1e-6", "mixed-1e-8"])
def test_hex8_against_fp64_cg_to_1e_11(pg, h8_case, arm, tol, lim):
    shape, bc, f, x, c_ref, u_ref, dc_ref = h8_case
    c, u, dc, res, _ = gpu_run(pg, shape, bc, f, x, 2.5, "strain", 4, arm, tol)
    err = errors(c, u, dc, c_ref, u_ref, dc_ref)
    print(f"\n{shape} hex8 {arm} tol {tol:g}: true residual {res:.2e}, errors {err}")
    assert res <= tol * 1.0001
    for k, v in lim.items():
        assert err[k] <= v, (k, err[k], v)


def test_hex8_central_differences_on_64_elements(pg, h8_case):
    """dc/dx of the FP64 path against central differences (h = 1e-3 x_e: the compliance changes by ~1e-7 of
    itself, far above the solves' rounding, while the O(h^2) truncation stays near 1e-7 of dc) on 64 elements
    drawn by rng.choice(nel, 64); every perturbed solve runs to a relative residual of 1e-12."""
    shape, bc, f, x, _, _, _ = h8_case
    c0, _, dc, _, (fn, sx, c) = gpu_run(pg, shape, bc, f, x, 2.5, "strain", 4, "fp64", 1e-12)
    idx = np.random.default_rng(0).choice(x.size, 64, replace=False)
    fd = np.empty(64)
    for k, e in enumerate(idx):
        h = 1e-3 * x[e]
        vals = []
        for s in (+1.0, -1.0):
            xp = x.copy()
            xp[e] += s * h
            sx.state = dev(xp)
            fn.response()
            vals.append(float(c.state))
        fd[k] = (vals[0] - vals[1]) / (2 * h)
    err = np.linalg.norm(fd - dc[idx]) / np.linalg.norm(dc[idx])
    print(f"\n{shape} central differences on 64 elements: relative error {err:.2e}")
    assert err <= 1e-4
