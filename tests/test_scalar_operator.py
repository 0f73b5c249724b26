"""One-component operator (AssemblePoisson, AssembleMass(ndof=1)): node stencils, products, transfer operators,
Galerkin coarse operators and sensitivities against the oracle's one-component assembly
(pymoto/modules/assembly.py:245-296 with ndof = 1) and prolongation (pymoto/solvers/iterative.py:178-220)."""
import numpy as np
import pytest
import scipy.sparse as sps
import scipy.sparse.linalg as spla
import torch

import oracle as O
import pymoto_gb300 as pg
from pymoto_gb300._lib import F32, F64, call, stream
from pymoto_gb300.operators import Grid, ScalarOperator, bc_node_mask, element_mass, element_poisson

# (nelx, nely, nelz, unit sizes): 3D and 2D, odd and even counts
SHAPES = [(6, 4, 4, (1.0, 0.5, 0.8)), (5, 3, 2, (0.3, 0.3, 0.7)), (7, 5, 0, (1.0, 2.0, 0.5)), (8, 6, 0, (0.5, 0.5, 1.0))]
TOL = {F64: 1e-13, F32: 2e-6}      # relative to the largest entry: FP64 sums, and one FP32 rounding of them


def _case(shape, seed=0, bc=True, constant=True, mass=False):
    nx, ny, nz, unit = shape
    d = pg.VoxelDomain(nx, ny, nz, *unit)
    og = O.Grid(nx, ny, nz)
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.05, 1.0, og.nel)
    P0 = element_mass(d, 1, 2.0) if mass else element_poisson(d, 1.7)
    nodes = np.unique(rng.choice(og.nnodes, max(2, og.nnodes // 7), replace=False)) if bc else None
    c = rng.uniform(0.0, 0.3, og.nnodes) if constant else None
    bcdiag = float(np.max(P0))
    A = O.assemble(og, P0, x, bc=nodes, bcdiagval=bcdiag, ndof=1).tocsr()
    if c is not None:
        A = (A + sps.diags(c)).tocsr()
    return d, og, x, P0, nodes, c, bcdiag, A


def _operator(og, x, P0, nodes, c, bcdiag, code=F64):
    g = Grid(og.nelx, og.nely, og.nelz)
    mask = torch.from_numpy(bc_node_mask(g.nnodes, 1, nodes)).cuda()
    cd = None if c is None else torch.from_numpy(c).cuda()
    return ScalarOperator.assemble(g, torch.from_numpy(x).cuda(), P0, mask, bcdiag, cdiag=cd, code=code)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("code", [F64, F32])
@pytest.mark.parametrize("mass", [False, True])
def test_stencil_is_the_assembled_matrix(shape, code, mass):
    d, og, x, P0, nodes, c, bcdiag, A = _case(shape, mass=mass)
    op = _operator(og, x, P0, nodes, c, bcdiag, code)
    dense = op.to_dense().cpu().numpy()
    ref = A.toarray()
    np.testing.assert_allclose(dense, ref, rtol=0, atol=TOL[code] * np.abs(ref).max())
    np.testing.assert_allclose(op.diagonal().double().cpu().numpy(), ref.diagonal(), rtol=TOL[code], atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("code", [F64, F32])
def test_products_and_smoothing_modes(shape, code):
    d, og, x, P0, nodes, c, bcdiag, A = _case(shape, seed=1)
    op = _operator(og, x, P0, nodes, c, bcdiag, code)
    rng = np.random.default_rng(3)
    u, b = rng.standard_normal(og.nnodes), rng.standard_normal(og.nnodes)
    td = op.torch_dtype
    ud, bd = torch.from_numpy(u).to("cuda", td), torch.from_numpy(b).to("cuda", td)
    diag = op.diagonal()
    Au = A @ u
    scale = np.abs(A).sum(axis=1).max() * np.abs(u).max()
    y = op.matvec(ud).double().cpu().numpy()
    np.testing.assert_allclose(y, Au, rtol=0, atol=TOL[code] * 4 * scale)
    r = op.apply(pg._lib.RESIDUAL, ud, bd).double().cpu().numpy()
    np.testing.assert_allclose(r, b - Au, rtol=0, atol=TOL[code] * 4 * scale)
    w = 0.6
    j = op.apply(pg._lib.JACOBI, ud, bd, diag, w).double().cpu().numpy()
    ref = u + w * (b - Au) / A.diagonal()
    np.testing.assert_allclose(j, ref, rtol=0, atol=TOL[code] * 8 * np.abs(ref).max() * scale / np.abs(b - Au).max())
    # l1 row sums
    l1 = torch.empty_like(diag)
    op.l1_diagonal(l1)
    np.testing.assert_allclose(l1.double().cpu().numpy(), np.asarray(np.abs(A).sum(axis=1)).ravel(), rtol=TOL[code])
    # products are deterministic
    assert torch.equal(op.matvec(ud), op.matvec(ud))


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(8, 6, 4, (1.0, 1.0, 1.0)), (6, 4, 0, (1.0, 0.5, 1.0)), (4, 4, 2, (0.5, 1.0, 2.0))])
@pytest.mark.parametrize("code", [F64, F32])
def test_transfer_and_galerkin_match_the_prolongation(shape, code):
    d, og, x, P0, nodes, c, bcdiag, A = _case(shape, seed=2)
    op = _operator(og, x, P0, nodes, c, bcdiag, code)
    R = O.prolongation(og, ndof=1)
    oc = og.coarse()
    assert R.shape == (og.nnodes, oc.nnodes)
    rng = np.random.default_rng(4)
    rf, uc = rng.standard_normal(og.nnodes), rng.standard_normal(oc.nnodes)
    td = op.torch_dtype
    rc = torch.empty(oc.nnodes, dtype=td, device="cuda")
    op.restrict(torch.from_numpy(rf).to("cuda", td), rc)
    np.testing.assert_allclose(rc.double().cpu().numpy(), R.T @ rf, rtol=0, atol=TOL[code] * 8 * np.abs(rf).max())
    uf0 = rng.standard_normal(og.nnodes)
    uf = torch.from_numpy(uf0).to("cuda", td)
    op.prolong_add(torch.from_numpy(uc).to("cuda", td), uf)
    np.testing.assert_allclose(uf.double().cpu().numpy(), uf0 + R @ uc, rtol=0, atol=TOL[code] * 4 * np.abs(uc).max())
    Ac = op.galerkin()
    ref = (R.T @ A @ R).toarray()
    np.testing.assert_allclose(Ac.to_dense().cpu().numpy(), ref, rtol=0, atol=TOL[code] * 4 * np.abs(ref).max())
    # in place, and the next level down
    op.galerkin(out=Ac)
    np.testing.assert_allclose(Ac.to_dense().cpu().numpy(), ref, rtol=0, atol=TOL[code] * 4 * np.abs(ref).max())
    if Grid(oc.nelx, oc.nely, oc.nelz).can_coarsen():
        R2 = O.prolongation(oc, ndof=1)
        ref2 = (R2.T @ sps.csr_matrix(ref) @ R2).toarray()
        np.testing.assert_allclose(Ac.galerkin().to_dense().cpu().numpy(), ref2, rtol=0,
                                   atol=TOL[code] * 16 * np.abs(ref2).max())


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES)
def test_sensitivity_contraction(shape):
    d, og, x, P0, nodes, c, bcdiag, A = _case(shape, seed=5)
    rng = np.random.default_rng(6)
    u, v = rng.standard_normal(og.nnodes), rng.standard_normal(og.nnodes)
    mask = torch.from_numpy(bc_node_mask(og.nnodes, 1, nodes)).cuda()
    dx = torch.full((og.nel,), 7.0, dtype=torch.float64, device="cuda")
    ud, vd = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    call("pmg_scalar_sens", og.nelx, og.nely, og.nelz, P0, mask, ud, vd, 2.0, 0, dx, stream())
    ref = 2.0 * O.sensitivity_contract(og, P0, [u], [v], bc=nodes, ndof=1)
    np.testing.assert_allclose(dx.cpu().numpy(), ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
    call("pmg_scalar_sens", og.nelx, og.nely, og.nelz, P0, mask, vd, ud, -1.0, 1, dx, stream())
    np.testing.assert_allclose(dx.cpu().numpy(), 0.5 * ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def _thermal_case(shape, seed=7):
    """Heat sink: a plate with a fixed-temperature patch in the middle of the x = 0 face and a uniform heat load."""
    nx, ny, nz = shape
    og = O.Grid(nx, ny, nz)
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.01, 1.0, og.nel)
    jj = np.arange(ny // 4, 3 * ny // 4 + 1)
    kk = np.arange(nz // 4, 3 * nz // 4 + 1) if nz else np.array([0])
    nodes = og.nodes_where(i=0, j=jj, k=kk)
    f = np.full(og.nnodes, 1.0 / og.nnodes)
    return og, x, nodes, f


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["cg_mg_fp64", "cg_mg_fp32_chebyshev", "mixed_cg"])
@pytest.mark.parametrize("shape", [(16, 8, 8), (32, 16, 0)])
def test_multigrid_solves_of_the_poisson_problem(solver, shape):
    og, x, nodes, f = _thermal_case(shape)
    d = pg.VoxelDomain(*shape)
    P0 = element_poisson(d, 1.0)
    A = O.assemble(og, P0, x, bc=nodes, bcdiagval=float(P0.max()), ndof=1).tocsc()
    ref = spla.spsolve(A, f)
    if solver == "cg_mg_fp64":
        mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smoother_w=0.6, smooth_steps=2)
        sol = pg.CG(preconditioner=mgs[0], tol=1e-10, maxit=300)
    elif solver == "cg_mg_fp32_chebyshev":
        mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smooth_steps=2, precision="fp32", smoother="chebyshev")
        sol = pg.CG(preconditioner=mgs[0], tol=1e-10, maxit=300)
    else:
        mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smooth_steps=2, precision="fp32", smoother="chebyshev",
                                              coarse_lag=True)
        sol = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=1e-10, inner_iters=2)
    sx = pg.Signal("x", torch.from_numpy(x).cuda())
    fd = torch.from_numpy(f).cuda()
    with pg.Network() as fn:
        sK = pg.AssemblePoisson(d, bc=nodes)(sx)
        su = pg.LinSolve(hermitian=True, symmetric=True, solver=sol)(sK, fd)
        sc = pg.EinSum("i,i->")(su, fd)
    assert isinstance(sK.state, ScalarOperator)
    np.testing.assert_allclose(su.state.cpu().numpy(), ref, rtol=0, atol=1e-8 * np.abs(ref).max())
    assert sol.iterations < 60
    fn.reset()
    sc.sensitivity = 1.0
    fn.sensitivity()
    dref = O.sensitivity_contract(og, P0, [-ref], [ref], bc=nodes, ndof=1)
    np.testing.assert_allclose(sx.sensitivity.cpu().numpy(), dref, rtol=0, atol=1e-7 * np.abs(dref).max())
    # a second design: the hierarchy is refreshed in place
    x2 = np.clip(x * 1.3, 0.01, 1.0)
    sx.state = torch.from_numpy(x2).cuda()
    fn.response()
    A2 = O.assemble(og, P0, x2, bc=nodes, bcdiagval=float(P0.max()), ndof=1).tocsc()
    ref2 = spla.spsolve(A2, f)
    np.testing.assert_allclose(su.state.cpu().numpy(), ref2, rtol=0, atol=1e-8 * np.abs(ref2).max())


@pytest.mark.gpu
def test_scalar_operator_properties_at_128x64x64():
    """At 545,025 nodes: a Poisson matrix without Dirichlet nodes annihilates constants, and the product is
    symmetric (u.(A v) = v.(A u)); the Galerkin operator keeps both."""
    d = pg.VoxelDomain(128, 64, 64)
    g = Grid(128, 64, 64)
    rng = np.random.default_rng(8)
    x = torch.from_numpy(rng.uniform(1e-3, 1.0, g.nel)).cuda()
    mask = torch.zeros(g.nnodes, dtype=torch.uint8, device="cuda")
    op = ScalarOperator.assemble(g, x, element_poisson(d, 1.0), mask, 1.0)
    one = torch.ones(g.nnodes, dtype=torch.float64, device="cuda")
    scale = float(op.diagonal().abs().max())
    assert float(op.matvec(one).abs().max()) < 1e-12 * scale
    u = torch.from_numpy(rng.standard_normal(g.nnodes)).cuda()
    v = torch.from_numpy(rng.standard_normal(g.nnodes)).cuda()
    a, b = float(u @ op.matvec(v)), float(v @ op.matvec(u))
    assert abs(a - b) <= 1e-11 * (abs(a) + abs(b))
    Ac = op.galerkin()
    onec = torch.ones(g.coarse().nnodes, dtype=torch.float64, device="cuda")
    assert float(Ac.matvec(onec).abs().max()) < 1e-11 * float(Ac.diagonal().abs().max())


@pytest.mark.gpu
def test_poisson_with_a_constant_diagonal_solves_the_shifted_system():
    """add_constant (a diagonal, e.g. convection to ambient) is added after the Dirichlet rows, as pyMOTO adds its
    constant matrix to the assembled one (assembly.py:294-295)."""
    og, x, nodes, f = _thermal_case((8, 6, 4))
    d = pg.VoxelDomain(8, 6, 4)
    P0 = element_poisson(d, 1.0)
    c = np.random.default_rng(9).uniform(0.0, 0.5, og.nnodes)
    A = (O.assemble(og, P0, x, bc=nodes, bcdiagval=float(P0.max()), ndof=1) + sps.diags(c)).tocsc()
    ref = spla.spsolve(A, f)
    sx = pg.Signal("x", torch.from_numpy(x).cuda())
    fd = torch.from_numpy(f).cuda()
    with pg.Network() as fn:
        sK = pg.AssemblePoisson(d, bc=nodes, add_constant=sps.diags(c))(sx)
        su = pg.LinSolve(hermitian=True, symmetric=True)(sK, fd)
    np.testing.assert_allclose(su.state.cpu().numpy(), ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    np.testing.assert_allclose(sK.state.to_dense().cpu().numpy(), A.toarray(), rtol=0, atol=1e-13 * abs(A).max())


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["s3", "s2"])
def test_galerkin_and_vcycle_match_pymotos_multigrid(tag, golden):
    """The device hierarchy of an AssemblePoisson operator against pyMOTO's GeometricMultigrid on the same matrix
    (two levels, damped Jacobi w = 0.6, 2 sweeps, direct coarsest solve): R^T P R and one V-cycle."""
    g = golden("poisson_mg.npz")
    shp = tuple(int(v) for v in g[f"{tag}_shape"])
    d = pg.VoxelDomain(*shp)
    og = O.Grid(*shp) if len(shp) == 3 else O.Grid(*shp, 0)
    nc = og.coarse().nnodes
    Ac = sps.csr_matrix((g[f"{tag}_Ac_data"], g[f"{tag}_Ac_indices"], g[f"{tag}_Ac_indptr"]), shape=(nc, nc))
    P = pg.AssemblePoisson(d, bc=g[f"{tag}_bc"])(torch.from_numpy(g[f"{tag}_x"]).cuda())
    np.testing.assert_allclose(P.galerkin().to_dense().cpu().numpy(), Ac.toarray(), rtol=0,
                               atol=1e-13 * abs(Ac).max())
    mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smoother_w=0.6, smooth_steps=2)
    mgs[0].update(P)
    z = mgs[0].solve(torch.from_numpy(g[f"{tag}_r"]).cuda()).cpu().numpy()
    np.testing.assert_allclose(z, g[f"{tag}_z"], rtol=0, atol=1e-11 * np.abs(g[f"{tag}_z"]).max())


@pytest.mark.gpu
def test_poisson_with_a_neighbour_coupling_constant():
    """A constant with off-diagonal entries between neighbouring nodes (add_constant, assembly.py:294-295) enters
    the one-component stencils exactly: the operator, the multigrid solve and the sensitivities against the
    oracle's P(x) + C."""
    from test_poisson import _neighbour_constant
    og, x, nodes, f = _thermal_case((8, 6, 4))
    d = pg.VoxelDomain(8, 6, 4)
    P0 = element_poisson(d, 1.0)
    C = _neighbour_constant(og)
    A = (O.assemble(og, P0, x, bc=nodes, bcdiagval=float(P0.max()), ndof=1) + C).tocsc()
    ref = spla.spsolve(A, f)
    sx = pg.Signal("x", torch.from_numpy(x).cuda())
    fd = torch.from_numpy(f).cuda()
    with pg.Network() as fn:
        sK = pg.AssemblePoisson(d, bc=nodes, add_constant=C)(sx)
        su = pg.LinSolve(hermitian=True, symmetric=True)(sK, fd)
        sc = pg.EinSum("i,i->")(su, fd)
    np.testing.assert_allclose(sK.state.to_dense().cpu().numpy(), A.toarray(), rtol=0, atol=1e-13 * abs(A).max())
    np.testing.assert_allclose(su.state.cpu().numpy(), ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    fn.reset()
    sc.sensitivity = 1.0
    fn.sensitivity()
    dref = O.sensitivity_contract(og, P0, [-ref], [ref], bc=nodes, ndof=1)
    np.testing.assert_allclose(sx.sensitivity.cpu().numpy(), dref, rtol=0, atol=1e-8 * np.abs(dref).max())
    K32 = sK.state.astype(F32)
    np.testing.assert_allclose(K32.to_dense().cpu().numpy(), A.toarray(), rtol=0, atol=2e-6 * abs(A).max())
