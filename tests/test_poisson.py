"""AssemblePoisson: the scalar element matrix and the one-component assembly, against pyMOTO's AssemblePoisson and a
thermal compliance network."""
import numpy as np
import pytest
import scipy.sparse as sps
import scipy.sparse.linalg as spla
import torch

import oracle as O
import pymoto_gb300 as pg
from pymoto_gb300.operators import element_poisson


@pytest.mark.parametrize("tag,shp,size,k", [("p2", (3, 2, 0), (0.5, 2.0, 0.3), 2.5),
                                            ("p3", (2, 2, 2), (0.1, 0.2, 0.3), 1.7)])
def test_element_matrix_matches_pymoto(tag, shp, size, k, golden):
    P0 = element_poisson(pg.VoxelDomain(*shp, *size), k)
    np.testing.assert_allclose(P0, golden("poisson.npz")[f"{tag}_P0"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(P0.sum(axis=1), 0.0, atol=1e-13)     # constants are in the null space


def _scalar_system(golden):
    g = golden("poisson.npz")
    d = pg.VoxelDomain(6, 4, 4, 1.0, 0.5, 0.8)
    m = pg.AssemblePoisson(d, bc=g["net_bc"], material_property=2.0)
    grid = O.Grid(6, 4, 4)
    A = O.assemble(grid, m.poisson_element, g["net_x"], bc=g["net_bc"], bcdiagval=m.bcdiagval, ndof=1).tocsr()
    return g, m, grid, A


def test_one_component_oracle_is_pymotos_matrix(golden):
    g, m, grid, A = _scalar_system(golden)
    assert A.shape == (grid.nnodes, grid.nnodes)
    np.testing.assert_allclose(A @ g["net_urand"], g["net_Pu"], rtol=1e-13, atol=1e-15)
    assert m._mask_host.max() <= 1 and np.flatnonzero(m._mask_host).tolist() == sorted(set(g["net_bc"].tolist()))


def test_one_component_solve_and_sensitivity_reproduce_the_thermal_network(golden):
    g, m, grid, A = _scalar_system(golden)
    u = spla.spsolve(A.tocsc(), g["net_f"])   # Dirichlet rows are bcdiag I: their solution is load / bcdiag
    np.testing.assert_allclose(u, g["net_u"], rtol=1e-10, atol=1e-14)
    assert float(u @ g["net_f"]) == pytest.approx(float(g["net_c"]), rel=1e-10)
    dx = O.sensitivity_contract(grid, m.poisson_element, [-u], [u], bc=g["net_bc"], ndof=1)
    np.testing.assert_allclose(dx, g["net_dx"], rtol=1e-9, atol=1e-14)


@pytest.mark.gpu
def test_thermal_compliance_network_on_device(golden):
    g = golden("poisson.npz")
    d = pg.VoxelDomain(6, 4, 4, 1.0, 0.5, 0.8)
    f = torch.from_numpy(g["net_f"]).cuda()
    sx = pg.Signal("x", torch.from_numpy(g["net_x"]).cuda())
    with pg.Network() as fn:
        sK = pg.AssemblePoisson(d, bc=g["net_bc"], material_property=2.0)(sx)
        su = pg.LinSolve(hermitian=True, symmetric=True)(sK, f)
        sc = pg.EinSum("i,i->")(su, f)
    np.testing.assert_allclose(su.state.cpu().numpy(), g["net_u"], rtol=1e-8, atol=1e-12)
    assert float(sc.state) == pytest.approx(float(g["net_c"]), rel=1e-8)
    fn.reset()
    sc.sensitivity = 1.0
    fn.sensitivity()
    np.testing.assert_allclose(sx.sensitivity.cpu().numpy(), g["net_dx"], rtol=1e-7, atol=1e-12)


def _golden_mg(golden, tag):
    g = golden("poisson_mg.npz")
    shp = tuple(int(v) for v in g[f"{tag}_shape"])
    og = O.Grid(*shp) if len(shp) == 3 else O.Grid(*shp, 0)
    nn = og.nnodes
    R = sps.coo_matrix((g[f"{tag}_R_val"], (g[f"{tag}_R_row"], g[f"{tag}_R_col"])),
                       shape=(nn, og.coarse().nnodes)).tocsr()
    nc = og.coarse().nnodes
    Ac = sps.csr_matrix((g[f"{tag}_Ac_data"], g[f"{tag}_Ac_indices"], g[f"{tag}_Ac_indptr"]), shape=(nc, nc))
    return g, shp, og, R, Ac


@pytest.mark.parametrize("tag", ["s3", "s2"])
def test_one_component_multigrid_oracle_matches_pymoto(tag, golden):
    """pyMOTO's GeometricMultigrid on AssemblePoisson matrices (one dof per node): the oracle's prolongation,
    Galerkin operator and V-cycle (iterative.py:124-256) reproduce it."""
    g, shp, og, R, Ac = _golden_mg(golden, tag)
    P0 = element_poisson(pg.VoxelDomain(*shp), 1.0)
    A = O.assemble(og, P0, g[f"{tag}_x"], bc=g[f"{tag}_bc"], bcdiagval=float(P0.max()), ndof=1).tocsr()
    Ro = O.prolongation(og, ndof=1)
    assert abs(Ro - R).max() == 0
    Aco = (Ro.T @ A @ Ro).tocsr()
    np.testing.assert_allclose(Aco.toarray(), Ac.toarray(), rtol=0, atol=1e-13 * abs(Ac).max())
    lv = O.build_hierarchy(og, A, 3, w=0.6, smooth_steps=2, ndof=1)
    z = O.vcycle(lv[0], g[f"{tag}_r"])
    np.testing.assert_allclose(z, g[f"{tag}_z"], rtol=0, atol=1e-11 * np.abs(g[f"{tag}_z"]).max())


@pytest.mark.parametrize("shp", [(6, 4, 4), (5, 3, 2), (7, 5, 0)])
def test_one_component_host_layout(shp):
    """Host side of the one-component operator: the natural-numbering half bandwidth the coarsest direct solve
    uses is that of the oracle's assembled matrix, and the Dirichlet mask marks bit 0 of the constrained nodes."""
    from pymoto_gb300.operators import Grid, ScalarOperator, bc_node_mask, scalar_stencil_offsets
    og = O.Grid(*shp)
    rng = np.random.default_rng(3)
    P0 = element_poisson(pg.VoxelDomain(*shp), 1.0)
    A = O.assemble(og, P0, rng.uniform(0.1, 1.0, og.nel), ndof=1).tocoo()
    g = Grid(*shp)
    op = ScalarOperator(g, None, 0)
    assert op.bandwidth() == int(np.abs(A.row - A.col).max())
    assert op.shape == (og.nnodes, og.nnodes) and op.ncomp == 1
    assert scalar_stencil_offsets(g.dim) == (27 if g.dim == 3 else 9)
    nodes = np.array([0, 3, og.nnodes - 1])
    m = bc_node_mask(og.nnodes, 1, nodes)
    assert np.flatnonzero(m).tolist() == nodes.tolist() and m.max() == 1
    with pytest.raises(IndexError):
        bc_node_mask(og.nnodes, 1, [og.nnodes])


def _neighbour_constant(og, a=0.3):
    """A symmetric constant coupling x-neighbours in the right half of the grid (a convection-like term)."""
    rows, cols, vals = [], [], []
    for k in range(og.nelz + 1):
        for j in range(og.nely + 1):
            for i in range(og.nelx // 2, og.nelx):
                n = int(og.node_number(i, j, k))
                rows += [n, n + 1, n, n + 1]
                cols += [n, n + 1, n + 1, n]
                vals += [a, a, -a, -a]
    return sps.coo_matrix((vals, (rows, cols)), shape=(og.nnodes, og.nnodes)).tocsr()


@pytest.mark.parametrize("shp", [(8, 6, 4), (8, 6, 0)])
def test_neighbour_coupling_constant_in_stencil_layout(shp):
    """add_constant of a one-component operator: its diagonal and its neighbour couplings in the node-stencil
    layout reproduce the matrix; couplings beyond the neighbours, non-symmetric constants and couplings of
    constrained nodes are refused."""
    from pymoto_gb300.modules import _stencil_constant
    from pymoto_gb300.operators import Grid
    og = O.Grid(*shp)
    g = Grid(*shp)
    C = _neighbour_constant(og)
    diag, st = _stencil_constant(C, g)
    dense = np.diag(diag)
    for o in range(st.shape[0]):
        dx, dy, dz = o % 3 - 1, (o // 3) % 3 - 1, (o // 9 - 1 if g.dim == 3 else 0)
        for n in np.flatnonzero(st[o]):
            dense[n, n + dx + dy * (og.nelx + 1) + dz * (og.nelx + 1) * (og.nely + 1)] += st[o, n]
    np.testing.assert_array_equal(dense, C.toarray())
    diag2, st2 = _stencil_constant(sps.diags(np.arange(og.nnodes, dtype=float)), g)
    assert st2 is None and np.array_equal(diag2, np.arange(og.nnodes))
    far = sps.coo_matrix(([1.0, 1.0], ([0, 2], [2, 0])), shape=(og.nnodes, og.nnodes))
    with pytest.raises(NotImplementedError):
        _stencil_constant(far, g)
    skew = sps.coo_matrix(([1.0], ([0], [1])), shape=(og.nnodes, og.nnodes))
    with pytest.raises(NotImplementedError):
        _stencil_constant(skew, g)
    d = pg.VoxelDomain(*shp)
    pg.AssemblePoisson(d, bc=og.nodes_where(i=0), add_constant=C)
    with pytest.raises(NotImplementedError):
        pg.AssemblePoisson(d, bc=og.nodes_where(i=og.nelx), add_constant=C)


def test_constant_inputs_of_one_component_operators():
    """add_constant as a sparse matrix, a dense matrix or a diagonal vector gives the same stencil layout."""
    from pymoto_gb300.modules import _stencil_constant
    from pymoto_gb300.operators import Grid
    og, g = O.Grid(6, 4, 2), Grid(6, 4, 2)
    C = _neighbour_constant(og) + sps.diags(np.linspace(0.1, 1.0, og.nnodes))
    d1, s1 = _stencil_constant(C, g)
    d2, s2 = _stencil_constant(C.toarray(), g)
    np.testing.assert_array_equal(d1, d2)
    np.testing.assert_array_equal(s1, s2)
    d3, s3 = _stencil_constant(np.linspace(0.1, 1.0, og.nnodes), g)
    assert s3 is None
    np.testing.assert_array_equal(d3, np.linspace(0.1, 1.0, og.nnodes))
    assert _stencil_constant(None, g) == (None, None)
    with pytest.raises(ValueError):
        _stencil_constant(sps.eye(og.nnodes + 1), g)


def test_learned_warm_start_refuses_one_component_operators():
    """The learned warm start predicts displacement fields: a mixed solver with one refuses a one-component
    operator before touching the device."""
    from pymoto_gb300.operators import Grid, ScalarOperator
    solver = pg.MixedPrecisionCG(warm_start=object())
    with pytest.raises(NotImplementedError):
        solver.update(ScalarOperator(Grid(4, 4, 4), None, 0))
