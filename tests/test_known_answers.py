"""Known-answer checks of pyMOTO's own tests, restated for the oracle and the product's host side (CPU):
numbering and geometry of the voxel domain (tests/test_domain.py), Dirichlet rows and columns of the assembly
(tests/test_assembly.py:37-61), and the convolution filter's stencil placement, symmetric boundary and
agreement with the density filter (tests/test_filter.py:13-40, 147-247)."""
import numpy as np
import pytest

import oracle as O
import pymoto_gb300 as pg
from test_filter_variants import _emulate


# ---- voxel domain ---------------------------------------------------------------------------------------
@pytest.mark.parametrize("tag", ["d2", "d3"])
def test_domain_helpers_match_pymoto(tag, golden):
    g = golden("domain_helpers.npz")
    shp, size, origin = {"d2": ((5, 3, 0), (0.5, 0.25, 1.0), (1.0, -2.0, 0.0)),
                         "d3": ((4, 3, 2), (0.1, 0.2, 0.3), (0.5, 0.0, -1.0))}[tag]
    d = pg.VoxelDomain(*shp, *size)
    d.origin = np.array(origin)
    np.testing.assert_array_equal(d.get_node_indices(), g[f"{tag}_node_idx"])
    np.testing.assert_allclose(d.get_node_position(), g[f"{tag}_node_pos"], rtol=1e-15)
    np.testing.assert_array_equal(d.get_element_indices(), g[f"{tag}_el_idx"])
    np.testing.assert_allclose(d.get_element_position(), g[f"{tag}_el_pos"], rtol=1e-15)
    ii, jj, kk = g[f"{tag}_ijk"]
    np.testing.assert_array_equal(d.get_elemconnectivity(ii, jj, kk), g[f"{tag}_econn"])
    np.testing.assert_allclose(d.get_rigid_body_modes(), g[f"{tag}_rbm"], rtol=1e-15)
    np.testing.assert_allclose([d.eval_shape_fun(p) for p in g[f"{tag}_pts"]], g[f"{tag}_N"], rtol=1e-14)
    np.testing.assert_allclose([d.eval_shape_fun_der(p) for p in g[f"{tag}_pts"]], g[f"{tag}_dN"], rtol=1e-14,
                               atol=1e-14)
    np.testing.assert_allclose(d.domain_size, g[f"{tag}_domain_size"], rtol=1e-15)


@pytest.mark.parametrize("shape", [(100, 142, 0), (10, 14, 28)])
def test_node_numbering_round_trip(shape):
    """Every (i, j, k) has a unique number in [0, nnodes) that maps back to it; positions are i * unit."""
    units = (0.1, 0.2, 0.3)
    d = pg.VoxelDomain(*shape, *units)
    axes = [np.arange(n + 1) for n in shape[:d.dim]]
    ijk = np.meshgrid(*axes, indexing="ij")
    num = d.get_nodenumber(*ijk)
    assert num.min() == 0 and num.max() == d.nnodes - 1 and np.unique(num).size == num.size
    back = d.get_node_indices(num.ravel())
    for c in range(d.dim):
        np.testing.assert_array_equal(back[c], ijk[c].ravel())
        np.testing.assert_allclose(d.get_node_position(num.ravel())[c], ijk[c].ravel() * units[c])


@pytest.mark.parametrize("dofs", [0, np.array([0, 1])])
@pytest.mark.parametrize("nodes_i", [0, slice(0, 10), np.array([0, 1, 2])])
def test_dof_numbering_shapes(nodes_i, dofs):
    d = pg.VoxelDomain(100, 142, 0, 0.1, 0.2)
    n = d.nodes[nodes_i, 0]
    dof = d.get_dofnumber(n, dofs, 2)
    assert np.shape(dof) == (*np.shape(n), *np.shape(dofs))
    assert set(np.ravel(dof) // 2) <= set(np.ravel(n)) and set(np.ravel(dof) % 2) <= set(np.ravel(dofs))


def test_shape_functions_interpolate_at_the_nodes():
    for shape, units in [((1, 1, 0), (0.8, 0.3, 1.0)), ((1, 1, 1), (0.8, 0.3, 0.5))]:
        d = pg.VoxelDomain(*shape, *units)
        for a, sg in enumerate(d.node_numbering):
            pos = np.array([sg[c] * units[c] / 2 for c in range(d.dim)])
            np.testing.assert_allclose(d.eval_shape_fun(pos), np.eye(d.elemnodes)[a], atol=1e-15)
        # partition of unity: the derivatives sum to zero everywhere
        np.testing.assert_allclose(d.eval_shape_fun_der(np.full(d.dim, 0.05)).sum(axis=1), 0.0, atol=1e-14)


# ---- assembly: Dirichlet rows and columns --------------------------------------------------------------
def test_dirichlet_rows_and_columns_hold_only_the_diagonal_value():
    g = O.Grid(3, 3)
    K0 = np.arange(8 * 8, dtype=float).reshape(8, 8)      # a non-symmetric element matrix, as in pyMOTO's test
    bc = np.array([1, 2, 8, 15])
    A = O.assemble(g, K0, np.ones(g.nel), bc=bc, bcdiagval=1.5).toarray()
    np.testing.assert_allclose(A[bc, bc], 1.5)
    A[bc, bc] -= 1.5
    np.testing.assert_allclose(A[bc, :], 0.0)
    np.testing.assert_allclose(A[:, bc], 0.0)
    from pymoto_gb300.operators import bc_node_mask   # the device operator's form of the same set
    m = bc_node_mask(g.nnodes, 2, bc)
    got = sorted(2 * n + c for n in range(g.nnodes) for c in range(2) if (m[n] >> c) & 1)
    assert got == sorted(bc.tolist())


# ---- convolution filter --------------------------------------------------------------------------------
def _delta(d, *ijk):
    x = np.zeros(d.nel)
    x[d.get_elemnumber(*ijk)] = 1.0
    return x


def test_filter_stencil_placement_2d():
    """A unit value in the interior spreads the (flipped) kernel over its 3x3 neighbourhood."""
    d = pg.VoxelDomain(10, 12)
    fc = pg.FilterConv(d, radius=2, relative_units=True)
    y, _ = _emulate(fc, _delta(d, 5, 6), np.zeros(d.nel))
    w = fc.weights
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            assert y[d.get_elemnumber(5 + a, 6 + b)] == pytest.approx(w[1 - a, 1 - b, 0], rel=1e-14)


def test_filter_stencil_placement_and_symmetric_boundary_3d():
    d = pg.VoxelDomain(10, 11, 12)
    fc = pg.FilterConv(d, radius=2, relative_units=True)
    w = fc.weights
    y, _ = _emulate(fc, _delta(d, 5, 6, 7), np.zeros(d.nel))
    for a in range(3):
        for b in range(3):
            for c in range(3):
                assert y[d.get_elemnumber(4 + a, 5 + b, 6 + c)] == pytest.approx(w[a, b, c], rel=1e-14)
    # at z = 0 the symmetric padding mirrors the layer onto itself: the first layer gets two kernel layers
    y, _ = _emulate(fc, _delta(d, 5, 6, 0), np.zeros(d.nel))
    for a in range(3):
        for b in range(3):
            assert y[d.get_elemnumber(4 + a, 5 + b, 0)] == pytest.approx(w[a, b, 1] + w[a, b, 0], rel=1e-14)
            assert y[d.get_elemnumber(4 + a, 5 + b, 1)] == pytest.approx(w[a, b, 2], rel=1e-14)


def test_filter_adjoint_identity_with_absolute_units():
    """<F x, d> = <x, F^T d> for a non-cubic element and an absolute radius (filter.py:189-205)."""
    rng = np.random.default_rng(0)
    d = pg.VoxelDomain(7, 6, 5, unitx=0.5, unity=1.0, unitz=1.2)
    fc = pg.FilterConv(d, radius=2.3, relative_units=False)
    x, dy = rng.random(d.nel), rng.standard_normal(d.nel)
    y, _ = _emulate(fc, x, dy)
    _, dx = _emulate(fc, np.zeros(d.nel), dy)
    assert np.dot(y, dy) == pytest.approx(np.dot(x, dx), rel=1e-12)
    assert fc.weights.shape == (9, 5, 3) and fc.weights.sum() == pytest.approx(1.0, rel=1e-14)


def test_conv_filter_close_to_density_filter_somewhere():
    """The two filters differ only through their boundary treatment (pyMOTO: min |y1 - y2| <= 1e-4)."""
    rng = np.random.default_rng(0)
    g = O.Grid(6, 6, 6)
    x = rng.random(g.nel)
    y1 = O.conv_filter(g, O.conv_filter_weights(g, 5.0), x)
    H, s = O.density_filter_matrix(g, 5.0)
    assert np.abs(y1 - O.density_filter(H, s, x)).min() <= 1e-4


# ---- dyad contraction ----------------------------------------------------------------------------------
def test_element_contraction_of_a_dyad_sum():
    """pyMOTO's batched contract(K0, rows=dofconn, cols=dofconn) of a two-term dyad (test_dyadicmatrix.py:
    599-704): per element sum_k u_k[dofs_e] . K0 v_k[dofs_e], here with a non-symmetric K0 and u != v, and with
    the Dirichlet entries of the dyad zeroed first (dyadcarrier.py:179-189)."""
    rng = np.random.default_rng(0)
    g = O.Grid(3, 2, 2)
    K0 = rng.standard_normal((24, 24))
    us, vs = [rng.random(g.ndof) for _ in range(2)], [rng.random(g.ndof) for _ in range(2)]
    bc = np.array([0, 4, 17])
    got = O.sensitivity_contract(g, K0, us, vs, bc=bc)
    dc = g.dofconn()
    want = np.zeros(g.nel)
    for u, v in zip(us, vs):
        u, v = u.copy(), v.copy()
        u[bc] = v[bc] = 0.0
        for e in range(g.nel):
            want[e] += u[dc[e]] @ K0 @ v[dc[e]]
    np.testing.assert_allclose(got, want, rtol=1e-13)
