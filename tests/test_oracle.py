"""The CPU oracle against pyMOTO's golden vectors and known-answer tests (no GPU)."""
import numpy as np
import pytest
import scipy.sparse as sps

import oracle as O


def grid_of(shape, units=(1.0, 1.0, 1.0)):
    shape = list(shape) + [0] * (3 - len(shape))
    return O.Grid(*shape, *units)


def test_index_maps_and_element_matrices(golden):
    g = golden("maps_k0.npz")
    for tag in ["q4", "q4s", "h8", "h8s"]:
        grid = grid_of(g[f"{tag}_shape"], g[f"{tag}_units"])
        assert np.array_equal(grid.conn(), g[f"{tag}_conn"])
        assert np.array_equal(grid.dofconn(), g[f"{tag}_dofconn"])
        np.testing.assert_allclose(O.element_stiffness(grid), g[f"{tag}_K0"], rtol=0, atol=1e-15 * np.abs(g[f"{tag}_K0"]).max())
        if grid.dim == 2:
            np.testing.assert_allclose(O.element_stiffness(grid, plane="stress"), g[f"{tag}_K0stress"], rtol=1e-15, atol=1e-16)


def test_assembly_matches_reference_csr(golden):
    g = golden("assembly.npz")
    for tag in ["q4", "h8"]:
        grid = grid_of(g[f"{tag}_shape"])
        K = O.assemble(grid, O.element_stiffness(grid), g[f"{tag}_x"], g[f"{tag}_bc"])
        Kr = sps.csr_matrix((g[f"{tag}_data"], g[f"{tag}_indices"], g[f"{tag}_indptr"]), shape=K.shape)
        assert abs(K - Kr).max() <= 1e-15 * abs(Kr).max()
        np.testing.assert_allclose(K @ g[f"{tag}_u"], g[f"{tag}_Ku"], rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("plane", ["stress"])
def test_bar_in_tension_2d(plane):
    """pyMOTO tests/test_assembly.py:101-135: one Q4 element, u = F L / (E A), Poisson contraction."""
    Lx, Ly, Lz = 0.1, 0.2, 0.3
    grid = O.Grid(1, 1, 0, Lx, Ly, Lz)
    E, nu, F = 210e9, 0.3, 1.5
    left = grid.nodes_where(i=0)
    right = grid.nodes_where(i=1)
    bc = np.concatenate([left * 2, [left[0] * 2 + 1]])
    K = O.assemble(grid, O.element_stiffness(grid, E, nu, plane), np.ones(1), bc)
    f = np.zeros(grid.ndof)
    f[right * 2] = F / right.size
    u = np.linalg.solve(K.toarray(), f)
    ux = F * Lx / (E * Ly * Lz)
    np.testing.assert_allclose(u[right * 2], ux, rtol=1e-10)
    np.testing.assert_allclose(u[right[1] * 2 + 1], -nu * ux / Lx * Ly, rtol=1e-10)


def test_bar_in_tension_3d():
    """pyMOTO tests/test_assembly.py:138-190."""
    Lx, Ly, Lz = 0.1, 0.2, 0.3
    g = O.Grid(1, 1, 1, Lx, Ly, Lz)
    E, nu, F = 210e9, 0.3, 1.5e3
    left = g.nodes_where(i=0)
    n00, n10, n01 = g.node_number(0, 0, 0), g.node_number(0, 1, 0), g.node_number(0, 0, 1)
    bc = np.concatenate([left * 3, np.array([n00, n01]) * 3 + 1, np.array([n00, n10]) * 3 + 2])
    right = g.nodes_where(i=1)
    K = O.assemble(g, O.element_stiffness(g, E, nu), np.ones(1), bc)
    f = np.zeros(g.ndof)
    f[right * 3] = F / right.size
    u = np.linalg.solve(K.toarray(), f)
    ux = F * Lx / (E * Ly * Lz)
    np.testing.assert_allclose(u[right * 3], ux, rtol=1e-10)
    et = -nu * ux / Lx
    np.testing.assert_allclose(u[g.node_number(1, 1, 0) * 3 + 1], et * Ly, rtol=1e-10)
    np.testing.assert_allclose(u[g.node_number(1, 0, 1) * 3 + 2], et * Lz, rtol=1e-10)


def test_prolongation_known_answers():
    """pyMOTO tests/test_solvers_multigrid.py:9-91: R^T 1 = 8/6/4.5/3.375 (3D), R 1 = 1."""
    g = O.Grid(10, 10, 10)
    R = O.prolongation(g)
    uc = R.T @ np.ones(g.ndof)
    cg = g.coarse()
    I, J, K = np.meshgrid(np.arange(6), np.arange(6), np.arange(6), indexing="ij")
    nb = (I == 0) | (I == 5)
    nb = nb.astype(int) + ((J == 0) | (J == 5)) + ((K == 0) | (K == 5))
    expect = {0: 8.0, 1: 6.0, 2: 4.5, 3: 3.375}
    vals = uc.reshape(-1, 3)[cg.node_number(I, J, K).ravel()]
    for cnt, v in expect.items():
        np.testing.assert_allclose(vals[nb.ravel() == cnt], v)
    np.testing.assert_allclose(R @ np.ones(cg.ndof), 1.0)
    g2 = O.Grid(10, 10)
    uc2 = (O.prolongation(g2).T @ np.ones(g2.ndof)).reshape(-1, 2)
    c2 = g2.coarse()
    I, J = np.meshgrid(np.arange(6), np.arange(6), indexing="ij")
    nb2 = ((I == 0) | (I == 5)).astype(int) + ((J == 0) | (J == 5))
    for cnt, v in {0: 4.0, 1: 3.0, 2: 2.25}.items():
        np.testing.assert_allclose(uc2[c2.node_number(I, J).ravel()][nb2.ravel() == cnt], v)


def test_filters_match_reference(golden):
    g = golden("filters.npz")
    for tag in ["q4", "q4r3", "h8", "h8r15"]:
        grid = grid_of(g[f"{tag}_shape"])
        r = float(g[f"{tag}_r"])
        x, dy = g[f"{tag}_x"], g[f"{tag}_dy"]
        H, s = O.density_filter_matrix(grid, r)
        np.testing.assert_allclose(O.density_filter(H, s, x), g[f"{tag}_density_y"], rtol=1e-14, atol=1e-15)
        np.testing.assert_allclose(O.density_filter_T(H, s, dy), g[f"{tag}_density_dx"], rtol=1e-13, atol=1e-15)
        W = O.conv_filter_weights(grid, r)
        np.testing.assert_allclose(W, g[f"{tag}_conv_w"], rtol=1e-15)
        np.testing.assert_allclose(O.conv_filter(grid, W, x), g[f"{tag}_conv_y"], rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(O.conv_filter_T(grid, W, dy), g[f"{tag}_conv_dx"], rtol=1e-13, atol=1e-14)


def test_multigrid_matches_reference(golden):
    g = golden("multigrid.npz")
    for tag in ["q4", "h8", "h8b"]:
        grid = grid_of(g[f"{tag}_shape"])
        R = O.prolongation(grid)
        Rr = sps.coo_matrix((g[f"{tag}_R_val"], (g[f"{tag}_R_row"], g[f"{tag}_R_col"])), shape=R.shape)
        assert abs(R - Rr).max() == 0
        K = O.assemble(grid, O.element_stiffness(grid), g[f"{tag}_x"], g[f"{tag}_bc"])
        hier = O.build_hierarchy(grid, K, 3, w=0.6, smooth_steps=2)
        Ac = sps.csr_matrix((g[f"{tag}_Ac_data"], g[f"{tag}_Ac_indices"], g[f"{tag}_Ac_indptr"]), shape=hier[0].Ac.shape)
        assert abs(hier[0].Ac - Ac).max() <= 1e-13 * abs(Ac).max()
        z = O.vcycle(hier[0], g[f"{tag}_r"])
        np.testing.assert_allclose(z, g[f"{tag}_z"], rtol=1e-10, atol=1e-12 * np.abs(z).max())


@pytest.mark.parametrize("name", ["h8_mg", "q4_mg", "h8_direct"])
def test_pipeline_matches_reference(golden, name):
    g = golden(f"pipeline_{name}.npz")
    grid = grid_of(g["shape"])
    levels = int(g["levels"])
    kind = "conv" if name == "h8_mg" else "density"
    plane = "stress" if name == "q4_mg" else "strain"
    P = O.CompliancePipeline(grid, g["bc"], g["f"], filter_kind=kind, radius=float(g["radius"]), plane=plane,
                             levels=levels, w=0.6, smooth_steps=2, tol=float(g["tol"]))
    for it in range(2):
        c = P.response(g[f"x{it}"])
        dx = P.sensitivity()
        assert abs(c - float(g[f"c{it}"])) <= 1e-10 * abs(c)
        np.testing.assert_allclose(P.u, g[f"u{it}"], rtol=0, atol=1e-9 * np.abs(P.u).max())
        np.testing.assert_allclose(dx, g[f"dx{it}"], rtol=0, atol=1e-9 * np.abs(dx).max())


def test_oc_mbb_trajectory(golden):
    """Config-1 workload: 60x20 half-MBB, DensityFilter r=1.5, direct solve, OC move 0.2, 50 iterations."""
    g = golden("oc_mbb.npz")
    grid = O.Grid(60, 20)
    P = O.CompliancePipeline(grid, g["bc"], g["f"], filter_kind="density", radius=1.5, plane="stress", levels=0)
    x = np.full(grid.nel, 0.5)
    hist = []
    for _ in range(50):
        x_eval = x
        hist.append(P.response(x))
        dg = P.sensitivity()
        x = O.oc_step(x, dg, 0.5, move=0.2)
    np.testing.assert_allclose(hist, g["c_hist"], rtol=1e-9)
    # Optimizer.optimize leaves the design Signal at the last evaluated design (optimizers.py:267-316)
    np.testing.assert_allclose(x_eval, g["x_final"], atol=1e-8)
