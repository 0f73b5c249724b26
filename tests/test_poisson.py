"""AssemblePoisson: the scalar element matrix, and the embedding of the scalar problem as the first component of
the vector operator, against pyMOTO's AssemblePoisson and a thermal compliance network."""
import numpy as np
import pytest
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


def _embedded(golden):
    g = golden("poisson.npz")
    d = pg.VoxelDomain(6, 4, 4, 1.0, 0.5, 0.8)
    m = pg.AssemblePoisson(d, bc=g["net_bc"], material_property=2.0)
    grid = O.Grid(6, 4, 4)
    bc_dofs = np.array([n * 3 + c for n in range(grid.nnodes) for c in range(3) if (m._mask_host[n] >> c) & 1])
    A = O.assemble(grid, m.stiffness_element, g["net_x"], bc=bc_dofs, bcdiagval=m.bcdiagval).tocsr()
    return g, m, grid, bc_dofs, A


def test_embedded_operator_is_pymotos_matrix_plus_decoupled_identity(golden):
    g, m, grid, bc_dofs, A = _embedded(golden)
    np.testing.assert_allclose(A[0::3, 0::3] @ g["net_urand"], g["net_Pu"], rtol=1e-13, atol=1e-15)
    for c in (1, 2):
        np.testing.assert_allclose(A[c::3, c::3].toarray(), m.bcdiagval * np.eye(grid.nnodes))
        assert abs(A[0::3, c::3]).max() == 0 and abs(A[c::3, 0::3]).max() == 0


def test_embedded_solve_and_sensitivity_reproduce_the_thermal_network(golden):
    g, m, grid, bc_dofs, A = _embedded(golden)
    f = np.zeros(grid.ndof)
    f[0::3] = g["net_f"]   # the Dirichlet rows are bcdiag I: their solution is load / bcdiag, as in pyMOTO
    u = spla.spsolve(A.tocsc(), f)
    np.testing.assert_allclose(u[0::3], g["net_u"], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(u[1::3], 0.0, atol=0)
    assert float(u[0::3] @ g["net_f"]) == pytest.approx(float(g["net_c"]), rel=1e-10)
    dx = O.sensitivity_contract(grid, m.stiffness_element, [-u], [u], bc=bc_dofs)
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
