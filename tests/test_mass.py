"""AssembleMass: the consistent element mass matrix and the assembled operator against pyMOTO's AssembleMass."""
import numpy as np
import pytest
import torch

import oracle as O
import pymoto_gb300 as pg
from pymoto_gb300.operators import element_mass

CASES = {"m2": ((3, 2, 0), (0.5, 2.0, 0.3), 2, 7.8), "m2s": ((3, 2, 0), (1.0, 1.0, 1.0), 1, 1.0),
         "m3": ((2, 2, 2), (0.1, 0.2, 0.3), 3, 2.5), "m3s": ((2, 2, 2), (1.0, 0.5, 2.0), 1, 3.0)}


@pytest.mark.parametrize("tag", list(CASES))
def test_element_mass_matches_pymoto(tag, golden):
    shp, size, ndof, rho = CASES[tag]
    d = pg.VoxelDomain(*shp, *size)
    M0 = element_mass(d, ndof, rho)
    np.testing.assert_allclose(M0, golden("mass.npz")[f"{tag}_M0"], rtol=1e-14, atol=1e-16)
    # every component carries the element's mass: the entries of one component sum to rho * volume
    vol = np.prod(size[:d.dim]) * (size[2] if d.dim == 2 else 1.0)
    assert M0[0::ndof, 0::ndof].sum() == pytest.approx(rho * vol, rel=1e-13)


def test_oracle_assembly_of_the_mass_matrix(golden):
    g = golden("mass.npz")
    grid = O.Grid(4, 3, 2)
    M0 = element_mass(pg.VoxelDomain(4, 3, 2, 0.5, 1.0, 1.5), 3, 2.0)
    M = O.assemble(grid, M0, g["asm_x"], bc=g["asm_bc"], bcdiagval=0.0)
    np.testing.assert_allclose(M @ g["asm_u"], g["asm_Mu"], rtol=1e-13, atol=1e-15)


def test_one_component_oracle_assembles_the_scalar_mass_matrix():
    """ndof=1: the oracle's one-component assembly is the element loop over the node connectivity."""
    d = pg.VoxelDomain(3, 2, 2, 0.5, 1.0, 2.0)
    m = pg.AssembleMass(d, material_property=3.0)
    grid = O.Grid(3, 2, 2)
    rng = np.random.default_rng(1)
    x = rng.uniform(0.1, 1.0, grid.nel)
    A = O.assemble(grid, m.el_mat, x, ndof=1).toarray()
    Ms = np.zeros((grid.nnodes, grid.nnodes))
    conn = grid.conn()                             # element nodes in the local order
    for e in range(grid.nel):
        Ms[np.ix_(conn[e], conn[e])] += x[e] * m.el_mat
    np.testing.assert_allclose(A, Ms, rtol=1e-14, atol=1e-16)
    assert not m._mask_host.any()
    with pytest.raises(NotImplementedError):
        pg.AssembleMass(pg.VoxelDomain(4, 3, 2), ndof=2)


@pytest.mark.gpu
def test_mass_operator_product_on_device(golden):
    g = golden("mass.npz")
    d = pg.VoxelDomain(4, 3, 2, 0.5, 1.0, 1.5)
    M = pg.AssembleMass(d, bc=g["asm_bc"], material_property=2.0, ndof=3)(torch.from_numpy(g["asm_x"]).cuda())
    y = M @ torch.from_numpy(g["asm_u"]).cuda()
    np.testing.assert_allclose(y.cpu().numpy(), g["asm_Mu"], rtol=1e-12, atol=1e-14)


@pytest.mark.gpu
def test_scalar_mass_product_on_device():
    """ndof=1 on the device: one entry per node in and out of the product."""
    d = pg.VoxelDomain(3, 2, 2, 0.5, 1.0, 2.0)
    grid = O.Grid(3, 2, 2)
    rng = np.random.default_rng(2)
    x, u = rng.uniform(0.1, 1.0, grid.nel), rng.standard_normal(grid.nnodes)
    m = pg.AssembleMass(d, material_property=3.0)
    M = m(torch.from_numpy(x).cuda())
    Ms = np.zeros((grid.nnodes, grid.nnodes))
    conn = grid.conn()
    for e in range(grid.nel):
        Ms[np.ix_(conn[e], conn[e])] += x[e] * m.el_mat
    y = M @ torch.from_numpy(u).cuda()
    np.testing.assert_allclose(y.cpu().numpy(), Ms @ u, rtol=1e-12, atol=1e-14)
