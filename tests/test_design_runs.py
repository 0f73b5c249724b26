"""Design loops on the device (GPU): pyMOTO's minimize_oc loop on the half-MBB and run-to-run bitwise
reproducibility of a design iteration."""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import clamp_face_dofs
from test_gpu_pipeline import build_network, dev

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pymoto_gb300 as pg
    pg._lib.load()
    return pg


def test_minimize_oc_runs_pymotos_loop(pg, golden):
    """minimize_oc on the 60x20 half-MBB: the responses of the first 10 OC iterations equal the reference
    trajectory, and the loop leaves the design at the last evaluated one (as pyMOTO's optimize does)."""
    g = golden("oc_mbb.npz")
    d = pg.VoxelDomain(60, 20)
    sx = pg.Signal("x", dev(np.full(d.nel, 0.5)))
    with pg.Network() as fn:
        xf = pg.DensityFilter(d, radius=1.5)(sx)
        xs = pg.SIMP(xmin=1e-9, penal=3.0)(xf)
        K = pg.AssembleStiffness(d, bc=g["bc"], plane="stress")(xs)
        u = pg.LinSolve(hermitian=True, symmetric=True)(K, dev(g["f"]))
        c = pg.EinSum("i,i->")(u, dev(g["f"]))
    oc = pg.minimize_oc(sx, c, fn, maxit=10, tolx=0.0, tolf=0.0, move=0.2, verbosity=0)
    np.testing.assert_allclose(oc.history, g["c_hist"][:10], rtol=1e-6)
    fn.response()
    np.testing.assert_allclose(float(c.state), g["c_hist"][9], rtol=1e-6)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_design_iteration_is_bitwise_reproducible(pg, mixed):
    """Two runs of the same design iteration give the same bits: every reduction has a fixed order and no
    kernel uses floating-point atomics (the lagged coarse inverse, off here, trades this for latency)."""
    shape = (16, 8, 8)
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = np.zeros(g.ndof)
    f[3 * g.node_number(16, 4, 4) + 1] = -1.0
    x = np.random.default_rng(9).uniform(0.1, 1.0, g.nel)
    out = []
    for _ in range(2):
        _, sx, su, sc, fn = build_network(pg, shape, bc, f, "conv", 2.5, 3, 1e-8, mixed=mixed, state_kind="torch")
        sx.state = dev(x)
        fn.response()
        fn.reset()
        sc.sensitivity = 1.0
        fn.sensitivity()
        out.append((sc.state.clone(), su.state.clone(), sx.sensitivity.clone()))
    for a, b in zip(out[0], out[1]):
        assert torch.equal(a, b)
